"""The roofline arithmetic of bench.py: algorithmic bytes per kernel launch and per substep, and the
whole-job rate (no GPU: plain arithmetic on the configured workload sizes)."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

# 256 x 128 x 128 dam break: cells, faces, particles; system cells at one measured state
C = 256 * 128 * 128
F = 257 * 128 * 128 + 256 * 129 * 128 + 256 * 128 * 129
N = 8_001_504
CF = 518_964


def test_sizes_of_the_default_workload():
    assert C == 4_194_304 and F == 12_664_832


def test_red_black_sweep_counts_system_cells():
    # one colour sweep: 14 B per cell of the colour (list, record, div, p) + 4 B per other-colour cell
    assert bench.kernel_bytes("k_pressure_rb_list", N, F, C, CF) == 9 * CF
    # the dense sweep touches every cell of the grid
    assert bench.kernel_bytes("k_pressure_rb", N, F, C, CF) == 8 * C


def test_substep_bytes():
    assert bench.substep_bytes(N, F, C, CF, "gs", 80) == 96 * N + 60 * F + 40 * C + 18 * CF * 80
    assert bench.substep_bytes(N, F, C, CF, "pcg", 12) == 96 * N + 60 * F + 40 * C + 56 * CF * 12


def test_particle_kernels():
    assert bench.kernel_bytes("k_p2g", N, F, C, CF) == 32 * N + 8 * F + 4 * C
    assert bench.kernel_bytes("k_g2p", N, F, C, CF) == 64 * N + 8 * F
    assert bench.kernel_bytes("k_scatter", N, F, C, CF) == 64 * N
    assert bench.kernel_bytes("k_tile_weigh", N, F, C, CF) is None


def test_multigrid_kernels_average_over_a_v_cycle():
    lv = {"system_cells": [551128, 69320, 6977, 595, 9, 0], "tail": 3}
    sm = bench.kernel_bytes("k_mg_smooth", N, F, C, CF, lv)
    assert sm == pytest.approx(9 * (551128 + 69320 + 6977) / 3)
    rs = bench.kernel_bytes("k_mg_restrict", N, F, C, CF, lv)
    assert rs == pytest.approx((10 * (551128 + 69320 + 6977) + 10 * (69320 + 6977 + 595)) / 3)
    assert bench.kernel_bytes("k_mg_smooth", N, F, C, CF, None) is None


def test_whole_job_rate():
    # two ranks of N particles, 100 substeps, the slowest rank 500 ms
    assert bench.whole_job_rate(2 * N, 100, 500.0) == pytest.approx(2 * N * 100 / 0.5)
    assert bench.over_ranks(None, 3.5) == 3.5


def test_streamed_and_one_launch_red_black_kernels():
    # a streamed pass is two iterations; the one-launch solve is every iteration of the substep
    assert bench.kernel_bytes("k_gs_pass", N, F, C, CF) == 36 * CF
    assert bench.kernel_bytes("k_gs_resident", N, F, C, CF, None, 80) == 18 * CF * 80
    assert bench.kernel_bytes("k_gs_prep", N, F, C, CF) == 19 * C


def test_reference_arm_sample_on_the_cpu():
    """The CPU reference of a small workload: the reference's own shader where it was built
    (kind "reference"), the oracle port otherwise; with a time budget the timed substeps shrink
    to what fits it at the warm-up pace, never below two."""
    from oracle import ref
    r = bench.cpu_baseline_run(bench.CONFIGS["dam64"], 3, 1, budget_s=1e-6)
    assert r["kind"] == ("reference" if ref.available() else "port")
    assert r["timed_steps"] == 2 and r["particles"] == 108_000 and r["value"] > 0
    p = bench.cpu_baseline_run(dict(bench.CONFIGS["dam64"], solver="pcg"), 1, 0)
    assert p["kind"] == "port"
