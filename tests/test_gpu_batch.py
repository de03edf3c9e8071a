"""Batched form: simulations with uneven grids advanced by one launch per stage give the same
bits as each simulation advanced alone."""
import numpy as np
import pytest

import pxlengine_gb300 as P
from gpu_util import dam

pytestmark = pytest.mark.gpu


def _specs():
    return [
        (dam(res=32, ppc=4, iters=20), 0, "gs"),
        (P.Fluid("b", [[0, 0, 0], [0.8, 0.6, 0.5]], [P.FluidBlock([0.1, 0.0, 0.1], [0.5, 0.4, 0.4], [0.5, 0, 0])],
                 resolution=48, particles_per_cell=5, pressure_iterations=35), 3, "gs"),
        (P.Fluid("c", [[0, 0, 0], [0.3, 0.9, 0.3]], [P.FluidBlock([0.0, 0.3, 0.0], [0.3, 0.9, 0.15])],
                 resolution=36, particles_per_cell=7, pressure_iterations=10, flip=0.5), 9, "gs"),
        (dam(res=40, ppc=6, iters=20), 2, "pcg"),
    ]


def _make(spec):
    f, seed, solver = spec
    return P.FluidState(f, fps=24.0, seed=seed, options=P.make_options(solver=solver, velocity_sigma=0.5,
                                                                       velocity_seed=seed + 1))


def test_batch_equals_alone(lib):
    specs = _specs()
    alone = []
    for sp in specs:
        with _make(sp) as s:
            s.step(6)
            alone.append((s.read_particles(), s.read_grid("vel"), s.read_grid("pressure")))
    sims = [_make(sp) for sp in specs]
    b = P.Batch()
    for s in sims:
        b.add(s)
    assert len(b) == len(sims)
    b.step(4)
    b.step(2)
    b.sync()
    for s, (p, v, pr) in zip(sims, alone):
        assert s.steps_done == 6
        np.testing.assert_array_equal(s.read_particles(), p)
        np.testing.assert_array_equal(s.read_grid("vel"), v)
        if s is not sims[-1]:   # the precision solver's reductions are per simulation as well
            np.testing.assert_array_equal(s.read_grid("pressure"), pr)
        else:
            np.testing.assert_array_equal(s.read_grid("pressure"), pr)
    b.close()
    for s in sims:
        s.close()


def test_batch_membership_changes(lib):
    specs = _specs()[:3]
    sims = [_make(sp) for sp in specs]
    ref = []
    for sp in specs:
        with _make(sp) as s:
            s.step(3)
            ref.append(s.read_particles())
    b = P.Batch()
    b.add(sims[0])
    b.step(1)
    b.add(sims[1])
    b.step(1)
    b.add(sims[2])
    b.step(1)
    b.remove(sims[0])
    b.step(2)
    b.sync()
    np.testing.assert_array_equal(sims[0].read_particles(), ref[0])
    with pytest.raises(P.FluidError):
        sims[1].step(1)   # stepped only through its batch while a member
    b.close()
    sims[1].step(0)
    for s in sims:
        s.close()


def test_autotune_substep_is_a_normal_substep(lib):
    """The autotuner's substep (every P2G variant timed on the sorted particles) leaves the same
    bits as a plain substep, and later substeps with the chosen variant stay identical."""
    spec = _specs()[1]
    with _make(spec) as a, _make(spec) as b:
        a.step(1)
        r = b.autotune()
        assert b.steps_done == 1
        assert 0 <= r["tile_shape"] < 5 and r["lanes"] in (0, 1)
        assert len(r["variant_ms"]) == 10 and all(m > 0 for m in r["variant_ms"])
        assert r["variant_ms"][2 * r["tile_shape"] + r["lanes"]] == min(r["variant_ms"])
        np.testing.assert_array_equal(a.read_particles(), b.read_particles())
        np.testing.assert_array_equal(a.read_grid("vel"), b.read_grid("vel"))
        a.step(3)
        b.step(3)
        np.testing.assert_array_equal(a.read_particles(), b.read_particles())


def test_batch_autotune(lib):
    specs = _specs()
    alone = []
    for sp in specs:
        with _make(sp) as s:
            s.step(3)
            alone.append(s.read_particles())
    sims = [_make(sp) for sp in specs]
    b = P.Batch()
    for s in sims:
        b.add(s)
    r = b.autotune()
    assert r["chosen"].startswith("p2g ")
    b.step(2)
    b.sync()
    for s, ref in zip(sims, alone):
        assert s.steps_done == 3
        np.testing.assert_array_equal(s.read_particles(), ref)
    b.close()
    for s in sims:
        s.close()


def test_batch_grows_and_shrinks_one_by_one(lib):
    """Membership changing one simulation at a time (as the serving loop does) reallocates the
    batch's tables repeatedly; every member still matches its own run."""
    specs = [(dam(res=16 + 2 * k, ppc=4, iters=10), k, "pcg" if k % 2 else "gs") for k in range(7)]
    n = len(specs)
    ref = []
    for k, sp in enumerate(specs):
        with _make(sp) as s:
            s.step(n - k)          # added k-th, then one batched substep after every addition
            ref.append(s.read_particles())
    sims = [_make(sp) for sp in specs]
    b = P.Batch()
    for s in sims:
        b.add(s)
        b.step(1)
    b.sync()
    for s, r in zip(sims, ref):
        np.testing.assert_array_equal(s.read_particles(), r)
    for s in sims[:5]:
        b.remove(s)
        b.step(1)
    b.sync()
    b.close()
    for s in sims:
        s.close()
