#!/usr/bin/env python3
"""FLIP liquid substep benchmark (particle-substeps/s on one GB300 per rank).

Default workload (N=1): the stress double dam break, the largest single-GPU configuration —
bounds [[0,0,0],[2,1,1]] at resolution 512 (512 x 256 x 256 MAC grid, h = 1/256), two fluid
boxes x in [0, 0.6] and [1.4, 2.0], y in [0, 0.6], full z, 8 particles per cell seeded with the
reference LCG (95,126,400 particles), zero initial velocity, gravity -9.81, dt = 1/120 (fps 15,
8 substeps), FLIP 0.95, the reference's red-black Gauss-Seidel pressure solve with 80 iterations,
FP32 throughout. --config dam256 is the large single dam break with the precision solver (PCG
with FP64 dot products and restarts to relative residual 1e-6); dam256_gs the same grid with the
reference solver; dam64 the reference's own CPU-runnable case.

A step is one substep of that simulation. `value` is device time of K substeps (CUDA events on
the library's stream, inputs resident in HBM); `e2e` goes through the public C ABI with host
buffers: per step one pxf_write_particles from pinned memory, one pxf_advance_to_frame of a
whole frame (`substeps` substeps) and one pxf_read_particles into pinned memory.

--impl reference times the reference on the host cores (all threads) on the same workload, one
step = one substep: pxlengine's own shaders/fluid.slang compiled for the CPU (oracle/_ref, built by
oracle/ref_build.py) for the reference solver, the oracle's restatement (oracle/) where that build
is absent and for the precision solver.
Multi-GPU (torchrun): replicas only — every rank runs its own simulation, no exchange.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # the reference's plain CPU-runnable case: 64 x 32 x 32, red-black GS, 80 iterations
    "dam64": dict(bounds=((0, 0, 0), (1, 0.5, 0.5)), resolution=64, fill=[((0, 0, 0), (0.25, 0.5, 0.5))],
                  ppc=8, fps=15.0, substeps=8, solver="gs", iterations=80, lift=False),
    # large single dam break, precision solver (the metric's headline configuration)
    "dam256": dict(bounds=((0, 0, 0), (1, 0.5, 0.5)), resolution=256, fill=[((0, 0, 0), (0.25, 0.5, 0.5))],
                   ppc=8, fps=15.0, substeps=8, solver="pcg", iterations=80, lift=False),
    # the same grid with the reference's red-black GS (80 iterations)
    "dam256_gs": dict(bounds=((0, 0, 0), (1, 0.5, 0.5)), resolution=256, fill=[((0, 0, 0), (0.25, 0.5, 0.5))],
                      ppc=8, fps=15.0, substeps=8, solver="gs", iterations=80, lift=False),
    # stress double dam break 512 x 256 x 256 (benchmark entry: beyond the scene limits)
    "dam512": dict(bounds=((0, 0, 0), (2, 1, 1)), resolution=512,
                   fill=[((0, 0, 0), (0.6, 0.6, 1.0)), ((1.4, 0, 0), (2.0, 0.6, 1.0))],
                   ppc=8, fps=15.0, substeps=8, solver="gs", iterations=80, lift=True),
}


def over_ranks(dist, x, op="max"):
    """x reduced over the ranks of the process group (identity without one)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_all_ranks, steps, max_ms):
    """Particle-substeps per second of the whole job: every rank's particles times the steps, over
    the slowest rank's time."""
    return units_all_ranks * steps / (max_ms / 1e3)


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of a kernel from one ncu
# capture of this workload, keyed by (config, kernel); the captures are summarised in profiles/.
KERNEL_TRAFFIC = {
    ("dam256", "k_p2g"): 408.48e6,
    ("dam256", "k_g2p"): 545.89e6,
    ("dam256", "k_pcg_update"): 30.11e6,
    ("dam256", "k_mg_smooth"): 4.349e6,      # mean over the V-cycle's levels (500 launches)
    ("dam256_gs", "k_pressure_rb_list"): 12.47e6,
    ("dam256_gs", "k_gs_resident"): 17.61e6,
    ("dam512", "k_gs_pass"): 211.6e6,
}
# DRAM traffic per system cell of one launch, from a capture of a smaller grid, for kernels whose
# traffic grows with the system cells (a full-size capture would exceed the profiler's size rules);
# the traffic of a launch is this figure times the workload's system cells.
KERNEL_TRAFFIC_PER_SYSTEM_CELL = {}


def kernel_traffic(config, kernel, system_cells):
    """DRAM bytes of one launch from a capture of this workload, else scaled from a smaller grid's
    capture by the system cells; None when no capture covers the kernel."""
    t = KERNEL_TRAFFIC.get((config, kernel))
    if t is None and kernel in KERNEL_TRAFFIC_PER_SYSTEM_CELL:
        t = KERNEL_TRAFFIC_PER_SYSTEM_CELL[kernel] * system_cells
    return t


def make_fluid(P, cfg):
    return P.Fluid("bench", [list(cfg["bounds"][0]), list(cfg["bounds"][1])],
                   [P.FluidBlock(list(a), list(b)) for a, b in cfg["fill"]], resolution=cfg["resolution"],
                   particles_per_cell=cfg["ppc"], substeps=cfg["substeps"], pressure_iterations=cfg["iterations"])


L2_BYTES = 129e6


def state_bytes(dims, n):
    """Device state one substep streams: particle records (current and sorted, 32 B each), the two
    face velocity fields and the per-cell fields (13 B per cell)."""
    nx, ny, nz = dims
    C = nx * ny * nz
    F = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)
    return 64 * n + 8 * F + 13 * C


def workload_config(name, cfg, dims, n):
    sb = state_bytes(dims, n)
    l2 = (f"inputs larger than L2: {sb / 1e9:.2f} GB of particle and grid state per substep against 129 MB"
          if sb > L2_BYTES else
          f"working set inside L2 ({sb / 1e6:.0f} MB of particle and grid state): L2 not flushed between steps")
    return {"workload": f"dam_break_{name}", "grid": list(dims), "particles": n, "ppc": cfg["ppc"],
            "dt": f"1/{int(cfg['fps'] * cfg['substeps'])}", "pressure": (
                "pcg_fp64dots_rtol1e-6" if cfg["solver"] == "pcg" else f"rbgs_{cfg['iterations']}"),
            "seed": 0, "l2": l2, "parallelism": "replicas"}


def kernel_bytes(kernel, N, F, C, Cf, lv=None, iters=0):
    """Algorithmic bytes of one launch of a kernel: each array the kernel must touch counted once,
    4 B per face or cell value, 32 B per particle, 1 B per cell flag, 2 B per neighbour record,
    4 B per cell-list entry (Cf = system cells). Multigrid kernels: the mean over the launches of
    one V-cycle, from the per-level system cells (lv). The one-launch red-black solve: all `iters`
    iterations."""
    if kernel in ("k_mg_smooth", "k_mg_restrict"):
        if not lv or lv["tail"] <= 0:
            return None
        cf, T = lv["system_cells"], lv["tail"]
        if kernel == "k_mg_smooth":
            # half sweep over one colour: list, r, record in, z out (14 B per colour cell) and
            # z of the other colour in (4 B per cell): 9 B per system cell of the level
            return sum(9 * cf[l] for l in range(T)) / T
        # fine r, z, record in (10 B per fine system cell); coarse list in, r and red z out
        return sum(10 * cf[l] + 10 * cf[l + 1] for l in range(T)) / T
    return {
        "k_scan_chunks": 4 * C,                      # counts in (chunk sums out)
        "k_scan_apply": 4 * C + 4 * C + 1 * C,       # counts in; starts and cell flags out
        "k_gs_lists": 2 * C + 4 * Cf,                # neighbour records in; system-cell lists out
        "k_cell_lists": 2 * C + 4 * Cf,
        "k_scatter": 64 * N,                         # particle records in and out (sorted order)
        "k_p2g": 32 * N + 8 * F + 4 * C,             # sorted particles and cell starts in; vel, vel_old out
        "k_divergence": 4 * F + 1 * C + 4 * C + 2 * C,   # faces, flags in; divergence, neighbour record out
        "k_pressure_rb": 8 * C,                      # one colour: 16C per red-black iteration
        "k_gs_pass": 36 * Cf,                        # two red-black iterations of the system cells
                                                     # (18 B per system cell per iteration, as above)
        "k_gs_prep": 19 * C,                         # pressure, divergence, record in; p_alt, rhs, count out
        "k_pressure_rb_list": 9 * Cf,                # one colour of the system cells: list, record, div in,
                                                     # p out (14 B per colour cell), other colour's p in
        "k_gs_resident": 18 * Cf * iters,            # every red-black iteration in one launch, 18 B per
                                                     # system cell per iteration as above
        "k_pcg_dir": 22 * Cf,                        # list, z, p, record in; p', Ap out
        "k_pcg_update": 38 * Cf,                     # list, p, Ap, r, x (8 B) in; r, x, red z out
        "k_project": 8 * F + 5 * C,                  # faces in and out; pressure, flags in
        "k_g2p": 64 * N + 8 * F,                     # particles in and out; vel, vel_old in
    }.get(kernel)


def substep_bytes(N, F, C, Cf, solver, iters):
    """Algorithmic bytes of one substep: 96N + 60F + 40C plus the pressure solve (red-black GS:
    18 B per system cell per iteration, two colour sweeps over the system cells; PCG: 56 B per
    system cell per iteration)."""
    press = 18 * Cf * iters if solver == "gs" else 56 * Cf * iters
    return 96 * N + 60 * F + 40 * C + press


def cpu_baseline_run(cfg, steps, warmup, sample_substeps=1, budget_s=None):
    """The reference on all host cores, one substep per step, from the seeded state: for the
    reference solver pxlengine's own shaders/fluid.slang compiled for the CPU (oracle/_ref, kind
    "reference") where it was built, else the oracle's restatement (kind "port"; also the precision
    solver, which the reference does not have). With budget_s, the timed substeps are cut to what
    fits that many seconds at the warm-up pace (at least two)."""
    import oracle
    from oracle import ref
    fill = [{"min": list(a), "max": list(b)} for a, b in cfg["fill"]]
    bounds = [list(cfg["bounds"][0]), list(cfg["bounds"][1])]
    dims, h = oracle.grid(bounds, cfg["resolution"])
    p = oracle.seed_particles(bounds, cfg["resolution"], fill, cfg["ppc"], 0)
    dt = oracle.dt_for(cfg["fps"], cfg["substeps"])
    if cfg["solver"] == "gs" and ref.available():
        kind, threads = "reference", ref.num_threads(0)
        s = ref.RefSim(dims, h, dt, 0.95, bounds[0], [0, -9.81, 0], cfg["iterations"], p)
    else:
        kind, threads = "port", oracle.num_threads(0)
        s = oracle.OracleSim(dims, h, dt, 0.95, bounds[0], [0, -9.81, 0], cfg["iterations"], p)
        if cfg["solver"] == "pcg":
            # the same algorithm as the GPU path: multigrid-preconditioned CG, FP64 dots and restarts
            s.set_pressure("mgpcg", rtol=1e-6, max_iter=4000, restart=50)
    t0 = time.perf_counter()
    for _ in range(warmup):
        s.step(sample_substeps)
    if budget_s and warmup:
        pace = (time.perf_counter() - t0) / warmup
        steps = max(2, min(steps, int(budget_s / max(pace, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(steps):
        s.step(sample_substeps)
    el = time.perf_counter() - t0
    n = p.shape[0]
    return {"value": n * steps * sample_substeps / el, "ms_per_step": 1e3 * el / steps, "cores": threads,
            "particles": n, "dims": dims, "kind": kind, "timed_steps": steps}


# ------------------------------------------------------------------------------------ batched
H0 = 1.0 / 64   # cell size of the generated domains (sides are whole numbers of cells)


def box_fluid(P, name, dims, rng, ppc):
    """A domain of dims cells with one seeded fluid box of 10-60% of each axis."""
    import numpy as np
    size = np.asarray(dims, dtype=np.float64) * H0
    ext = rng.uniform(0.1, 0.6, 3)
    pos = rng.uniform(0.0, 1.0, 3) * (1.0 - ext)
    lo, hi = pos * size, (pos + ext) * size
    return P.Fluid(name, [[0.0, 0.0, 0.0], size.tolist()], [P.FluidBlock(lo.tolist(), hi.tolist())],
                   resolution=int(max(dims)), particles_per_cell=int(ppc), substeps=8)


def batched_specs(P, n, seed):
    """n simulations: each grid side drawn from {32, 48, ..., 192} per axis, one seeded box,
    4-8 particles per cell (velocities N(0, 0.5) per component via the options)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sides = np.arange(32, 193, 16)
    return [box_fluid(P, f"b{i}", rng.choice(sides, 3).tolist(), rng, rng.integers(4, 9)) for i in range(n)]


def divergence_linf(sim):
    """max |div v| * dt over fluid cells after the substep's projection (volume change per step)."""
    import numpy as np
    nx, ny, nz = sim.dims
    v = sim.read_grid("vel")
    nu, nv = (nx + 1) * ny * nz, nx * (ny + 1) * nz
    u = v[:nu].reshape(nz, ny, nx + 1)
    w_ = v[nu:nu + nv].reshape(nz, ny + 1, nx)
    ww = v[nu + nv:].reshape(nz + 1, ny, nx)
    ct = sim.read_grid("cell_type").reshape(nz, ny, nx)
    d = (u[:, :, 1:] - u[:, :, :-1]) + (w_[:, 1:, :] - w_[:, :-1, :]) + (ww[1:] - ww[:-1])
    d = d / sim.cell
    fl = ct == 1
    return float(np.max(np.abs(d[fl])) * sim.dt) if fl.any() else 0.0


def fp64_check(sim, origin, iterations):
    """One more substep of the GPU simulation against the oracle's FP64 solve of the same pressure
    system (the oracle's pre-pressure stages are bit-exact with the GPU's): max pressure error
    relative to max |p64|, and max |div v| * dt after the GPU's projection."""
    import numpy as np
    import oracle
    p0 = sim.read_particles()
    o = oracle.OracleSim(sim.dims, sim.cell, sim.dt, 0.95, list(origin), [0, -9.81, 0], iterations, p0)
    o.set_pressure("pcg64", rtol=1e-10, max_iter=100000)
    sim.step(1)
    for st in ("clear", "p2g", "normalize", "forces", "divergence", "pressure"):
        o.stage(st)
    p64 = o.read(oracle.PRESSURE64)
    pg = sim.read_grid("pressure64")
    scale = max(1e-30, float(np.max(np.abs(p64))))
    return {"pressure_rel_err_vs_fp64": float(np.max(np.abs(pg - p64))) / scale,
            "divergence_linf_dt": divergence_linf(sim), "fp64_rtol": 1e-10}


# The reference's example scene's liquid (examples/dam-break.json: 64 x 38 x 32 grid, 139,200
# particles, 8 substeps of red-black GS with 80 iterations per frame at 24 fps).
DAM_BREAK_SCENE = ('{"version":1,"nodes":[{"type":"camera"}],"fluids":[{"name":"water",'
                   '"bounds":[[-1,0,-0.5],[1,1.2,0.5]],"resolution":64,'
                   '"fill":[{"min":[-0.97,0.03,-0.47],"max":[-0.35,0.95,0.47]}],"substeps":8,"flip":0.95}]}')


def reference_scene_frames(P, frames=24):
    """Device time per frame of the example scene's liquid: 8 substeps plus the surface mesh (the
    reference publishes about 12 ms per frame for simulation, surface nets and BLAS on a laptop
    RTX 4080, docs/ROADMAP.md:83)."""
    with P.FluidState.from_json(DAM_BREAK_SCENE) as s:
        s.step_timed(16)
        s.surface_mesh()
        sim_ms, mesh_ms, tris = 0.0, 0.0, 0
        for _ in range(frames):
            sim_ms += s.step_timed(8)
            m = s.surface_mesh()
            mesh_ms += m["device_ms"]
            tris = len(m["indices"])
        return {"particles": s.particle_count(), "grid": list(s.dims), "frames": frames,
                "sim_ms_per_frame": sim_ms / frames, "mesh_ms_per_frame": mesh_ms / frames,
                "ms_per_frame": (sim_ms + mesh_ms) / frames, "triangles": tris,
                "reference_published_ms_per_frame": 12.0,
                "reference_hardware": "RTX 4080 Laptop (simulation, surface nets and BLAS per frame)"}


def pct(xs, q):
    import numpy as np
    return float(np.percentile(np.asarray(xs, dtype=np.float64), q)) if len(xs) else None


def run_batched(args, world, rank, local):
    import numpy as np
    import pxlengine_gb300 as P
    n = args.batch_sims
    fl = batched_specs(P, n, seed=1000 + rank)
    sims = [P.FluidState(f, fps=15.0, seed=i, options=P.make_options(
        solver="pcg", rtol=1e-6, max_iter=4000, restart=50, velocity_sigma=0.5, velocity_seed=i + 1))
        for i, f in enumerate(fl)]
    N = sum(s.particle_count() for s in sims)
    cells = sum(int(np.prod(s.dims)) for s in sims)
    b = P.Batch()
    for s in sims:
        b.add(s)
    tune = b.autotune()
    b.step(max(0, args.warmup - 1))
    b.sync()
    clocks = ClockSampler(local)
    clocks.start()
    lat = [b.step_timed(1) for _ in range(args.steps)]
    clk = clocks.stop()
    ms = sum(lat)
    value = N * args.steps / (ms / 1e3)
    div = max(divergence_linf(s) for s in sims[:4])
    iters = [s.solver_stats()[0] for s in sims]
    b.close()
    # FP64 reference of one more substep of the two smallest members (the oracle's FP64 solve)
    fp64 = None
    if rank == 0 and not args.no_fp64_check:
        small = sorted(range(n), key=lambda i: int(np.prod(sims[i].dims)))[:2]
        fp64 = [dict(member=i, grid=list(sims[i].dims), **fp64_check(sims[i], fl[i].bounds[0], fl[i].pressure_iterations))
                for i in small]
    # the plain per-simulation loop on the same GPU: each simulation advanced alone, one after another
    for s in sims:
        s.step(1)
        s.sync()
    loop_steps = max(1, min(args.steps, 3))
    loop_ms = 0.0
    for _ in range(loop_steps):
        for s in sims:
            loop_ms += s.step_timed(1)
    loop_value = N * loop_steps / (loop_ms / 1e3)
    for s in sims:
        s.close()
    return {"value": value, "value_local": value, "ms": ms, "lat": lat, "N": N, "cells": cells, "clk": clk, "tune": tune,
            "div_linf": div, "iters": iters, "loop_value": loop_value, "loop_ms_per_round": loop_ms / loop_steps,
            "fp64": fp64}


def serve_request(P, rng, i):
    import numpy as np
    side = int(np.clip(round(rng.lognormal(np.log(96.0), 0.5)), 32, 256))
    f = box_fluid(P, f"r{i}", [side, side, side], rng, rng.integers(4, 9))
    return f, int(rng.integers(50, 501))


def run_serve(args, lam, duration, seed, budget_bytes=150_000_000_000):
    """Poisson arrivals at rate lam for `duration` seconds into a server with a worker thread;
    then the queue drains. Substep latency = device time of one batched substep; queue wait =
    admission time - submission time of each request."""
    import numpy as np
    import pxlengine_gb300 as P
    from pxlengine_gb300 import _lib as L
    rng = np.random.default_rng(seed)
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / lam)
        if t > duration:
            break
        arrivals.append(t)
    reqs = [serve_request(P, rng, i) for i in range(len(arrivals))]
    opts = P.make_options(solver="pcg", rtol=1e-6, max_iter=4000, restart=50, lift_grid_limits=True,
                          velocity_sigma=0.5, velocity_seed=7)
    srv = P.Server(hbm_budget_bytes=budget_bytes, max_active=256, substeps_per_tick=1, wait_timeout_s=600.0)
    srv.start()
    t0 = time.perf_counter()
    ids = []
    for ta, (f, nsub) in zip(arrivals, reqs):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        ids.append(srv.submit(f, nsub, fps=15.0, seed=len(ids), options=opts))
    deadline = time.perf_counter() + args.serve_drain_s
    while time.perf_counter() < deadline:
        st = srv.stats()
        if st["active"] == 0 and st["queued"] == 0:
            break
        time.sleep(0.05)
    srv.stop()
    wall = time.perf_counter() - t0
    st = srv.stats()
    done = [srv.status(i) for i in ids]
    lat = [d.finish_s - d.submit_s for d in done if d.state == L.REQ_DONE]
    qwait = [d.admit_s - d.submit_s for d in done if d.state == L.REQ_DONE]
    out = {"lambda_per_s": lam, "hbm_budget_gb": budget_bytes / 1e9, "requests": len(ids),
           "completed": int(st["completed"]), "p50_queue_wait_s": pct(qwait, 50), "p99_queue_wait_s": pct(qwait, 99),
           "rejected": int(st["rejected"]), "particle_substeps_per_s": st["particle_substeps"] / wall,
           "p50_substep_ms": st["p50_substep_ms"], "p99_substep_ms": st["p99_substep_ms"],
           "p50_tick_wall_ms": st["p50_tick_wall_ms"], "p99_tick_wall_ms": st["p99_tick_wall_ms"],
           "p50_request_s": pct(lat, 50), "p99_request_s": pct(lat, 99),
           "peak_reserved_gb": st["peak_reserved_bytes"] / 1e9, "wall_s": wall,
           "device_busy_frac": st["busy_device_ms"] / 1e3 / wall}
    srv.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="dam512", choices=sorted(CONFIGS) + ["batched", "serve"])
    ap.add_argument("--batch-sims", type=int, default=64)
    ap.add_argument("--serve-rates", default="2,8,32,64")
    ap.add_argument("--serve-pressure-gb", type=float, default=3.0,
                    help="HBM budget of the extra serving run that makes admission queue (0: none)")
    ap.add_argument("--serve-pressure-rate", type=float, default=16.0)
    ap.add_argument("--serve-duration-s", type=float, default=15.0)
    ap.add_argument("--serve-drain-s", type=float, default=120.0)
    ap.add_argument("--e2e-steps", type=int, default=8, help="frames of the end-to-end measurement")
    ap.add_argument("--reference-budget-s", type=float, default=150.0,
                    help="--impl reference: timed substeps cut to fit this many seconds at the warm-up pace")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="skip the comparison of one precision-solver substep's pressure with the oracle's FP64 solve")
    args = ap.parse_args()
    cfg = CONFIGS.get(args.config)
    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)
    local = env_int("LOCAL_RANK", 0)
    metric = "FLIP particle-substeps/s"
    unit = "particle-substeps/s"

    if args.impl == "reference" and cfg is None:
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched or serving form; "
                              "its CPU arm is timed on the single-simulation configs"}), flush=True)
        return
    if args.impl == "reference":
        if rank != 0:
            return
        # warm-up substeps on the CPU only load caches and pages: at most two, so that the run stays
        # within a few minutes at 512 x 256 x 256 (about 5 s per substep on 16 cores)
        r = cpu_baseline_run(cfg, args.steps, min(args.warmup, 2), budget_s=args.reference_budget_s)
        line = {"metric": metric, "value": r["value"], "unit": unit, "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded dam break, reference LCG seeding)",
                "config": workload_config(args.config, cfg, r["dims"], r["particles"]),
                "cpu_baseline": {"value": r["value"], "unit": unit, "cores": r["cores"], "kind": r["kind"],
                                 "sample": f"{r['timed_steps']} full substeps of the workload from the seeded state "
                                           f"after {min(args.warmup, 2)} warm-up substeps, all host threads"
                                           + (" (pxlengine's shaders/fluid.slang compiled for the CPU)"
                                              if r["kind"] == "reference" else " (the oracle's restatement)")},
                "e2e": {"value": r["value"], "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo", init_method="env://")
        dist = dist_mod

    from pxlengine_gb300 import build
    build.build()
    import numpy as np
    import pxlengine_gb300 as P
    from pxlengine_gb300 import _lib as L
    lib = L.load()
    if lib.pxf_set_device(local) != 0:
        raise RuntimeError(lib.pxf_last_error(None).decode())

    if args.config == "batched":
        r = run_batched(args, world, rank, local)
        r["value"] = whole_job_rate(over_ranks(dist, r["N"], "sum"), args.steps, over_ranks(dist, r["ms"]))
        if rank == 0:
            line = {"metric": metric, "value": r["value"], "unit": unit, "n_gpus": world, "steps": args.steps,
                    "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                    "data": "synthetic (seeded boxes, reference LCG seeding, N(0,0.5) velocities)",
                    "config": {"workload": f"batched_{args.batch_sims}_sims", "sims": args.batch_sims,
                               "particles": r["N"], "cells": r["cells"], "sides": "32..192 per axis",
                               "pressure": "pcg_fp64dots_rtol1e-6", "parallelism": "replicas",
                               "l2": "inputs larger than L2"},
                    "p50_substep_ms": pct(r["lat"], 50), "p99_substep_ms": pct(r["lat"], 99),
                    "plain_loop": {"value": r["loop_value"], "unit": unit,
                                   "ms_per_round": r["loop_ms_per_round"],
                                   "how": "each simulation advanced alone (own graph), one after another"},
                    "batched_over_loop": r["value_local"] / r["loop_value"], "autotune": r["tune"],
                    "divergence_linf_dt": r["div_linf"], "pcg_iterations": [min(r["iters"]), max(r["iters"])],
                    "precision_vs_fp64": r["fp64"],
                    "clocks": r["clk"], "roofline": None, "cpu_baseline": None, "e2e": None}
            print(json.dumps(line), flush=True)
        if dist:
            dist.destroy_process_group()
        return
    if args.config == "serve":
        rows = [run_serve(args, float(lam), args.serve_duration_s, seed=17 + rank)
                for lam in args.serve_rates.split(",")]
        # admission under memory pressure: the same stream against a small budget, so requests
        # wait in the queue for earlier ones to retire
        if args.serve_pressure_gb > 0:
            rows.append(run_serve(args, float(args.serve_pressure_rate), args.serve_duration_s, seed=29 + rank,
                                  budget_bytes=int(args.serve_pressure_gb * 1e9)))
        if rank == 0:
            best = max(rows[:len(args.serve_rates.split(","))], key=lambda r: r["particle_substeps_per_s"])
            line = {"metric": metric, "value": best["particle_substeps_per_s"] * world, "unit": unit,
                    "n_gpus": world, "steps": None, "warmup": 0, "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "f32",
                    "data": "synthetic (Poisson arrivals, lognormal sides median 96 in [32, 256], seeded boxes)",
                    "config": {"workload": "serving", "hbm_budget_gb": 150, "substeps": "50..500",
                               "pressure": "pcg_fp64dots_rtol1e-6", "duration_s": args.serve_duration_s,
                               "parallelism": "replicas"},
                    "sweep": rows, "roofline": None, "cpu_baseline": None, "e2e": None}
            print(json.dumps(line), flush=True)
        if dist:
            dist.destroy_process_group()
        return

    fluid = make_fluid(P, cfg)
    opts = P.make_options(solver=cfg["solver"], rtol=1e-6, max_iter=4000, restart=50,
                          lift_grid_limits=cfg["lift"])
    sim = P.FluidState(fluid, fps=cfg["fps"], seed=0, options=opts)
    N = sim.particle_count()
    nx, ny, nz = sim.dims
    C = nx * ny * nz
    F = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)

    sim.step_timed(args.warmup)
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    t_wall = time.perf_counter()
    ms = sim.step_timed(args.steps)
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    if dist:
        dist.barrier()
    ms = over_ranks(dist, ms)
    value = whole_job_rate(over_ranks(dist, N, "sum"), args.steps, ms)

    # Roofline of the dominant kernel: a kernel-by-kernel substep with a CUDA event after every
    # kernel on the library's stream (eager launches behind a hold kernel, so gaps are device time).
    roofline = None
    substep_roofline = None
    kernels = []
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    iters = cfg["iterations"]
    if cfg["solver"] == "pcg":
        iters = sim.solver_stats()[0]
    ct = sim.read_grid("cell_type")
    Cf = int(np.count_nonzero(ct == 1))
    lv = sim.mg_levels() if cfg["solver"] == "pcg" else None
    if not args.no_profile:
        prof = sim.profile_substep()
        total = sum(r[2] for r in prof)
        kernels = []
        for n, k, m in prof:
            rec = {"kernel": n, "launches": k, "ms": m, "share": m / total}
            b = kernel_bytes(n, N, F, C, Cf, lv, iters)
            if b:
                gbs = b / (m / k / 1e3) / 1e9
                rec.update({"alg_bytes_per_launch": b, "achieved_gbs": gbs, "frac_of_peak": gbs / peak})
            kernels.append(rec)
        ranked = sorted(prof, key=lambda r: -r[2])
        top = next((r for r in ranked if kernel_bytes(r[0], N, F, C, Cf, lv, iters)), None)
        if top:
            name, launches, tot = top
            per_launch = kernel_bytes(name, N, F, C, Cf, lv, iters)
            achieved = per_launch / (tot / launches / 1e3) / 1e9
            roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": kernel_traffic(args.config, name, Cf),
                        "peak_source": peak_src, "alg_bytes_per_launch": per_launch,
                        "launches_per_substep": launches, "avg_launch_us": 1e3 * tot / launches,
                        "share_of_substep": tot / total, "largest_kernel": ranked[0][0]}
    B = substep_bytes(N, F, C, Cf, cfg["solver"], iters)
    achieved = B / (ms / args.steps / 1e3) / 1e9
    substep_roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "alg_bytes_per_substep": B, "pressure_iterations": iters, "system_cells": Cf,
                        "peak_source": peak_src, "mg_levels": lv}

    # End to end through the C ABI with pinned host buffers, one frame per step.
    e2e = None
    if args.e2e_steps > 0:
        hb_in = P.HostBuffer((N, 8))
        hb_out = P.HostBuffer((N, 8))
        hb_in.array[:] = sim.read_particles()
        sim.fluid_advance(0.0)
        frame = 0
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            frame += 1
            lib.pxf_write_particles(sim.h, hb_in.ptr, N)
            rc = lib.pxf_advance_to_frame(sim.h, float(frame))
            if rc != 0:
                raise RuntimeError(lib.pxf_last_error(sim.h).decode())
            lib.pxf_read_particles(sim.h, hb_out.ptr, N)
        el = time.perf_counter() - t0
        e2e = {"value": N * cfg["substeps"] * args.e2e_steps * world / el, "unit": unit,
               "h2d_bytes_per_step": 32 * N, "d2h_bytes_per_step": 32 * N,
               "step": f"one frame: pxf_write_particles + pxf_advance_to_frame ({cfg['substeps']} substeps) "
                       "+ pxf_read_particles, pinned host buffers"}
        hb_in.close()
        hb_out.close()

    # Surface nets of the final particles (the meshing half of the per-frame call): device time of
    # the second call (the first allocates the surface buffers).
    surface = None
    if not args.no_profile:
        sim.surface_mesh()
        m = sim.surface_mesh()
        info = sim.surface_info()
        surface = {"device_ms": m["device_ms"], "vertices": int(m["vertices"].shape[0]),
                   "triangles": int(m["indices"].shape[0]), "overflow": m["overflow"],
                   "surface_cells": list(info["dims"])}

    scene = None
    if rank == 0 and not args.no_profile:
        scene = reference_scene_frames(P)

    precision = None
    if cfg["solver"] == "pcg" and rank == 0:
        precision = {"divergence_linf_dt": divergence_linf(sim)}
        if not args.no_fp64_check:
            precision = fp64_check(sim, cfg["bounds"][0], cfg["iterations"])

    launches_per_substep = sum(k["launches"] for k in kernels) if kernels else None
    solver_stats = None
    if cfg["solver"] == "pcg":
        it, rel, st = sim.solver_stats()
        solver_stats = {"pcg_iterations_last_substep": it, "relres": rel, "status": st}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r = cpu_baseline_run(cfg, 2, 0)
        cpu = {"value": r["value"], "unit": unit, "cores": r["cores"], "kind": r["kind"],
               "sample": "two full substeps of the same workload from the seeded state, all host threads"
                         + (" (pxlengine's shaders/fluid.slang compiled for the CPU)" if r["kind"] == "reference"
                            else " (the oracle's restatement)")}

    if rank == 0:
        line = {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam break, reference LCG seeding)",
                "config": workload_config(args.config, cfg, sim.dims, N), "roofline": roofline,
                "substep_roofline": substep_roofline,
                "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": (launches_per_substep * args.steps) if launches_per_substep else None,
                "solver": solver_stats, "precision": precision, "kernels": kernels, "surface_mesh": surface,
                "reference_scene": scene,
                "wall_s_timed": t_wall}
        print(json.dumps(line), flush=True)
    sim.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
