"""Generates tests/golden/golden.json: known-answer vectors for the liquid path.

Two kinds of entries:
  * values stated by the pxlengine project itself:
      - Fluid::grid of bounds [[0,0,0],[2,1,1]] at resolution 32 is [32,16,16] with h = 0.0625
        (crates/pxl-scene/src/lib.rs:886-899, the reference's unit test `fluids_validate`);
      - the dam-break scene (fill [-0.97,0.03,-0.47]..[-0.35,0.95,0.47] in bounds
        [[-1,0,-0.5],[1,1.2,0.5]], resolution 64, 8 particles per cell) has 139k particles
        (docs/ROADMAP.md:83);
  * vectors computed here by an independent pure-Python restatement (float32 through numpy) of
    lcg() (crates/pxl-render/src/fluid.rs:97-100), the seeding loop (fluid.rs:119-148),
    Fluid::grid (crates/pxl-scene/src/lib.rs:123-128) and steps_for_frame (fluid.rs:234-236).
Seeded particles are stored as a count, a SHA-256 of the first `hashed` particles as float32
[N, 8] and the first 64 particles in clear. The CPU oracle (C++) and the CUDA library are both
checked against this file.

Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import math
import os

import numpy as np

F = np.float32
MASK = (1 << 64) - 1


def lcg(s):
    s = (s * 6364136223846793005 + 1442695040888963407) & MASK
    return F(F(s >> 40) / F(1 << 24)), s


def rust_round(x):
    # f32::round: half away from zero
    return F(math.floor(abs(float(x)) + 0.5) * (1 if x >= 0 else -1))


def grid(bounds, res):
    size = [F(F(bounds[1][a]) - F(bounds[0][a])) for a in range(3)]
    h = F(max(size) / F(res))
    n = []
    for a in range(3):
        v = rust_round(F(size[a] / h))
        n.append(int(max(v, F(4.0))))
    return n, h


def seed_particles(bounds, res, fill, ppc, seed, limit=None):
    n, h = grid(bounds, res)
    o = [F(x) for x in bounds[0]]
    rng = 0x9E3779B97F4A7C15 ^ seed
    out = []
    count = 0
    for b in fill:
        mn = [F(x) for x in b["min"]]
        mx = [F(x) for x in b["max"]]
        vel = [F(x) for x in b.get("velocity", [0, 0, 0])]
        for k in range(1, n[2] - 1):
            for j in range(1, n[1] - 1):
                for i in range(1, n[0] - 1):
                    c = [F(o[0] + F(F(F(i) + F(0.5)) * h)), F(o[1] + F(F(F(j) + F(0.5)) * h)),
                         F(o[2] + F(F(F(k) + F(0.5)) * h))]
                    if any(c[a] < mn[a] or c[a] > mx[a] for a in range(3)):
                        continue
                    for _ in range(ppc):
                        rx, rng = lcg(rng)
                        ry, rng = lcg(rng)
                        rz, rng = lcg(rng)
                        p = [F(o[0] + F(F(F(i) + rx) * h)), F(o[1] + F(F(F(j) + ry) * h)),
                             F(o[2] + F(F(F(k) + rz) * h))]
                        if limit is None or count < limit:
                            out.append([float(p[0]), float(p[1]), float(p[2]), 0.0,
                                        float(vel[0]), float(vel[1]), float(vel[2]), 0.0])
                        count += 1
    return count, out


def steps_for_frame(warmup, fps, substeps, frame):
    v = (warmup + frame / fps) * fps * substeps
    r = math.floor(abs(v) + 0.5) * (1 if v >= 0 else -1)
    return int(max(r, 0.0))


def main():
    g = {}
    g["grid"] = []
    for bounds, res in [([[0, 0, 0], [2, 1, 1]], 32), ([[-1, 0, -0.5], [1, 1.2, 0.5]], 64),
                        ([[0, 0, 0], [1, 0.5, 0.5]], 64), ([[0, 0, 0], [1, 0.5, 0.5]], 256),
                        ([[0, 0, 0], [0.3, 0.05, 1]], 16), ([[-2, -1, 0], [2.5, 1.5, 0.75]], 100)]:
        n, h = grid(bounds, res)
        g["grid"].append({"bounds": bounds, "resolution": res, "n": n, "h": float(h)})
    s = 0x9E3779B97F4A7C15
    vals = []
    for _ in range(64):
        v, s = lcg(s)
        vals.append(float(v))
    g["lcg_seed0_first64"] = vals
    g["lcg_seed0_state_after64"] = str(s)
    g["seeding"] = []
    cases = [
        ("dam_break", [[-1, 0, -0.5], [1, 1.2, 0.5]], 64,
         [{"min": [-0.97, 0.03, -0.47], "max": [-0.35, 0.95, 0.47]}], 8, 0, 512),
        ("two_blocks_seed7", [[0, 0, 0], [1, 0.5, 0.5]], 32,
         [{"min": [0, 0, 0], "max": [0.3, 0.3, 0.5], "velocity": [1.0, 0.0, -0.5]},
          {"min": [0.7, 0.0, 0.1], "max": [1.0, 0.3, 0.4], "velocity": [-1.0, 0.25, 0.0]}], 4, 7, None),
        ("small_ppc1_seed3", [[0, 0, 0], [1, 1, 1]], 16, [{"min": [0.2, 0.2, 0.2], "max": [0.8, 0.6, 0.9]}], 1, 3,
         None),
    ]
    for name, bounds, res, fill, ppc, seed, limit in cases:
        count, parts = seed_particles(bounds, res, fill, ppc, seed, limit)
        digest = hashlib.sha256(np.asarray(parts, dtype=np.float32).tobytes()).hexdigest()
        g["seeding"].append({"name": name, "bounds": bounds, "resolution": res, "fill": fill, "ppc": ppc,
                             "seed": seed, "count": count, "hashed": len(parts), "sha256_f32": digest,
                             "first": parts[:64]})
    g["steps_for_frame"] = [
        {"warmup": w, "fps": fps, "substeps": ss, "frame": fr, "steps": steps_for_frame(w, fps, ss, fr)}
        for (w, fps, ss, fr) in [(0, 24, 8, 0), (0, 24, 8, 1), (0, 24, 8, 59.5), (0.5, 24, 8, 3),
                                 (0, 15, 8, 25), (0.25, 30, 5, 10.25), (0, 24, 8, -3)]]
    g["reference_stated"] = {"fluids_validate_grid": [32, 16, 16], "fluids_validate_h": 0.0625,
                             "dam_break_particles_approx": 139000}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as f:
        json.dump(g, f, separators=(",", ":"))
    print(path)


if __name__ == "__main__":
    main()
