"""CPU oracle for the FLIP liquid substep — test infrastructure only.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU legs as the checker and as the
timed CPU baseline. Never imported by the pxlengine_gb300 package.
"""
from .oracle import (PARTICLES, VEL, VEL_OLD, ACC, WACC, CELL_COUNT, CELL_TYPE, PRESSURE,  # noqa: F401
                     DIVERGENCE, PRESSURE64, STAGES)
from .oracle import OracleSim, grid, lcg, seed_particles, steps_for_frame, dt_for, num_threads, load  # noqa: F401
from .oracle import surface_nets  # noqa: F401
