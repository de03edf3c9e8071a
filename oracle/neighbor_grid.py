"""CPU restatement of the agent neighbour grid (test infrastructure: the checker of pxf_grid_sort).

Follows shaders/sim.slang:28-104 and crates/pxl-render/src/sim.rs:129,181:
- cell_hash (sim.slang:28-30): ((uint(cx) * 73856093) ^ (uint(cy) * 19349663) ^ (uint(cz) * 83492791))
  & (table_size - 1), 32-bit unsigned arithmetic, with c = int3(floor(position / cell_size))
  (agent_cell, sim.slang:31) and cell_size = max(cell_size, 1e-6) (sim.rs:181);
- grid_count (sim.slang:39-41): agents per hashed cell;
- scan_local / scan_blocks / scan_add (sim.slang:43-95): exclusive prefix sum of the counts;
- grid_scatter (sim.slang:97-103): agent ids grouped by cell. The reference's order inside a cell
  follows its atomics; this restatement lists them in ascending id order.
The division is IEEE float32 (numpy), the same operation the CUDA kernel uses.
Pinned to the reference's own shader: tests/test_oracle_vs_reference.py runs sim.slang's grid
kernels on the CPU (oracle/ref_sim.cpp) and finds the same offsets and counts and the same ids per
cell.
"""
import numpy as np

TABLE_MIN, TABLE_MAX = 1024, 1 << 23


def table_size(count: int) -> int:
    """(count * 2).next_power_of_two().clamp(1024, 1 << 23) (sim.rs:129)."""
    t = 1
    while t < count * 2:
        t <<= 1
    return int(min(max(t, TABLE_MIN), TABLE_MAX))


def cells(positions, cell_size, table_size):
    p = np.asarray(positions, dtype=np.float32).reshape(-1, 3)
    cs = np.float32(max(np.float32(cell_size), np.float32(1e-6)))
    c = np.floor(p / cs).astype(np.int64) & 0xFFFFFFFF
    h = ((c[:, 0] * 73856093) & 0xFFFFFFFF) ^ ((c[:, 1] * 19349663) & 0xFFFFFFFF) ^ ((c[:, 2] * 83492791) & 0xFFFFFFFF)
    return (h & (table_size - 1)).astype(np.uint32)


def grid_sort(positions, cell_size, table_size):
    """(offsets, counts, sorted) of the neighbour grid; sorted lists each cell's ids ascending."""
    h = cells(positions, cell_size, table_size)
    counts = np.bincount(h, minlength=table_size).astype(np.uint32)
    offsets = np.zeros(table_size, dtype=np.uint32)
    offsets[1:] = np.cumsum(counts[:-1], dtype=np.uint64).astype(np.uint32)
    order = np.argsort(h, kind="stable").astype(np.uint32)
    return offsets, counts, order
