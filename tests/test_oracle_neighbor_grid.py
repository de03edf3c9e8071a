"""The agent neighbour grid restatement (oracle/neighbor_grid.py) against a literal, loop-by-loop
restatement of the reference's six kernels (shaders/sim.slang:28-104), and the table-size rule of
crates/pxl-render/src/sim.rs:129 in the oracle and in the library (a host-only call)."""
import numpy as np

from oracle import neighbor_grid as NG


def _reference_kernels(pos, cell_size, table):
    """grid_clear, grid_count, scan_local (1024 counts per group), scan_blocks, scan_add and
    grid_scatter, one invocation after another in index order."""
    cs = np.float32(max(np.float32(cell_size), np.float32(1e-6)))
    def cell(i):
        c = [int(np.floor(np.float32(pos[i, a]) / cs)) & 0xFFFFFFFF for a in range(3)]
        return (((c[0] * 73856093) & 0xFFFFFFFF) ^ ((c[1] * 19349663) & 0xFFFFFFFF) ^
                ((c[2] * 83492791) & 0xFFFFFFFF)) & (table - 1)
    counts = [0] * table                                   # grid_clear
    for i in range(pos.shape[0]):                          # grid_count
        counts[cell(i)] += 1
    n_blocks = table // 1024
    offsets, block_sums = [0] * table, [0] * max(n_blocks, 1)
    for g in range(n_blocks):                              # scan_local
        run = 0
        for k in range(1024):
            offsets[g * 1024 + k] = run
            run += counts[g * 1024 + k]
        block_sums[g] = run
    run = 0                                                # scan_blocks
    for g in range(n_blocks):
        x = block_sums[g]
        block_sums[g] = run
        run += x
    cursor = [0] * table                                   # scan_add
    for i in range(table):
        offsets[i] += block_sums[i // 1024]
        cursor[i] = offsets[i]
    out = [0] * pos.shape[0]                               # grid_scatter
    for i in range(pos.shape[0]):
        h = cell(i)
        out[cursor[h]] = i
        cursor[h] += 1
    return np.array(offsets, np.uint32), np.array(counts, np.uint32), np.array(out, np.uint32)


def test_oracle_matches_reference_kernels():
    rng = np.random.default_rng(3)
    pos = rng.uniform(-3.0, 3.0, (3000, 3)).astype(np.float32)
    pos[:200] = pos[0]                                      # a crowded cell
    pos[200:210, 0] = 0.0                                   # cell boundaries
    for cell_size, table in ((0.25, 1024), (0.05, 4096), (0.0, 2048)):
        o, c, s = NG.grid_sort(pos, cell_size, table)
        ro, rc, rs = _reference_kernels(pos, cell_size, table)
        np.testing.assert_array_equal(c, rc)
        np.testing.assert_array_equal(o, ro)
        np.testing.assert_array_equal(s, rs)   # the sequential scatter lists ids ascending too


def test_table_size_rule(lib):
    for n, want in ((0, 1024), (1, 1024), (512, 1024), (513, 2048), (600, 2048), (100000, 262144),
                    (4194304, 1 << 23), (50000000, 1 << 23)):
        assert NG.table_size(n) == want
        assert lib.pxf_grid_table_size(n) == want
    assert lib.pxf_grid_scratch_bytes(1000, 1024) >= 4000
