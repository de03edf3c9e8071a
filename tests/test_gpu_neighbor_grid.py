"""pxf_grid_sort, the agent neighbour grid (shaders/sim.slang:28-104), through the C ABI against the
oracle restatement: counts and offsets bit for bit, every cell's agent ids equal as a set (the
order inside a cell is unspecified, as in the reference). Device buffers come from torch."""
import ctypes as C

import numpy as np
import pytest

from oracle import neighbor_grid as NG

pytestmark = pytest.mark.gpu
STRIDE = 16   # floats per agent record (the reference's Agent: position, size, velocity, age, colour, data)


def _run(lib, torch, pos, cell_size, table, calls=1):
    n = pos.shape[0]
    rec = np.zeros((n, STRIDE), dtype=np.float32)
    rec[:, :3] = pos
    rec[:, 3:] = np.float32(7.0)   # other fields: not read
    d_rec = torch.from_numpy(rec).to("cuda")
    off = torch.full((table,), -1, dtype=torch.int32, device="cuda")
    cnt = torch.full((table,), -1, dtype=torch.int32, device="cuda")
    srt = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    sb = lib.pxf_grid_scratch_bytes(n, table)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    for _ in range(calls):
        rc = lib.pxf_grid_sort(C.c_void_p(d_rec.data_ptr()), STRIDE, n, C.c_float(cell_size), table,
                               C.c_void_p(off.data_ptr()), C.c_void_p(cnt.data_ptr()), C.c_void_p(srt.data_ptr()),
                               C.c_void_p(scratch.data_ptr()), sb, None)
        assert rc == 0, lib.pxf_last_error(None).decode()
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    return u(off), u(cnt), u(srt)[:n]


def _check(pos, cell_size, table, got):
    off, cnt, srt = got
    wo, wc, ws = NG.grid_sort(pos, cell_size, table)
    np.testing.assert_array_equal(cnt, wc)
    np.testing.assert_array_equal(off, wo)
    # same ids per cell: sort each cell's slice of the GPU output, compare with the oracle's
    h = NG.cells(pos, cell_size, table)
    key = h[srt].astype(np.int64) * (len(srt) + 1) + srt
    np.testing.assert_array_equal(np.sort(key), (h[ws].astype(np.int64) * (len(srt) + 1) + ws))
    np.testing.assert_array_equal(h[srt], np.repeat(np.arange(table, dtype=np.uint32), wc))


@pytest.mark.parametrize("n,cell_size,spread", [(300000, 0.05, 4.0), (100000, 0.5, 40.0), (5000, 0.01, 0.001),
                                                 (70000, 0.0, 1.0)])
def test_grid_sort_matches_oracle(lib, n, cell_size, spread):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    pos = rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
    table = lib.pxf_grid_table_size(n)
    _check(pos, cell_size, table, _run(lib, torch, pos, cell_size, table, calls=2))


def test_grid_sort_edges(lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    # every agent in one cell, a small table with many collisions, the largest table, no agents
    pile = np.full((20000, 3), 0.3, dtype=np.float32)
    _check(pile, 0.1, 1024, _run(lib, torch, pile, 0.1, 1024))
    many = rng.uniform(-50, 50, (200000, 3)).astype(np.float32)
    _check(many, 0.2, 1024, _run(lib, torch, many, 0.2, 1024))
    _check(many, 0.2, 1 << 23, _run(lib, torch, many, 0.2, 1 << 23))
    off, cnt, _ = _run(lib, torch, np.zeros((0, 3), np.float32), 0.1, 1024)
    assert not off.any() and not cnt.any()


def test_grid_sort_rejects_bad_arguments(lib):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(4096, dtype=torch.int32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    assert lib.pxf_grid_sort(p, 16, 10, C.c_float(0.1), 1000, p, p, p, p, 1 << 20, None) == -1
    assert "power of two" in lib.pxf_last_error(None).decode()
    assert lib.pxf_grid_sort(p, 16, 10, C.c_float(0.1), 1024, p, p, p, p, 16, None) == -1
    assert "scratch" in lib.pxf_last_error(None).decode()
