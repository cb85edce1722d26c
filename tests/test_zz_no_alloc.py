"""The allocation-free broad phase against the context's broad phase and a
numpy stable sort.

dem_broad_phase_noalloc() serves callers that cannot call cudaMalloc (a
framework pool owning the device heap, an allocator that forbids it, a loop
that must not block on it): they pass device buffers they own, and the
library's only scratch is a fixed array compiled into it, which every call
shares and which keeps the previous call's contents.  The test calls it
several times in a row, each call seeing the scratch the one before left:

- twice on the context's grid and current positions, requiring keys, stable
  order and cell table identical to the context's own broad phase
  (dem_debug_broad_phase, which uses device memory the context allocated;
  the scene has no large particles, the one case where the two differ);
- then on a finer grid (more cells) and a coarser one (fewer cells), with
  some radii set to 0 and some particles moved beyond the grid, against a
  numpy stable lexsort of the keys numpy derives with the same float32
  arithmetic.

Integer outputs: exact equality.  The file sorts last so that a run stopping
at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import dem
import dem_scenes

pytestmark = pytest.mark.gpu


def _lib():
    import build_lib
    build_lib.build()
    L = dem.lib()
    L.dem_broad_phase_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float,
                                          C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]
    L.dem_broad_phase_noalloc.restype = C.c_int
    L.dem_noalloc_last_error.restype = C.c_char_p
    return L


def _numpy_broad_phase(pr, x0, y0, inv, gw, gh):
    f = np.float32
    qx = np.floor((pr[:, 0] - f(x0)) * f(inv)).astype(np.int64)
    qy = np.floor((pr[:, 1] - f(y0)) * f(inv)).astype(np.int64)
    keys = np.clip(qy, 0, gh - 1) * gw + np.clip(qx, 0, gw - 1)
    keys[pr[:, 2] == 0] = gw * gh
    order = np.lexsort((np.arange(len(keys)), keys))
    counts = np.bincount(keys, minlength=gw * gh + 1)
    return keys, order, np.concatenate([[0], np.cumsum(counts)])


def _call(L, torch, dev, pr, grid):
    n = pr.shape[0]
    x0, y0, inv, gw, gh = grid
    d_pr = torch.from_numpy(np.ascontiguousarray(pr)).to(dev)
    d_keys = torch.full((n,), -7, dtype=torch.int32, device=dev)
    d_order = torch.full((n,), -7, dtype=torch.int32, device=dev)
    d_cs = torch.full((gw * gh + 2,), -7, dtype=torch.int32, device=dev)
    torch.cuda.synchronize(dev)
    rc = L.dem_broad_phase_noalloc(d_pr.data_ptr(), n, x0, y0, inv, gw, gh, d_keys.data_ptr(),
                                   d_order.data_ptr(), d_cs.data_ptr(), None)
    assert rc == 0, L.dem_noalloc_last_error()
    torch.cuda.synchronize(dev)
    return d_keys.cpu().numpy(), d_order.cpu().numpy(), d_cs.cpu().numpy()


def test_noalloc_broad_phase_equals_context_broad_phase_and_numpy():
    torch = pytest.importorskip("torch")
    L = _lib()
    n = 3000
    sc, p, ext = dem_scenes.dense_bed(n=n, seed=4)
    dev = torch.device("cuda", 0)
    with dem.Context(sc, p, device=0) as ctx:
        grid = ctx.search_grid()
        x0, y0, inv, gw, gh = grid
        assert gw * gh + 1 <= 262144
        for call in range(2):
            ctx.step(25)
            st = ctx.download()
            keys_ref, order_ref, cs_ref = ctx.broad_phase()
            pr = np.zeros((n, 4), np.float32)
            pr[:, :2] = st["pos"].reshape(-1, 2)
            pr[:, 2] = st["radii"]
            keys, order, cs = _call(L, torch, dev, pr, grid)
            assert np.array_equal(keys, keys_ref), "keys differ on call %d" % call
            assert np.array_equal(order, order_ref), "order differs on call %d" % call
            assert np.array_equal(cs, cs_ref), "cell table differs on call %d" % call
            nk, no, ncs = _numpy_broad_phase(pr, *grid)
            assert np.array_equal(keys, nk) and np.array_equal(order, no) and np.array_equal(cs, ncs)
    # zero radii, particles beyond the grid on every side, then a finer and a coarser grid
    rng = np.random.default_rng(3)
    pr[rng.choice(n, 300, replace=False), 2] = 0.0
    far = rng.choice(n, 120, replace=False)
    span = np.float32(gw / inv)
    pr[far[:30], 0] += 3 * span
    pr[far[30:60], 0] -= 3 * span
    pr[far[60:90], 1] += 3 * span
    pr[far[90:], :2] -= 3 * span
    for cell in (0.5, 2.0):  # cell side relative to the context's: more cells, then fewer
        g2 = (x0, y0, float(np.float32(inv / cell)), int(gw / cell) + 1, int(gh / cell) + 1)
        assert g2[3] * g2[4] + 1 <= 262144
        keys, order, cs = _call(L, torch, dev, pr, g2)
        nk, no, ncs = _numpy_broad_phase(pr, *g2)
        assert np.array_equal(keys, nk), "keys differ with cells %g x the context's" % cell
        assert np.array_equal(order, no), "order differs with cells %g x the context's" % cell
        assert np.array_equal(cs, ncs), "cell table differs with cells %g x the context's" % cell


def test_noalloc_crowded_cells():
    """Every particle in one cell, and half of them with radius 0: the order
    is still the index order within each cell (a counting sort, whose cost
    does not depend on how many particles share a cell)."""
    torch = pytest.importorskip("torch")
    L = _lib()
    n = 200000
    pr = np.zeros((n, 4), np.float32)
    pr[:, 0] = 1e6
    pr[:, 1] = -1e6
    pr[:, 2] = 1.0
    pr[::2, 2] = 0.0
    grid = (0.0, 0.0, 0.5, 400, 300)
    keys, order, cs = _call(L, torch, torch.device("cuda", 0), pr, grid)
    nk, no, ncs = _numpy_broad_phase(pr, *grid)
    assert np.array_equal(keys, nk) and np.array_equal(order, no) and np.array_equal(cs, ncs)


def test_noalloc_rejects_sizes_beyond_its_limits():
    L = _lib()
    rc = L.dem_broad_phase_noalloc(None, 0, 0.0, 0.0, 1.0, 1024, 1024, None, None, None, None)
    assert rc == -7  # DEM_E_CAPACITY, before any device work
    assert b"DEM_NOALLOC_MAX_CELLS" in L.dem_noalloc_last_error()
    rc = L.dem_broad_phase_noalloc(None, (1 << 30) + 1, 0.0, 0.0, 1.0, 16, 16, None, None, None, None)
    assert rc == -7
    assert b"2^30" in L.dem_noalloc_last_error()
