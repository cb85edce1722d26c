"""The allocation-free broad phase against the context's broad phase.

dem_broad_phase_noalloc() serves callers that cannot call cudaMalloc (a
framework pool owning the device heap, an allocator that forbids it, a loop
that must not block on it): they pass device buffers they own, and the
library's only scratch is a fixed array compiled into it.  This test runs it
twice in a row on the same context state -- the second call sees the scratch
left over by the first -- and requires keys, stable order and cell table to be
identical to the context's own broad phase (dem_debug_broad_phase), which uses
device memory the context allocated.  Integer outputs: exact equality.

The file sorts last so that a run stopping at the first failure has already
run every other test.
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


def test_noalloc_broad_phase_equals_context_broad_phase():
    torch = pytest.importorskip("torch")
    L = _lib()
    n = 3000
    sc, p, ext = dem_scenes.dense_bed(n=n, seed=4)
    dev = torch.device("cuda", 0)
    with dem.Context(sc, p, device=0) as ctx:
        x0, y0, inv, gw, gh = ctx.search_grid()
        assert gw * gh + 1 <= 262144
        d_keys = torch.empty(n, dtype=torch.int32, device=dev)
        d_order = torch.empty(n, dtype=torch.int32, device=dev)
        d_cs = torch.empty(gw * gh + 2, dtype=torch.int32, device=dev)
        for call in range(2):
            ctx.step(25)
            st = ctx.download()
            keys_ref, order_ref, cs_ref = ctx.broad_phase()
            pr = np.zeros((n, 4), np.float32)
            pr[:, :2] = st["pos"].reshape(-1, 2)
            pr[:, 2] = st["radii"]
            d_pr = torch.from_numpy(pr).to(dev)
            d_keys.fill_(-7)
            d_order.fill_(-7)
            d_cs.fill_(-7)
            torch.cuda.synchronize(dev)
            rc = L.dem_broad_phase_noalloc(d_pr.data_ptr(), n, x0, y0, inv, gw, gh, d_keys.data_ptr(),
                                           d_order.data_ptr(), d_cs.data_ptr(), None)
            assert rc == 0, L.dem_noalloc_last_error()
            torch.cuda.synchronize(dev)
            assert np.array_equal(d_keys.cpu().numpy(), keys_ref), "keys differ on call %d" % call
            assert np.array_equal(d_order.cpu().numpy(), order_ref), "order differs on call %d" % call
            assert np.array_equal(d_cs.cpu().numpy(), cs_ref), "cell table differs on call %d" % call


def test_noalloc_rejects_grids_beyond_its_scratch():
    L = _lib()
    rc = L.dem_broad_phase_noalloc(None, 0, 0.0, 0.0, 1.0, 1024, 1024, None, None, None, None)
    assert rc == -7  # DEM_E_CAPACITY, before any device work
    assert b"DEM_NOALLOC_MAX_CELLS" in L.dem_noalloc_last_error()
