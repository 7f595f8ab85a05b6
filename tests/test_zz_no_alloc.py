"""The allocation-free mean removal, pcd_subtract_average_noalloc.

It exists for callers that cannot let a library allocate device memory (a
host application whose device-memory budget belongs to its own pool, or a
latency-critical path where cudaMalloc would synchronise the device).  Its
scratch is a static device array sized for at most 16384 grid rows.

This file is collected last, so a run that stops at the first failure has
already run every other test.  It must also pass on its own in a fresh
process: the first call on the device performs the symbol-address set-up.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from poisson_caustic_design_gb300 import _lib

    return _lib.load()


def _run_existing(L, ctx, g, w, h, stream):
    st = L.pcd_subtract_average_device(ctx.handle, C.c_void_p(g.data_ptr()), w, h, C.c_void_p(stream))
    assert st == 0


def test_noalloc_matches_existing_entry_point_twice():
    import torch

    import poisson_caustic_design_gb300 as pcd

    L = _lib()
    ctx = pcd.Context(0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(123)
    # two calls in a row with different grids: the second must not see the
    # first call's scratch contents
    for (h, w, shift) in ((300, 257, 3.0), (1024, 96, -7.5)):
        a = rng.standard_normal((h, w)) + shift
        a[5, 7] = np.nan                       # NaN cells are skipped, as in utils.cpp:60-86
        ref = torch.from_numpy(a).cuda()
        out = ref.clone()
        _run_existing(L, ctx, ref, w, h, stream)
        st = L.pcd_subtract_average_noalloc(C.c_void_p(out.data_ptr()), w, h, C.c_void_p(stream))
        assert st == 0, L.pcd_last_error().decode()
        torch.cuda.synchronize()
        r, o = ref.cpu().numpy(), out.cpu().numpy()
        assert np.array_equal(np.isnan(r), np.isnan(o))
        m = ~np.isnan(r)
        # both reduce in FP64, in different orders: agree to rounding
        np.testing.assert_allclose(o[m], r[m], rtol=0, atol=1e-12 * np.abs(a[m]).max())
        assert abs(np.nanmean(o)) < 1e-12 * np.abs(a[m]).max()
    ctx.close()


@pytest.mark.parametrize("h,w,fill", [
    (16384, 8, "normal"),   # the largest accepted height: the scratch's last row slot
    (4, 4, "nan"),          # every cell NaN: the 0/0 mean leaves every cell NaN, as utils.cpp:60-86 does
    (3, 5000, "normal"),    # rows much wider than the 256-thread block (row-strided loop)
])
def test_noalloc_edges_match_existing_entry_point(h, w, fill):
    import torch

    import poisson_caustic_design_gb300 as pcd

    L = _lib()
    ctx = pcd.Context(0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(h * 7 + w)
    a = np.full((h, w), np.nan) if fill == "nan" else rng.standard_normal((h, w)) + 2.5
    ref = torch.from_numpy(a).cuda()
    _run_existing(L, ctx, ref, w, h, stream)
    for _ in range(2):   # two calls in a row on fresh copies of the same grid
        o_t = torch.from_numpy(a).cuda()
        st = L.pcd_subtract_average_noalloc(C.c_void_p(o_t.data_ptr()), w, h, C.c_void_p(stream))
        assert st == 0, L.pcd_last_error().decode()
        torch.cuda.synchronize()
        r, o = ref.cpu().numpy(), o_t.cpu().numpy()
        assert np.array_equal(np.isnan(r), np.isnan(o))
        m = ~np.isnan(r)
        if m.any():
            np.testing.assert_allclose(o[m], r[m], rtol=0, atol=1e-12 * np.abs(a[m]).max())
    ctx.close()


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch

    L = _lib()
    g = torch.zeros((4,), dtype=torch.float64, device="cuda")
    st = L.pcd_subtract_average_noalloc(C.c_void_p(g.data_ptr()), 1, 16385, None)
    assert st == 2  # PCD_BAD_ARG
    assert "16384" in L.pcd_last_error().decode()
