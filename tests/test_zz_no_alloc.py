"""The allocation-free entry point pgsvt_svd_window_noalloc, through the C ABI.

It exists for callers that cannot allocate device memory while they work
(acquisition loops with memory reserved up front, code under an allocator
that owns the device, or processes that avoid cudaMalloc/cudaFree because
they synchronise the device).  Its intermediates live in a fixed static
device array shared by all calls, so two calls in a row on different windows
must each match the allocating entry point, pgsvt_svd_window.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _noalloc(capi, u, rows, cols, bs, with_output=True, expect=None):
    """Call the entry point on device copies of (u, rows, cols); with `expect`
    set, return the status code of the computing call instead of asserting."""
    import torch
    side, nwin = u.shape[0], u.shape[2]
    ud = torch.from_numpy(np.ascontiguousarray(np.asarray(u, np.float32).ravel(order="F"))).cuda()
    rd = torch.from_numpy(np.ascontiguousarray(rows, np.int32)).cuda()
    cd = torch.from_numpy(np.ascontiguousarray(cols, np.int32)).cuda()
    n = ctypes.c_uint32()
    L = capi.load()
    rc = L.pgsvt_svd_window_noalloc(ctypes.c_void_p(ud.data_ptr()), side, nwin, bs, 1,
                                    ctypes.c_void_p(rd.data_ptr()), ctypes.c_void_p(cd.data_ptr()),
                                    None, ctypes.byref(n), None)
    assert rc == capi.OK, L.pgsvt_last_error()
    if not with_output:
        return n.value, None
    S = torch.zeros(n.value * nwin, dtype=torch.float32, device="cuda")
    rc = L.pgsvt_svd_window_noalloc(ctypes.c_void_p(ud.data_ptr()), side, nwin, bs, 1,
                                    ctypes.c_void_p(rd.data_ptr()), ctypes.c_void_p(cd.data_ptr()),
                                    ctypes.c_void_p(S.data_ptr()), ctypes.byref(n), None)
    torch.cuda.synchronize()
    if expect is not None:
        return rc, S.cpu().numpy().reshape(n.value, nwin)
    assert rc == capi.OK, L.pgsvt_last_error()
    return n.value, S.cpu().numpy().reshape(n.value, nwin)


def _window(pkg, side, seed):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=seed, side=side, nt=15)
    u = noisy.astype(np.float64)
    return u / u.max()


def test_noalloc_matches_allocating_entry_point_twice(capi, pkg):
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    cases = [(g["u_8"], g["rows_8"], g["cols_8"], 4)]
    u2 = _window(pkg, 24, 9)  # a different, smaller window on the second call
    r2, c2 = capi.arps_window(u2, 4, 5, 7, 7, 15)
    cases.append((u2, r2, c2, 4))
    u3 = _window(pkg, 20, 5)[:, :, 4:11]  # 3x3 patches, 7 frames: the 10-column kernel
    r3, c3 = capi.arps_window(u3, 3, 5, 3, 3, 7)
    cases.append((u3, r3, c3, 3))
    for u, rows, cols, bs in cases:
        u32 = np.asarray(u, np.float32).astype(np.float64)  # the entry point takes float
        ref = capi.svd_window(u32, bs, 1, rows, cols)
        n, _ = _noalloc(capi, u32, rows, cols, bs, with_output=False)  # size query
        assert n == ref.shape[0] == (u.shape[0] - bs + 1) ** 2
        n, S = _noalloc(capi, u32, rows, cols, bs)
        assert n == ref.shape[0]
        # the same kernel on the same data: equal to FP32 rounding
        np.testing.assert_allclose(S, ref, rtol=1e-6, atol=1e-7)
    # and the first case against the frozen FP64 oracle singular values, at the
    # tolerance of the parity tests (2e-5 of each patch's largest value)
    n, S = _noalloc(capi, np.asarray(g["u_8"], np.float32).astype(np.float64), g["rows_8"],
                    g["cols_8"], 4)
    So = g["S_8"]
    assert np.all(np.abs(S - So) <= 2e-5 * So[:, :1])


def test_noalloc_rejects_out_of_frame_trajectories(capi):
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    u, rows, cols = g["u_8"], g["rows_8"].copy(), g["cols_8"].copy()
    side, bs = u.shape[0], 4
    rows[3, 17] = side - bs + 1  # one patch row past the last valid position
    rc, _ = _noalloc(capi, u, rows, cols, bs, expect=True)
    assert rc == capi.ERR_INVALID_ARG
    assert b"outside the frame" in capi.load().pgsvt_last_error()
    # the shared array holds no state that breaks the next good call
    n, S = _noalloc(capi, u, g["rows_8"], g["cols_8"], bs)
    assert np.all(np.abs(S - g["S_8"]) <= 2e-5 * g["S_8"][:, :1])


def test_noalloc_non_finite_pixels_return_cleanly(capi):
    """An infinite or huge pixel gives non-finite singular values for the
    patches that cover it and finite ones elsewhere; no factor is written."""
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    rows, cols, bs = g["rows_8"], g["cols_8"], 4
    for bad in (np.inf, 3e38):
        u = np.asarray(g["u_8"], np.float64).copy()
        u[5, 9, 7] = bad
        rc, S = _noalloc(capi, u, rows, cols, bs, expect=True)
        assert rc == capi.OK, capi.load().pgsvt_last_error()
        assert S.shape == g["S_8"].shape
        assert np.isfinite(S).sum() > 0.9 * S.size


def test_noalloc_rejects_oversize_windows(capi):
    import torch
    L = capi.load()
    n = ctypes.c_uint32()
    buf = torch.zeros(16, device="cuda")
    side = capi.NOALLOC_MAX_SIDE + 1
    rc = L.pgsvt_svd_window_noalloc(ctypes.c_void_p(buf.data_ptr()), side, 15, 4, 1,
                                    ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()),
                                    ctypes.c_void_p(buf.data_ptr()), ctypes.byref(n), None)
    assert rc == capi.ERR_INVALID_ARG
    assert b"no-allocation limit" in L.pgsvt_last_error()
