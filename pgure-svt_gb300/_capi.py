"""ctypes binding of libpgsvt.so (include/pgsvt.h).

This is the Python-side binding a maintainer of the reference would add in
place of its Cython extension (pguresvt/_pguresvt.pyx:143-383): plain
pointers and sizes, no Armadillo and no torch types.  Loading fails loudly
when the CUDA library is missing; there is no CPU path behind it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpgsvt.so")

PGSVT_U8, PGSVT_U16, PGSVT_F32, PGSVT_F64 = 0, 1, 2, 3
DTYPES = {np.dtype("uint8"): PGSVT_U8, np.dtype("uint16"): PGSVT_U16,
          np.dtype("float32"): PGSVT_F32, np.dtype("float64"): PGSVT_F64}

OK, ERR_INVALID_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_OOM, ERR_TIMEOUT, ERR_NONFINITE = range(7)

COMPAT_SWAP_MU_SIGMA = 0x1
COMPAT_ZERO_MOTION = 0x2
COMPAT_INT_DELTA1 = 0x4
COMPAT_ALL = 0x7

# every symbol include/pgsvt.h declares
EXPORTS = ("pgsvt_default_params", "pgsvt_denoise", "pgsvt_denoise_device",
           "pgsvt_arps_window", "pgsvt_svd_window", "pgsvt_reconstruct_window",
           "pgsvt_risk_window", "pgsvt_svd_window_noalloc", "pgsvt_last_error",
           "pgsvt_version")
NOALLOC_MAX_SIDE = 64
NOALLOC_MAX_NWIN = 15


class Params(ctypes.Structure):
    """pgsvt_params: the arguments of PGURESVT (pguresvt.hpp:17-38)."""
    _fields_ = [
        ("traj_length", ctypes.c_uint32), ("block_size", ctypes.c_uint32),
        ("block_overlap", ctypes.c_uint32), ("motion_window", ctypes.c_uint32),
        ("median_size", ctypes.c_int64), ("noise_method", ctypes.c_uint32),
        ("max_iter", ctypes.c_uint32), ("n_jobs", ctypes.c_int64),
        ("random_seed", ctypes.c_int64), ("optimize_pgure", ctypes.c_int32),
        ("exp_weighting", ctypes.c_int32), ("motion_estimation", ctypes.c_int32),
        ("verbose", ctypes.c_int32), ("lambda_", ctypes.c_double),
        ("alpha", ctypes.c_double), ("mu", ctypes.c_double), ("sigma", ctypes.c_double),
        ("tol", ctypes.c_double), ("compat_flags", ctypes.c_uint32),
        ("search_points", ctypes.c_uint32), ("search_rounds", ctypes.c_uint32),
        ("window_batch", ctypes.c_uint32), ("lambda_hint", ctypes.c_double),
        ("hint_span", ctypes.c_double), ("frame_begin", ctypes.c_uint32),
        ("frame_end", ctypes.c_uint32),
    ]


STAGES = ("convert", "normalise", "arps", "fields", "svd", "search", "output", "uploads")


class Status(ctypes.Structure):
    _fields_ = [
        ("code", ctypes.c_int32), ("cuda_error", ctypes.c_int32),
        ("windows", ctypes.c_uint64), ("risk_evals", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64), ("h2d_bytes", ctypes.c_uint64),
        ("d2h_bytes", ctypes.c_uint64), ("seconds", ctypes.c_double),
        ("stage_seconds", ctypes.c_double * 8), ("svd_launches", ctypes.c_uint64),
        ("svd_matrices", ctypes.c_uint64), ("arps_exact_steps", ctypes.c_uint64),
        ("svd_fp64_tests", ctypes.c_uint64), ("svd_warp_sweeps", ctypes.c_uint64),
        ("message", ctypes.c_char * 256),
    ]


class PgsvtError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("pgsvt error %d: %s" % (code, message))
        self.code = code


_lib = None


def load(path=LIB_PATH):
    """Load libpgsvt.so and declare its signatures (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("libpgsvt.so not built at %s: run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    vp, u32, i32, i64, dbl = (ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32,
                              ctypes.c_int64, ctypes.c_double)
    P = ctypes.POINTER
    L.pgsvt_default_params.argtypes = [P(Params)]
    L.pgsvt_denoise.argtypes = [vp, i32, u32, u32, u32, vp, vp, P(Params), P(Status)]
    L.pgsvt_denoise_device.argtypes = [vp, i32, u32, u32, u32, vp, vp, P(Params), vp, P(Status)]
    L.pgsvt_arps_window.argtypes = [vp, u32, u32, u32, u32, u32, u32, u32, i32, u32, vp, vp]
    L.pgsvt_svd_window.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp, P(u32)]
    L.pgsvt_reconstruct_window.argtypes = [vp, u32, u32, u32, u32, i32, vp, vp, dbl, vp]
    L.pgsvt_risk_window.argtypes = [vp, u32, u32, u32, u32, i32, vp, vp, dbl, dbl, dbl, i64,
                                    u32, vp, u32, vp]
    L.pgsvt_svd_window_noalloc.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp, P(u32), vp]
    L.pgsvt_last_error.restype = ctypes.c_char_p
    L.pgsvt_version.restype = ctypes.c_char_p
    for name in EXPORTS:
        L[name]  # every declared symbol must resolve
    _lib = L
    return L


def _check(rc):
    if rc != OK:
        raise PgsvtError(rc, load().pgsvt_last_error().decode())


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def version():
    return load().pgsvt_version().decode()


def default_params(**kw):
    p = Params()
    load().pgsvt_default_params(ctypes.byref(p))
    for k, v in kw.items():
        k = "lambda_" if k == "lambda" else k
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def denoise(X, params):
    """pgsvt_denoise on a (rows, cols, frames) array.  Returns (Y, est, status)."""
    X = np.asfortranarray(X)
    if X.dtype not in DTYPES:
        raise TypeError("Invalid dtype: got %s" % X.dtype)
    nr, nc, nt = X.shape
    Y = np.zeros((nr, nc, nt), np.float64, order="F")
    est = np.zeros((nt, 4), np.float64, order="F")
    st = Status()
    rc = load().pgsvt_denoise(_ptr(X), DTYPES[X.dtype], nr, nc, nt, _ptr(Y), _ptr(est),
                              ctypes.byref(params), ctypes.byref(st))
    if rc != OK:
        raise PgsvtError(rc, st.message.decode())
    return Y, est, st


def denoise_device(x_ptr, dtype_code, nr, nc, nt, y_ptr, est_ptr, params, stream=0):
    """pgsvt_denoise_device on raw device pointers (e.g. torch tensors)."""
    st = Status()
    rc = load().pgsvt_denoise_device(ctypes.c_void_p(x_ptr), dtype_code, nr, nc, nt,
                                     ctypes.c_void_p(y_ptr), ctypes.c_void_p(est_ptr),
                                     ctypes.byref(params), ctypes.c_void_p(stream),
                                     ctypes.byref(st))
    if rc != OK:
        raise PgsvtError(rc, st.message.decode())
    return st


def _window(u):
    u = np.asfortranarray(np.asarray(u, dtype=np.float64))
    return u, u.shape[0], u.shape[2]


def arps_window(w, bs, mw, time_iter, frame_window, nimages, motion=True, compat=COMPAT_ALL):
    """Trajectory table (rows, cols), each (nwin, P) int32 (arps.hpp:52-134)."""
    w, side, nwin = _window(w)
    P = (side - bs + 1) ** 2
    rows = np.zeros((nwin, P), np.int32)
    cols = np.zeros((nwin, P), np.int32)
    _check(load().pgsvt_arps_window(_ptr(w), side, nwin, bs, mw, time_iter, frame_window,
                                    nimages, int(motion), compat, _ptr(rows), _ptr(cols)))
    return rows, cols


def svd_window(u, bs, ov, rows, cols):
    """Singular values (npatch, nwin), descending per patch (svt.hpp:58-118)."""
    u, side, nwin = _window(u)
    rows = np.ascontiguousarray(rows, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    n = ctypes.c_uint32()
    _check(load().pgsvt_svd_window(_ptr(u), side, nwin, bs, ov, _ptr(rows), _ptr(cols), None,
                                   ctypes.byref(n)))
    S = np.zeros((n.value, nwin), np.float32)
    _check(load().pgsvt_svd_window(_ptr(u), side, nwin, bs, ov, _ptr(rows), _ptr(cols), _ptr(S),
                                   ctypes.byref(n)))
    return S


def reconstruct_window(u, bs, ov, rows, cols, lam, expw=True):
    """SVT reconstruction of one window at lambda (svt.hpp:121-167)."""
    u, side, nwin = _window(u)
    rows = np.ascontiguousarray(rows, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    v = np.zeros((side, side, nwin), np.float64, order="F")
    _check(load().pgsvt_reconstruct_window(_ptr(u), side, nwin, bs, ov, int(expw), _ptr(rows),
                                           _ptr(cols), float(lam), _ptr(v)))
    return v


def risk_window(u, bs, ov, rows, cols, lambdas, alpha, mu, sigma, seed, compat=COMPAT_ALL,
                expw=True):
    """PGURE risk of one window at each lambda (pgure.hpp:26-137)."""
    u, side, nwin = _window(u)
    rows = np.ascontiguousarray(rows, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    lam = np.ascontiguousarray(np.atleast_1d(lambdas), np.float64)
    out = np.zeros(len(lam), np.float64)
    _check(load().pgsvt_risk_window(_ptr(u), side, nwin, bs, ov, int(expw), _ptr(rows),
                                    _ptr(cols), alpha, mu, sigma, seed, compat, _ptr(lam),
                                    len(lam), _ptr(out)))
    return out
