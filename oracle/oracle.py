"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker.  The oracle restates the reference's FP64 path
(src/pguresvt.hpp, src/arps.hpp, src/svt.hpp, src/pgure.hpp); see
pgsvt_oracle.cpp for the line-by-line map.  LAPACK dgesdd comes from scipy's
``cython_lapack`` export table, which exists on every machine with scipy.
"""
import ctypes
import types
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build as _build  # noqa: E402

COMPAT_SWAP_MU_SIGMA = 0x1
COMPAT_ZERO_MOTION = 0x2
COMPAT_INT_DELTA1 = 0x4
COMPAT_ALL = 0x7


class OrcParams(ctypes.Structure):
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
        ("frame_end", ctypes.c_uint32), ("lambda_model", ctypes.c_void_p),
        ("hint_points", ctypes.c_uint32), ("hint_rounds", ctypes.c_uint32),
        ("hint_flat", ctypes.c_double), ("autotune", ctypes.c_uint32),
        ("lambda_hints", ctypes.c_void_p),
        ("risk_out", ctypes.c_void_p), ("evals_out", ctypes.c_void_p),
        ("window_threads", ctypes.c_uint32),
    ]


class OrcReport(ctypes.Structure):
    _fields_ = [("windows", ctypes.c_uint64), ("risk_evals", ctypes.c_uint64),
                ("seconds", ctypes.c_double)]


DEFAULTS = dict(traj_length=15, block_size=4, block_overlap=1, motion_window=7,
                median_size=-1, noise_method=4, max_iter=500, n_jobs=-1, random_seed=-1,
                optimize_pgure=1, exp_weighting=1, motion_estimation=1, verbose=0,
                lambda_=-1.0, alpha=-1.0, mu=-1.0, sigma=-1.0, tol=1e-7,
                compat_flags=COMPAT_ALL, search_points=8, search_rounds=4,
                window_batch=0, lambda_hint=-1.0, hint_span=2.0, frame_begin=0,
                frame_end=0, lambda_model=None, hint_points=4, hint_rounds=2, hint_flat=1e-3,
                autotune=0, lambda_hints=None, risk_out=None, evals_out=None,
                window_threads=1)

_lib = None


def _dgesdd_pointer():
    import scipy.linalg.cython_lapack as cl
    cap = cl.__pyx_capi__["dgesdd"]
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(cap, get_name(cap))


def lib():
    """Load (building if needed) the oracle library and bind LAPACK."""
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.orc_set_dgesdd.argtypes = [ctypes.c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_probes.argtypes = [ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_patch_list.argtypes = [ctypes.c_uint32] * 3 + [ctypes.c_void_p, P(ctypes.c_uint64)]
        L.orc_arps_window.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 7 + [
            ctypes.c_int32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_svd_window.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 4 + [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P(ctypes.c_uint64)]
        L.orc_reconstruct_window.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 4 + [
            ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        L.orc_risk_window.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 4 + [
            ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, ctypes.c_int64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
            ctypes.c_void_p]
        L.orc_noise_estimate.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 4 + [
            P(ctypes.c_double)] * 3
        L.orc_hot_pixel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 3 + [ctypes.c_double]
        L.orc_median_filter.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_uint32] * 3
        L.orc_denoise.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 3 + [
            P(OrcParams), ctypes.c_void_p, ctypes.c_void_p, P(OrcReport)]
        L.orc_set_threads.argtypes = [ctypes.c_uint32]
        L.orc_set_dgesdd(_dgesdd_pointer())
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle error %d: %s" % (rc, lib().orc_last_error().decode()))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_params(**kw):
    d = dict(DEFAULTS)
    for k, v in kw.items():
        k = "lambda_" if k == "lambda" else k
        if k not in d:
            raise KeyError(k)
        d[k] = v
    p = OrcParams()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def set_threads(n):
    """Threads inside one window for the per-stage functions below (arps_window,
    svd_window, reconstruct_window, risk_window); results do not depend on it."""
    lib().orc_set_threads(max(1, int(n)))


def window_geometry(traj_length, block_size):
    """(Nt clamped, frame window, window length) as pguresvt.hpp:57-58."""
    ntc = block_size * block_size - 1 if block_size * block_size < traj_length else traj_length
    fw = ntc // 2
    return ntc, fw, 2 * fw + 1


def probes(seed, n):
    d1 = np.empty(n, np.int8)
    d2 = np.empty(n, np.float64)
    _check(lib().orc_probes(seed, n, _ptr(d1), _ptr(d2)))
    return d1, d2


def patch_list(side, bs, ov):
    cnt = ctypes.c_uint64()
    _check(lib().orc_patch_list(side, bs, ov, None, ctypes.byref(cnt)))
    out = np.empty(cnt.value, np.int64)
    _check(lib().orc_patch_list(side, bs, ov, _ptr(out), ctypes.byref(cnt)))
    return out


def _cube(a):
    """Column-major float64 copy of a (rows, cols, frames) array."""
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def arps_window(w, bs, mw, time_iter, frame_window, nimages, motion=True, compat=COMPAT_ALL):
    w = _cube(w)
    side, nwin = w.shape[0], w.shape[2]
    P = (side - bs + 1) ** 2
    rows = np.zeros((nwin, P), np.int32)
    cols = np.zeros((nwin, P), np.int32)
    _check(lib().orc_arps_window(_ptr(w), side, nwin, bs, mw, time_iter, frame_window, nimages,
                                 int(motion), compat, _ptr(rows), _ptr(cols)))
    return rows, cols


def svd_window(u, bs, ov, rows, cols):
    u = _cube(u)
    side, nwin = u.shape[0], u.shape[2]
    n = ctypes.c_uint64()
    np_ = len(patch_list(side, bs, ov))
    S = np.empty((np_, nwin), np.float64)
    _check(lib().orc_svd_window(_ptr(u), side, nwin, bs, ov, _ptr(np.ascontiguousarray(rows, np.int32)),
                                _ptr(np.ascontiguousarray(cols, np.int32)), _ptr(S), ctypes.byref(n)))
    return S


def reconstruct_window(u, bs, ov, rows, cols, lam, expw=True):
    u = _cube(u)
    side, nwin = u.shape[0], u.shape[2]
    v = np.zeros((side, side, nwin), np.float64, order="F")
    _check(lib().orc_reconstruct_window(_ptr(u), side, nwin, bs, ov, int(expw),
                                        _ptr(np.ascontiguousarray(rows, np.int32)),
                                        _ptr(np.ascontiguousarray(cols, np.int32)), lam, _ptr(v)))
    return v


def risk_window(u, bs, ov, rows, cols, lambdas, alpha, mu, sigma, seed, compat=COMPAT_ALL,
                expw=True):
    u = _cube(u)
    side, nwin = u.shape[0], u.shape[2]
    lam = np.ascontiguousarray(np.atleast_1d(lambdas), dtype=np.float64)
    out = np.empty(len(lam), np.float64)
    _check(lib().orc_risk_window(_ptr(u), side, nwin, bs, ov, int(expw),
                                 _ptr(np.ascontiguousarray(rows, np.int32)),
                                 _ptr(np.ascontiguousarray(cols, np.int32)), alpha, mu, sigma, seed, compat,
                                 _ptr(lam), len(lam), _ptr(out)))
    return out


def noise_estimate(u, method=4, alpha=-1.0, mu=-1.0, sigma=-1.0):
    """NoiseEstimator::Estimate on a normalised window (rows, cols, slices);
    returns (alpha, mu, sigma), given values (>= 0) kept."""
    u = _cube(u)
    a, m, s = ctypes.c_double(alpha), ctypes.c_double(mu), ctypes.c_double(sigma)
    _check(lib().orc_noise_estimate(_ptr(u), u.shape[0], u.shape[1], u.shape[2], method,
                                    ctypes.byref(a), ctypes.byref(m), ctypes.byref(s)))
    return a.value, m.value, s.value


def hot_pixel_filter(frames, threshold):
    """HotPixelFilter on uint16 frames (rows, cols[, frames]); returns a copy."""
    a = np.array(frames, dtype=np.uint16, order="F", copy=True)
    shp = a.shape
    if a.ndim == 2:
        a = a.reshape(shp[0], shp[1], 1, order="F")
    _check(lib().orc_hot_pixel(_ptr(a), a.shape[0], a.shape[1], a.shape[2], float(threshold)))
    return a.reshape(shp, order="F")


def median_filter(frame, r):
    """Median pre-filter of one uint16 frame (rows, cols), column-major as the
    reference's slices."""
    a = np.asfortranarray(frame, dtype=np.uint16)
    out = np.zeros_like(a, order="F")
    _check(lib().orc_median_filter(_ptr(a), _ptr(out), a.shape[0], a.shape[1], r))
    return out


def denoise(X, lambda_hints=None, **kw):
    """Whole-sequence denoise; X is (rows, cols, frames).  Returns (Y, est, report);
    the report also carries per-frame `risk` and `evals`.  `lambda_hints` (one
    value per frame) centres each window's narrow search."""
    X = _cube(X)
    nr, nc, nt = X.shape
    risk = np.zeros(nt, np.float64)
    evals = np.zeros(nt, np.uint32)
    hints = None
    if lambda_hints is not None:
        hints = np.ascontiguousarray(lambda_hints, np.float64)
        assert hints.shape == (nt,)
        kw["lambda_hints"] = hints.ctypes.data
    kw["risk_out"] = risk.ctypes.data
    kw["evals_out"] = evals.ctypes.data
    p = make_params(**kw)
    Y = np.zeros((nr, nc, nt), np.float64, order="F")
    est = np.zeros((nt, 4), np.float64, order="F")
    rep = OrcReport()
    _check(lib().orc_denoise(_ptr(X), nr, nc, nt, ctypes.byref(p), _ptr(Y), _ptr(est),
                             ctypes.byref(rep)))
    out = types.SimpleNamespace(windows=rep.windows, risk_evals=rep.risk_evals,
                                seconds=rep.seconds, risk=risk, evals=evals)
    return Y, est, out
