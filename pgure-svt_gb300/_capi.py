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
           "pgsvt_denoise_ex", "pgsvt_denoise_device_ex", "pgsvt_lambda_predict",
           "pgsvt_lambda_grad", "pgsvt_lambda_train", "pgsvt_denoise_batch",
           "pgsvt_median_filter", "pgsvt_hot_pixel_filter",
           "pgsvt_arps_window", "pgsvt_svd_window", "pgsvt_svd_window_ex",
           "pgsvt_reconstruct_window",
           "pgsvt_risk_window", "pgsvt_svd_window_noalloc", "pgsvt_last_error",
           "pgsvt_version")
LAMBDA_FEATURES = 67
LAMBDA_HIDDEN = 128
LAMBDA_SAMPLES = 4096
LAMBDA_MODEL_FLOATS = 41993
LAMBDA_PARAM_OFFSET = 134
LAMBDA_PARAMS = 41857
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
        ("frame_end", ctypes.c_uint32), ("lambda_model", ctypes.c_void_p),
        ("hint_points", ctypes.c_uint32), ("hint_rounds", ctypes.c_uint32),
        ("hint_flat", ctypes.c_double), ("autotune", ctypes.c_uint32),
    ]


class Outputs(ctypes.Structure):
    """pgsvt_outputs: optional per-frame outputs of the _ex entry points."""
    _fields_ = [("lambda_features", ctypes.c_void_p), ("lambda_proposals", ctypes.c_void_p),
                ("risk", ctypes.c_void_p), ("risk_evals", ctypes.c_void_p)]


class TrainParams(ctypes.Structure):
    """pgsvt_train_params."""
    _fields_ = [("epochs", ctypes.c_uint32), ("batch", ctypes.c_uint32),
                ("lr", ctypes.c_float), ("lr_final", ctypes.c_float),
                ("weight_decay", ctypes.c_float), ("beta1", ctypes.c_float),
                ("beta2", ctypes.c_float), ("eps", ctypes.c_float), ("seed", ctypes.c_uint64)]


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
        ("message", ctypes.c_char * 256), ("svd_variant", ctypes.c_int32),
        ("svd_tuned", ctypes.c_int32),
    ]


class Sequence(ctypes.Structure):
    """pgsvt_sequence: one sequence of pgsvt_denoise_batch."""
    _fields_ = [("X", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("nrows", ctypes.c_uint32),
                ("ncols", ctypes.c_uint32), ("nframes", ctypes.c_uint32), ("Y", ctypes.c_void_p),
                ("estimates", ctypes.c_void_p), ("params", ctypes.c_void_p),
                ("lambdas", ctypes.c_void_p), ("nlambdas", ctypes.c_uint32),
                ("risks", ctypes.c_void_p), ("status", ctypes.c_void_p)]


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
    L.pgsvt_denoise_ex.argtypes = [vp, i32, u32, u32, u32, vp, vp, P(Params), P(Outputs), P(Status)]
    L.pgsvt_denoise_device_ex.argtypes = [vp, i32, u32, u32, u32, vp, vp, P(Params), P(Outputs),
                                          vp, P(Status)]
    L.pgsvt_lambda_predict.argtypes = [vp, vp, u32, vp]
    L.pgsvt_denoise_batch.argtypes = [vp, u32, u32, P(Status)]
    L.pgsvt_median_filter.argtypes = [vp, vp, u32, u32, u32, u32]
    L.pgsvt_hot_pixel_filter.argtypes = [vp, u32, u32, u32, dbl]
    L.pgsvt_lambda_grad.argtypes = [vp, vp, vp, u32, vp, P(dbl)]
    L.pgsvt_lambda_train.argtypes = [vp, vp, vp, u32, P(TrainParams), vp, P(Status)]
    L.pgsvt_arps_window.argtypes = [vp, u32, u32, u32, u32, u32, u32, u32, i32, u32, vp, vp]
    L.pgsvt_svd_window.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp, P(u32)]
    L.pgsvt_svd_window_ex.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp, P(u32), P(Status)]
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


def denoise_ex(X, params, features=False, proposals=False):
    """pgsvt_denoise_ex: (Y, est, status, extras) where extras holds per-frame
    `risk` and `evals`, plus `features` (frames x 67) and `proposals` when
    asked for."""
    X = np.asfortranarray(X)
    if X.dtype not in DTYPES:
        raise TypeError("Invalid dtype: got %s" % X.dtype)
    nr, nc, nt = X.shape
    Y = np.zeros((nr, nc, nt), np.float64, order="F")
    est = np.zeros((nt, 4), np.float64, order="F")
    ex = {"risk": np.zeros(nt, np.float64), "evals": np.zeros(nt, np.uint32)}
    out = Outputs(risk=ex["risk"].ctypes.data, risk_evals=ex["evals"].ctypes.data)
    if features:
        ex["features"] = np.zeros((nt, LAMBDA_FEATURES), np.float32)
        out.lambda_features = ex["features"].ctypes.data
    if proposals:
        ex["proposals"] = np.zeros(nt, np.float32)
        out.lambda_proposals = ex["proposals"].ctypes.data
    st = Status()
    rc = load().pgsvt_denoise_ex(_ptr(X), DTYPES[X.dtype], nr, nc, nt, _ptr(Y), _ptr(est),
                                 ctypes.byref(params), ctypes.byref(out), ctypes.byref(st))
    if rc != OK:
        raise PgsvtError(rc, st.message.decode())
    return Y, est, st, ex


def denoise_batch(sequences, slots=2):
    """pgsvt_denoise_batch.  `sequences`: dicts with X (rows, cols, frames),
    params (Params) and optionally lambdas (<= 16 values).  Returns
    (results, total status); each result is a dict with Y, est, status and,
    with a lambda list, risks (frames x len(lambdas))."""
    keep, res = [], []
    arr = (Sequence * max(1, len(sequences)))()
    for i, q in enumerate(sequences):
        X = np.asfortranarray(q["X"])
        if X.dtype not in DTYPES:
            raise TypeError("Invalid dtype: got %s" % X.dtype)
        nr, nc, nt = X.shape
        r = dict(Y=np.zeros((nr, nc, nt), np.float64, order="F"),
                 est=np.zeros((nt, 4), np.float64, order="F"), status=Status())
        s = arr[i]
        s.X, s.dtype, s.nrows, s.ncols, s.nframes = X.ctypes.data, DTYPES[X.dtype], nr, nc, nt
        s.Y, s.estimates = r["Y"].ctypes.data, r["est"].ctypes.data
        s.params = ctypes.addressof(q["params"])
        s.status = ctypes.addressof(r["status"])
        lam = q.get("lambdas")
        if lam is not None:
            lam = np.ascontiguousarray(lam, np.float64)
            r["risks"] = np.zeros((nt, lam.size), np.float64)
            s.lambdas, s.nlambdas, s.risks = lam.ctypes.data, lam.size, r["risks"].ctypes.data
        keep += [X, lam, q["params"]]
        res.append(r)
    st = Status()
    rc = load().pgsvt_denoise_batch(arr, len(sequences), slots, ctypes.byref(st))
    if rc != OK:
        raise PgsvtError(rc, st.message.decode())
    return res, st


def median_filter(frames, r):
    """pgsvt_median_filter on uint16 frames (rows, cols[, frames])."""
    a = np.asfortranarray(frames, dtype=np.uint16)
    shp = a.shape
    if a.ndim == 2:
        a = a.reshape(shp[0], shp[1], 1, order="F")
    out = np.zeros_like(a, order="F")
    _check(load().pgsvt_median_filter(_ptr(a), _ptr(out), a.shape[0], a.shape[1], a.shape[2], r))
    return out.reshape(shp, order="F")


def hot_pixel_filter(frames, threshold):
    """pgsvt_hot_pixel_filter on uint16 frames (rows, cols[, frames]); returns a copy."""
    a = np.array(frames, dtype=np.uint16, order="F", copy=True)
    shp = a.shape
    if a.ndim == 2:
        a = a.reshape(shp[0], shp[1], 1, order="F")
    _check(load().pgsvt_hot_pixel_filter(_ptr(a), a.shape[0], a.shape[1], a.shape[2],
                                         float(threshold)))
    return a.reshape(shp, order="F")


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError("expected shape %s, got %s" % (shape, a.shape))
    return a


def lambda_predict(model, features):
    """pgsvt_lambda_predict: network outputs log10(lambda/upper) per feature row."""
    model = _f32(model, (LAMBDA_MODEL_FLOATS,))
    f = _f32(features)
    n = f.shape[0]
    y = np.zeros(n, np.float32)
    _check(load().pgsvt_lambda_predict(_ptr(model), _ptr(f), n, _ptr(y)))
    return y


def lambda_grad(model, features, targets):
    """pgsvt_lambda_grad: (loss, gradient over the trainable parameters)."""
    model = _f32(model, (LAMBDA_MODEL_FLOATS,))
    f = _f32(features)
    t = _f32(targets, (f.shape[0],))
    g = np.zeros(LAMBDA_PARAMS, np.float32)
    loss = ctypes.c_double()
    _check(load().pgsvt_lambda_grad(_ptr(model), _ptr(f), _ptr(t), f.shape[0], _ptr(g),
                                    ctypes.byref(loss)))
    return loss.value, g


def lambda_train(model, features, targets, epochs, batch=256, lr=2e-3, lr_final=2e-5,
                 weight_decay=1e-4, beta1=0.9, beta2=0.999, eps=1e-8, seed=0):
    """pgsvt_lambda_train: (trained model, per-epoch mean loss, status)."""
    m = _f32(model, (LAMBDA_MODEL_FLOATS,)).copy()
    f = _f32(features)
    t = _f32(targets, (f.shape[0],))
    tp = TrainParams(epochs=epochs, batch=batch, lr=lr, lr_final=lr_final,
                     weight_decay=weight_decay, beta1=beta1, beta2=beta2, eps=eps, seed=seed)
    curve = np.zeros(epochs, np.float32)
    st = Status()
    rc = load().pgsvt_lambda_train(_ptr(m), _ptr(f), _ptr(t), f.shape[0], ctypes.byref(tp),
                                   _ptr(curve), ctypes.byref(st))
    if rc != OK:
        raise PgsvtError(rc, st.message.decode())
    return m, curve, st


def denoise_device_ex(x_ptr, dtype_code, nr, nc, nt, y_ptr, est_ptr, params, outputs=None,
                      stream=0):
    """pgsvt_denoise_device_ex: `outputs` is an Outputs struct of device
    pointers (or None)."""
    st = Status()
    rc = load().pgsvt_denoise_device_ex(ctypes.c_void_p(x_ptr), dtype_code, nr, nc, nt,
                                        ctypes.c_void_p(y_ptr), ctypes.c_void_p(est_ptr),
                                        ctypes.byref(params),
                                        ctypes.byref(outputs) if outputs is not None else None,
                                        ctypes.c_void_p(stream), ctypes.byref(st))
    if rc != OK:
        raise PgsvtError(rc, st.message.decode())
    return st


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


def svd_window(u, bs, ov, rows, cols, status=False):
    """Singular values (npatch, nwin), descending per patch (svt.hpp:58-118);
    with status=True also the call's Status (SVD sweep and FP64 counters)."""
    u, side, nwin = _window(u)
    rows = np.ascontiguousarray(rows, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    n = ctypes.c_uint32()
    _check(load().pgsvt_svd_window(_ptr(u), side, nwin, bs, ov, _ptr(rows), _ptr(cols), None,
                                   ctypes.byref(n)))
    S = np.zeros((n.value, nwin), np.float32)
    st = Status()
    _check(load().pgsvt_svd_window_ex(_ptr(u), side, nwin, bs, ov, _ptr(rows), _ptr(cols),
                                      _ptr(S), ctypes.byref(n), ctypes.byref(st)))
    return (S, st) if status else S


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
