"""Learned lambda proposal: training data, training and the shipped model.

Not part of the reference.  The plain PGURE search (the reference's lambda
optimisation, pgure.hpp:197-237) labels windows of seeded synthetic
sequences with their risk-optimal lambda; the library's own GPU kernels
(pgsvt_lambda_train: bf16 weights, FP32 accumulation, AdamW) fit the MLP of
include/pgsvt.h to those labels; at run time the network's proposal starts a
narrow search (hint_points values over [lambda/span, lambda*span], then
hint_rounds refinements), and the plain search remains the fallback.

Labels are y = log10(lambda*/upper) with upper = max(100, mean(u)) = 100 for
max-normalised windows (pguresvt.hpp:139-141), clipped to [-6, 0].
"""
import os

import numpy as np

from . import _capi, synth

HERE = os.path.dirname(os.path.abspath(__file__))
MODEL_PATH = os.path.join(HERE, "lambda_mlp.npz")
SIDES = (128, 192, 256, 320, 384, 448, 512)
POW2_SIDES = (128, 256, 512)
UPPER = 100.0
SEQ_FRAMES = 18          # frames 7..10 are full windows of a T=15 trajectory
LABEL_FRAMES = (7, 11)


def random_sequence(seed, estimated=False):
    """A seeded sequence of the training distribution: 128^2-512^2, blob or
    blob+lattice scenes, integer or sub-pixel drift, alpha in [0.05, 1],
    mu in [0, 2], sigma in [0.5, 5] (raw counts).  Returns (noisy float32,
    (alpha, mu, sigma)), or (noisy, None) with `estimated`: a power-of-two
    side (the noise estimator's F-test table has no other sizes) for the
    reference's default path, which estimates the noise parameters."""
    rng = np.random.default_rng(seed)
    side = int(rng.choice(POW2_SIDES if estimated else SIDES))
    nblobs = max(1, int(round(300 * (side / 512.0) ** 2 * rng.uniform(0.3, 1.5))))
    lattice = bool(rng.random() < 0.5)
    integer = bool(rng.random() < 0.3)
    max_step = 1 if integer else float(rng.uniform(0.0, 2.0))
    alpha = float(rng.uniform(0.05, 1.0))
    mu = float(rng.uniform(0.0, 2.0))
    sigma = float(rng.uniform(0.5, 5.0))
    clean = synth.blobs(side, SEQ_FRAMES, nblobs, int(rng.integers(1 << 31)), max_step, integer,
                        lattice)
    noisy = synth.poisson_gaussian(clean, alpha, mu, sigma, int(rng.integers(1 << 31)))
    return np.asfortranarray(noisy.astype(np.float32)), (None if estimated else (alpha, mu, sigma))


HELDOUT_SIDE = 512
HELDOUT_FRAMES = 200
HELDOUT_OUTPUTS = (7, 66, 133, 192)  # output frames whose full windows are evaluated


def heldout_windows(seed, estimated=False):
    """The sampled windows of one held-out 512x512x200 sequence: the same
    scene distribution as random_sequence (blob or blob+lattice, integer or
    sub-pixel drift over all 200 frames, alpha in [0.05, 1], mu in [0, 2],
    sigma in [0.5, 5]), rendered only on the 15-frame windows of the output
    frames HELDOUT_OUTPUTS (frame noise seeded per frame).  Returns a list of
    (noisy float32 window, clean window) and the noise parameters (None with
    `estimated`).  Output frame 7 of a window array is the window's centre,
    a middle window exactly as in the whole sequence."""
    rng = np.random.default_rng(seed)
    side, nt = HELDOUT_SIDE, HELDOUT_FRAMES
    nblobs = max(1, int(round(300 * rng.uniform(0.3, 1.5))))
    lattice = bool(rng.random() < 0.5)
    integer = bool(rng.random() < 0.3)
    max_step = 1 if integer else float(rng.uniform(0.0, 2.0))
    alpha = float(rng.uniform(0.05, 1.0))
    mu = float(rng.uniform(0.0, 2.0))
    sigma = float(rng.uniform(0.5, 5.0))
    scene = int(rng.integers(1 << 31))
    noise_seed = int(rng.integers(1 << 31))
    frames = [f for t in HELDOUT_OUTPUTS for f in range(t - 7, t + 8)]
    clean = synth.blobs(side, nt, nblobs, scene, max_step, integer, lattice, frames=frames)
    out = []
    for w, t in enumerate(HELDOUT_OUTPUTS):
        cw = np.asfortranarray(clean[:, :, 15 * w:15 * (w + 1)])
        nw = np.empty_like(cw)
        for k in range(15):
            nw[:, :, k] = synth.poisson_gaussian(cw[:, :, k:k + 1], alpha, mu, sigma,
                                                 noise_seed + t - 7 + k)[:, :, 0]
        out.append((np.asfortranarray(nw.astype(np.float32)), cw))
    return out, (None if estimated else (alpha, mu, sigma))


def search_params(noise, frames=None, model=None, **kw):
    """Parameters of the benchmark's PGURE search (4x4 patches, T=15,
    motion window 7, reference compat mode, probe seed 7) with the given
    noise parameters, or with noise=None the reference's defaults: median
    pre-filter 5 and the noise parameters estimated per window."""
    a, m, s = noise if noise is not None else (-1.0, -1.0, -1.0)
    p = dict(traj_length=15, block_size=4, block_overlap=1, motion_window=7,
             median_size=0 if noise is not None else 5,
             optimize_pgure=1, motion_estimation=1, alpha=a, mu=m, sigma=s, random_seed=7)
    if frames is not None:
        p.update(frame_begin=frames[0], frame_end=frames[1])
    if model is not None:  # the caller keeps `model` alive during the call
        if not (isinstance(model, np.ndarray) and model.dtype == np.float32
                and model.flags.c_contiguous and model.size == _capi.LAMBDA_MODEL_FLOATS):
            raise TypeError("lambda model must be a contiguous float32 array of %d values"
                            % _capi.LAMBDA_MODEL_FLOATS)
        p["lambda_model"] = model.ctypes.data
    p.update(kw)
    return _capi.default_params(**p)


def target(lam):
    return np.clip(np.log10(np.maximum(lam, 1e-300) / UPPER), -6.0, 0.0)


def label(noisy, noise, frames=LABEL_FRAMES):
    """Features and plain-search labels of frames [frames[0], frames[1])
    (noise=None: the reference's default path, noise estimated)."""
    p = search_params(noise, frames)
    _, est, st, ex = _capi.denoise_ex(noisy, p, features=True)
    f0, f1 = frames
    lam = est[f0:f1, 0].copy()
    return dict(features=ex["features"][f0:f1].copy(), targets=target(lam).astype(np.float32),
                lambdas=lam, risks=ex["risk"][f0:f1].copy(), evals=ex["evals"][f0:f1].copy())


def training_set(n_seq, seed=0, pool=None, estimated=False):
    """Labelled windows of n_seq random sequences (4 windows each), with
    given or (estimated=True) estimated noise parameters.  `pool` (a process
    pool started before any GPU call) generates sequences in the background
    while the GPU labels."""
    seeds = [seed * 1000003 + i for i in range(n_seq)]
    fn = _gen_estimated if estimated else random_sequence
    gen = pool.imap(fn, seeds, chunksize=2) if pool else map(fn, seeds)
    parts = [label(noisy, noise) for noisy, noise in gen]
    return {k: np.concatenate([q[k] for q in parts]) for k in parts[0]}


def _gen_estimated(seed):
    return random_sequence(seed, estimated=True)


def init_model(features, targets, seed=0):
    """Initial model: input/output standardisation from the data, weights
    N(0, 2/fan_in) (N(0, 0.01/fan_in) for the output row), zero biases."""
    F, H = _capi.LAMBDA_FEATURES, _capi.LAMBDA_HIDDEN
    rng = np.random.default_rng(seed)
    f = np.asarray(features, np.float64)
    t = np.asarray(targets, np.float64)
    parts = [f.mean(0), 1.0 / np.maximum(f.std(0), 1e-3)]
    for fan_in, fan_out in ((F, H), (H, H), (H, H)):
        parts += [rng.normal(0.0, np.sqrt(2.0 / fan_in), fan_out * fan_in), np.zeros(fan_out)]
    parts += [rng.normal(0.0, np.sqrt(0.01 / H), H), np.zeros(1)]
    parts += [np.array([t.mean()]), np.array([max(t.std(), 1e-3)])]
    m = np.concatenate(parts).astype(np.float32)
    assert m.size == _capi.LAMBDA_MODEL_FLOATS
    return m


def train(features, targets, epochs=600, batch=256, seed=0, **kw):
    """Train on the GPU from a fresh initialisation; returns (model, loss curve)."""
    m0 = init_model(features, targets, seed)
    m, curve, _ = _capi.lambda_train(m0, features, targets, epochs, batch=batch, seed=seed, **kw)
    return m, curve


def save_model(model, path=MODEL_PATH, **meta):
    np.savez_compressed(path, model=np.asarray(model, np.float32),
                        **{k: np.asarray(v) for k, v in meta.items()})


def load_model(path=MODEL_PATH):
    """The shipped model (float32, PGSVT_LAMBDA_MODEL_FLOATS values)."""
    with np.load(path) as z:
        m = z["model"].astype(np.float32)
    if m.shape != (_capi.LAMBDA_MODEL_FLOATS,):
        raise ValueError("lambda model has %d floats, expected %d"
                         % (m.size, _capi.LAMBDA_MODEL_FLOATS))
    return m


def compare(noisy, noise, model, frames=None, **kw):
    """Plain and learned searches on the same windows: per-frame risks,
    lambdas, evaluation counts and both outputs."""
    out = {}
    model = np.ascontiguousarray(model, np.float32)
    for name, mdl in (("plain", None), ("learned", model)):
        p = search_params(noise, frames, mdl, **kw)
        Y, est, st, ex = _capi.denoise_ex(noisy, p, proposals=mdl is not None)
        out[name] = dict(Y=Y, lambdas=est[:, 0].copy(), risk=ex["risk"], evals=ex["evals"],
                         seconds=st.seconds, proposals=ex.get("proposals"))
    return out
