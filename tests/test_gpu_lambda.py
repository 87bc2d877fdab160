"""Learned lambda proposal on the GPU against its FP64 oracle
(oracle/lambda_mlp.py) and against the plain search.

Tolerances: the network runs with the same bf16 weights on both sides; the
GPU sums in FP32, the oracle in FP64, so outputs agree to ~1e-5 and
gradients to ~1e-4 of their largest component.  Feature histograms come
from FP32 (GPU) and FP64 (oracle) singular values, so a value lying on a bin
edge may fall on either side: the L1 distance of the histograms is bounded
by a few values' worth.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import lambda_mlp as lm  # noqa: E402


def _model(pkg, n=256, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.normal(0.0, 1.0, (n, lm.NF)).astype(np.float32)
    f[:, 3:] = np.abs(f[:, 3:]) * 0.05
    t = (np.tanh(f[:, 0] - 0.5 * f[:, 1]) + 0.3 * f[:, 5] * 10 - 2.0).astype(np.float32)
    m = pkg.learned.init_model(f, t, seed=seed)
    # non-zero biases and a larger output row exercise every term
    m[lm.OFF_B1:lm.OFF_W2] = rng.normal(0, 0.1, lm.H)
    m[lm.OFF_B3:lm.OFF_W4] = rng.normal(0, 0.1, lm.H)
    m[lm.OFF_W4:lm.OFF_B4] = rng.normal(0, 0.1, lm.H)
    m[lm.OFF_B4] = 0.3
    return m, f, t


def test_predict_matches_oracle(capi, pkg):
    m, f, _ = _model(pkg, 100)
    y = capi.lambda_predict(m, f)
    y0 = lm.predict(m, f)
    assert np.abs(y - y0).max() <= 1e-4 * (1 + np.abs(y0).max())


def test_gradient_matches_oracle(capi, pkg):
    m, f, t = _model(pkg, 100, seed=1)  # 4 blocks, the last one partial
    loss, g = capi.lambda_grad(m, f, t)
    loss0, g0 = lm.loss_and_grad(m, f, t)
    assert abs(loss - loss0) <= 1e-5 * loss0
    err = np.abs(g - g0).max() / np.abs(g0).max()
    print("max gradient error relative to max |g|: %.2e" % err)
    assert err < 1e-4
    # every layer's block is non-trivial and matched
    for a, b in lm.WEIGHT_RANGES:
        sl = slice(a - lm.OFF_W1, b - lm.OFF_W1)
        assert np.abs(g0[sl]).max() > 0
        assert np.abs(g[sl] - g0[sl]).max() <= 1e-4 * np.abs(g0).max()


def test_one_training_step_is_adamw(capi, pkg):
    m, f, t = _model(pkg, 64, seed=2)
    lr, wd = 1e-3, 1e-2
    m1, curve, _ = capi.lambda_train(m, f, t, epochs=1, batch=64, lr=lr, lr_final=lr,
                                     weight_decay=wd)
    L0, g0 = lm.loss_and_grad(m, f, t)
    assert abs(curve[0] - L0) <= 1e-5 * L0
    ref, _, _ = lm.adamw_step(m, np.zeros(lm.NPARAM), np.zeros(lm.NPARAM), g0, 1, lr, wd)
    # first step = -lr * g/|g|: compare where the sign of g is well defined
    sel = np.abs(g0) > 1e-3 * np.abs(g0).max()
    P = slice(lm.OFF_W1, lm.OFF_YMEAN)
    assert np.abs(m1[P][sel] - ref[P][sel]).max() < 1e-6
    assert np.array_equal(m1[:lm.OFF_W1], m[:lm.OFF_W1])  # normalisation kept
    assert np.array_equal(m1[lm.OFF_YMEAN:], m[lm.OFF_YMEAN:])


def test_training_converges_and_is_deterministic(capi, pkg):
    m, f, t = _model(pkg, 1024, seed=3)
    ma, ca, _ = capi.lambda_train(m, f, t, epochs=150, batch=128, lr=3e-3, lr_final=3e-5, seed=5)
    mb, cb, _ = capi.lambda_train(m, f, t, epochs=150, batch=128, lr=3e-3, lr_final=3e-5, seed=5)
    assert np.array_equal(ma, mb) and np.array_equal(ca, cb)
    print("loss first %.4f last %.5f" % (ca[0], ca[-1]))
    assert ca[-1] < 0.1 * ca[0]
    L, _ = lm.loss_and_grad(ma, f, t)  # the oracle agrees with the trained fit
    assert L < 0.1 * ca[0]


def _risk_params(g):
    # PGSVT_COMPAT_SWAP_MU_SIGMA: the risk's mu is the caller's sigma and vice versa
    return float(g["alpha"]), float(g["sigma"]), float(g["mu"])


def test_features_match_oracle(capi, pkg):
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    p = capi.default_params(median_size=0, random_seed=11, alpha=float(g["alpha"]),
                            mu=float(g["mu"]), sigma=float(g["sigma"]), frame_begin=8,
                            frame_end=9)
    _, _, _, ex = capi.denoise_ex(g["X"].astype(np.float64), p, features=True)
    f = ex["features"][8]
    f0 = lm.features(g["S_8"], *_risk_params(g))  # 841 patches: all of them
    assert np.allclose(f[:3], f0[:3], rtol=1e-6)
    l1 = np.abs(f[3:] - f0[3:]).sum()
    print("histogram L1 distance", l1)
    assert l1 <= 4.0 / (841 * 15)
    assert abs(f[3:].sum() - 1) < 1e-5


def test_features_sampled_patches_match_oracle(capi, pkg, oracle):
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=4, side=96, nt=16)
    X = noisy.astype(np.float64)
    p = capi.default_params(median_size=0, random_seed=3, alpha=a, mu=m, sigma=s,
                            frame_begin=8, frame_end=9)
    _, _, _, ex = capi.denoise_ex(X, p, features=True)
    u = X[:, :, 1:16] / X[:, :, 1:16].max()
    rows, cols = oracle.arps_window(u, 4, 7, 8, 7, 16)
    S = oracle.svd_window(u, 4, 1, rows, cols)
    assert S.shape[0] == 93 * 93 > 4096
    f0 = lm.features(S, a, s, m)
    l1 = np.abs(ex["features"][8][3:] - f0[3:]).sum()
    print("histogram L1 distance", l1)
    assert l1 <= 8.0 / (4096 * 15)


def test_learned_search_matches_oracle(capi, pkg, oracle):
    """The GPU's narrow search from its own proposals against the oracle's
    narrow search from the same proposals."""
    g = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    model = pkg.learned.load_model()
    a, m, s = float(g["alpha"]), float(g["mu"]), float(g["sigma"])
    p = pkg.learned.search_params((a, m, s), model=model, random_seed=11)
    Y, est, st, ex = capi.denoise_ex(g["X"], p, proposals=True)
    prop = ex["proposals"].astype(np.float64)
    assert np.all(np.isfinite(prop))
    hints = 100.0 * 10.0 ** np.clip(prop, -6, 0)
    Y0, est0, rep = oracle.denoise(g["X"].astype(np.float64), lambda_hints=hints, median_size=-1,
                                   random_seed=11, alpha=a, mu=m, sigma=s, n_jobs=4)
    X = g["X"].astype(np.float64)
    gaps = []
    for t in (0, 4, 8, 12, 15):
        u = _window(X, t)
        rows, cols = oracle.arps_window(u, 4, 7, t, 7, 16)
        r = oracle.risk_window(u, 4, 1, rows, cols, [est[t, 0], est0[t, 0]], a, m, s, 11)
        gaps.append((r[0] - r[1]) / abs(r[1]))
    print("evals gpu", ex["evals"], "oracle", rep.evals, "gaps", gaps)
    assert max(gaps) < 0.01
    assert np.mean(ex["evals"] == rep.evals) >= 0.75


def _window(X, t, fw=7):
    nt = X.shape[2]
    s0 = 0 if t < fw else (nt - 2 * fw - 1 if t >= nt - fw else t - fw)
    u = X[:, :, s0:s0 + 2 * fw + 1]
    return u / u.max()


def test_learned_proposal_gains_over_plain_search(pkg):
    """Held-out sequences of the training distribution: the narrow search
    from the shipped model needs fewer risk evaluations than the plain
    search, at a risk gap of at most 1% per window."""
    L = pkg.learned
    model = L.load_model()
    ev_plain = ev_learned = 0
    gaps = []
    for i in range(4):
        noisy, noise = L.random_sequence(10 ** 7 + i)
        res = L.compare(noisy, noise, model, frames=L.LABEL_FRAMES)
        f0, f1 = L.LABEL_FRAMES
        rp, rl = res["plain"]["risk"][f0:f1], res["learned"]["risk"][f0:f1]
        gaps += list((rl - rp) / np.abs(rp))
        ev_plain += int(res["plain"]["evals"][f0:f1].sum())
        ev_learned += int(res["learned"]["evals"][f0:f1].sum())
    print("risk evaluations plain %d learned %d, max risk gap %.2e" % (ev_plain, ev_learned,
                                                                      max(gaps)))
    assert ev_learned < 0.8 * ev_plain
    assert max(gaps) <= 0.01


def test_learned_proposal_gains_on_default_path(pkg):
    """Held-out sequences of the reference's default path (median
    pre-filter 5, noise parameters estimated per window): the shipped model
    also proposes there; fewer risk evaluations than the plain search (about
    0.6 of them: the plain search refines with K/2 points per round), at a
    risk gap of at most 1% for nearly every window."""
    L = pkg.learned
    model = L.load_model()
    ev_plain = ev_learned = 0
    gaps = []
    for i in range(4):
        noisy, noise = L.random_sequence(10 ** 7 + 100 + i, estimated=True)
        assert noise is None
        res = L.compare(noisy, noise, model, frames=L.LABEL_FRAMES)
        f0, f1 = L.LABEL_FRAMES
        rp, rl = res["plain"]["risk"][f0:f1], res["learned"]["risk"][f0:f1]
        gaps += list((rl - rp) / np.abs(rp))
        ev_plain += int(res["plain"]["evals"][f0:f1].sum())
        ev_learned += int(res["learned"]["evals"][f0:f1].sum())
    gaps = np.array(gaps)
    print("risk evaluations plain %d learned %d, risk gaps %s" % (ev_plain, ev_learned, gaps))
    assert ev_learned < 0.7 * ev_plain
    assert np.mean(gaps <= 0.01) >= 0.9 and gaps.max() <= 0.02
