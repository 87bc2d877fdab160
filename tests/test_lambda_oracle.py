"""CPU checks of the learned-lambda oracle (oracle/lambda_mlp.py) and the
shipped model.  The GPU kernels are compared with this oracle in
tests/test_gpu_lambda.py."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import lambda_mlp as lm  # noqa: E402


def _model(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    m = rng.normal(0.0, 0.1 * scale, lm.TOTAL).astype(np.float32)
    m[lm.OFF_MEAN:lm.OFF_SCALE] = rng.normal(0, 0.1, lm.NF)
    m[lm.OFF_SCALE:lm.OFF_W1] = rng.uniform(0.5, 2.0, lm.NF)
    m[lm.OFF_YMEAN] = -2.0
    m[lm.OFF_YSCALE] = 1.5
    return m


def test_layout():
    assert lm.TOTAL == 41993 and lm.NPARAM == 41857 and lm.OFF_W1 == 134


def test_bf16_round_to_nearest_even():
    # 1 + 2^-8 is halfway between bf16 neighbours 1 and 1 + 2^-7: ties to even (1)
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.0e-3], np.float32)
    r = lm.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2.0 ** -6
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2.0 ** -8


def test_sample_indices_stratified():
    for npatch in (841, 4096, 8649, 259081):
        idx = lm.sample_indices(npatch)
        ns = min(npatch, 4096)
        assert idx.shape == (ns,)
        assert idx.min() >= 0 and idx.max() < npatch
        # one per stratum [i NP/ns, (i+1) NP/ns): non-decreasing, neighbours
        # can share a patch only where a stratum boundary is fractional
        assert np.all(np.diff(idx) >= 0)
        assert np.all(idx >= np.floor(np.arange(ns) * npatch / ns))
        if npatch <= 4096:
            assert np.array_equal(idx, np.arange(npatch))


def test_features_histogram():
    rng = np.random.default_rng(1)
    S = np.sort(rng.lognormal(-1.0, 1.5, (5000, 15)), axis=1)[:, ::-1]
    S[0, -1] = 0.0  # a zero singular value falls in bin 0
    f = lm.features(S, 0.5, 3.0, 1.0)
    assert f.shape == (67,)
    assert abs(f[3:].sum() - 1.0) < 1e-12
    assert np.allclose(f[:3], np.arcsinh(np.array([0.5, 3.0, 1.0]) * 1000) / 8)
    # bin edges: 10^-4 * 10^(6 b / 64)
    s = np.array([[10 ** (-4 + 6 * 10.5 / 64)]])
    assert np.argmax(lm.features(s, 0, 0, 0)[3:]) == 10


def test_gradient_matches_finite_differences():
    m = _model(2).astype(np.float64)
    rng = np.random.default_rng(3)
    feats = rng.normal(0, 1, (6, lm.NF))
    targets = rng.normal(-2, 1, 6)
    _, g = lm.loss_and_grad(m, feats, targets, exact=True)
    idx = np.concatenate([rng.choice(lm.NPARAM, 60, replace=False),
                          [lm.OFF_B4 - lm.OFF_W1, lm.OFF_W4 - lm.OFF_W1, 0,
                           lm.OFF_B1 - lm.OFF_W1]])
    h = 1e-6
    for i in idx:
        mp, mm = m.copy(), m.copy()
        mp[lm.OFF_W1 + i] += h
        mm[lm.OFF_W1 + i] -= h
        fd = (lm.loss_and_grad(mp, feats, targets, exact=True)[0] -
              lm.loss_and_grad(mm, feats, targets, exact=True)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, np.abs(g).max()), (i, fd, g[i])


def test_adamw_first_step_is_signed_lr():
    m = _model(4)
    g = np.random.default_rng(5).normal(0, 1e-2, lm.NPARAM)
    new, m1, m2 = lm.adamw_step(m, np.zeros(lm.NPARAM), np.zeros(lm.NPARAM), g, 1, 1e-3, 0.0)
    step = new[lm.OFF_W1:lm.OFF_YMEAN] - np.asarray(m, np.float64)[lm.OFF_W1:lm.OFF_YMEAN]
    # m1 / (1 - b1) = g and sqrt(m2 / (1 - b2)) = |g| on the first step
    assert np.allclose(step, -1e-3 * g / (np.abs(g) + 1e-8), rtol=1e-6, atol=1e-12)
    assert np.array_equal(new[:lm.OFF_W1], np.asarray(m, np.float64)[:lm.OFF_W1])


def test_shipped_model(pkg):
    m = pkg.learned.load_model()
    assert m.dtype == np.float32 and m.shape == (lm.TOTAL,)
    assert np.all(np.isfinite(m))
    assert m[lm.OFF_YSCALE] > 0
    # its outputs on the training features' mean lie in the label range
    y = lm.predict(m, m[lm.OFF_MEAN:lm.OFF_SCALE][None, :])
    assert -6.5 <= y[0] <= 0.5
    with np.load(pkg.learned.MODEL_PATH) as z:
        assert int(z["n_train"]) >= 4000
