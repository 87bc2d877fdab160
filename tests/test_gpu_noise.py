"""GPU noise estimation (NoiseEstimator::Estimate, noise.hpp:36-152) and the
reference's default API path (median pre-filter, estimated noise, PGURE)
against the FP64 oracle.

Tolerances: the estimator runs in FP64 on both sides, but the GPU sums in
another order and computes the split tests and leaf variances on the raw
frame (the oracle, like the reference, on the normalised window); the
robust-mean iterations stop on an absolute tolerance of 1e-6, so a sum that
lands on the other side of it changes a leaf mean by up to ~1e-6.  The
estimates are compared at 1e-4 relative.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("method", [1, 2, 3, 4])
def test_estimates_match_frozen_oracle(capi, method):
    """One window per case: a sequence of exactly T frames has one window,
    and its frames are the frozen normalised window (max 1)."""
    z = np.load(os.path.join(GOLDEN, "noise.npz"))
    for k in range(int(z["n"])):
        u = z["u_%d" % k]
        T = u.shape[2]
        p = capi.default_params(median_size=0, traj_length=T, noise_method=method,
                                random_seed=3, search_points=4, search_rounds=1)
        _, est, _ = capi.denoise(u, p)
        ref = z["est_%d" % k][method - 1]
        print(k, est[0, 1:], ref)
        np.testing.assert_allclose(est[:, 1:], np.tile(ref, (T, 1)), rtol=1e-4)


@pytest.mark.parametrize("method", [1, 2, 3, 4])
def test_estimates_of_a_flat_short_window(capi, oracle, method):
    """A flat 5-frame window (one leaf per frame): method 1's leaf count is
    clamped to the leaves on both sides."""
    rng = np.random.default_rng(0)
    u = np.asfortranarray(0.5 + 1e-3 * rng.standard_normal((32, 32, 5)))
    u /= u.max()
    p = capi.default_params(median_size=0, traj_length=5, noise_method=method,
                            random_seed=3, search_points=4, search_rounds=1)
    _, est, _ = capi.denoise(u, p)
    ref = oracle.noise_estimate(u, method=method)
    np.testing.assert_allclose(est[:, 1:], np.tile(ref, (5, 1)), rtol=1e-4)


def test_estimates_match_live_oracle(capi, pkg, oracle):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=21, side=64, nt=18)
    X = noisy.astype(np.float64)
    kw = dict(median_size=5, random_seed=9, frame_begin=6, frame_end=10)
    _, est, _ = capi.denoise(X, capi.default_params(**kw))
    _, est0, _ = oracle.denoise(X, n_jobs=4, **kw)
    f = slice(6, 10)
    print(est[f], est0[f])
    np.testing.assert_allclose(est[f, 1:], est0[f, 1:], rtol=1e-4)


def test_given_values_are_kept(capi, pkg):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=22, side=32, nt=16)
    p = capi.default_params(median_size=0, alpha=0.25, sigma=0.5, random_seed=1)
    _, est, _ = capi.denoise(noisy, p)
    assert np.all(est[:, 1] == 0.25) and np.all(est[:, 3] == 0.5)
    assert np.all(est[:, 2] >= 0) and np.all(np.isfinite(est[:, 2]))


def test_default_api_path_matches_oracle(pkg, oracle):
    """The SVT defaults (median filter 5, noise estimated, PGURE on) on the
    shape of the reference's end-to-end fixture (test_svt.py:61-72: a 32x32x16
    sequence with N(100, 100^2) noise, stored as uint16)."""
    clean = pkg.synth.blobs(32, 16, 6, seed=5) * 40.0
    rng = np.random.RandomState(101)
    Y = clean + 100.0 + 100.0 * rng.randn(*clean.shape)
    Y[Y < 0.0] = 0.0
    Y = Y.astype(np.uint16)
    s = pkg.SVT(random_seed=101)
    s.denoise(Y)
    Yo, est0, _ = oracle.denoise(np.asfortranarray(Y.astype(np.float64)), n_jobs=4,
                                 median_size=5, random_seed=101)
    np.testing.assert_allclose(s.noise_alphas_, est0[:, 1], rtol=1e-4)
    np.testing.assert_allclose(s.noise_mus_, est0[:, 2], rtol=1e-4)
    np.testing.assert_allclose(s.noise_sigmas_, est0[:, 3], rtol=1e-4)
    Yg = np.asarray(s.Y_, np.float64)
    if Yg.shape != Yo.shape:  # the shim returns the reference's (frames, rows, cols)
        Yg = np.transpose(Yg, (1, 2, 0))
    err = np.abs(Yg - Yo).max() / np.abs(Yo).max()
    print("max relative output difference", err, "lambda", s.lambda1s_[:4], est0[:4, 0])
    assert err < 1e-2


def test_estimation_limits(capi, pkg):
    X = np.ones((24, 24, 16), np.float32)  # side 24 > 8 is not a power of two
    with pytest.raises(pkg.PgsvtError) as e:
        capi.denoise(X, capi.default_params(median_size=0))
    assert e.value.code == capi.ERR_UNSUPPORTED
    X = np.ones((32, 32, 16), np.float32)
    with pytest.raises(pkg.PgsvtError) as e:
        capi.denoise(X, capi.default_params(median_size=0, noise_method=5))
    assert e.value.code == capi.ERR_INVALID_ARG
