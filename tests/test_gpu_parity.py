"""GPU parity tests: the CUDA library through its C ABI against the FP64 oracle
(live, on the same inputs) and against the frozen oracle vectors.

Tolerances: ARPS trajectories are integer decisions and must be identical.
The SVD, rebuild and reconstruction run in FP32 against an FP64 oracle, so
they are compared with FP32-level tolerances stated per test; the risk sums
are FP64 on both sides.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLDEN, "oracle_small.npz"))


def _window(X, t, fw):
    nt = X.shape[2]
    s0 = 0 if t < fw else (nt - 2 * fw - 1 if t >= nt - fw else t - fw)
    u = X[:, :, s0:s0 + 2 * fw + 1].astype(np.float64)
    return u / u.max()


def _psnr(ref, x):
    return 10 * np.log10(ref.max() ** 2 / np.mean((ref - x) ** 2))


# ---- ARPS: motion vectors identical to the FP64 reference decisions

def test_arps_matches_frozen_oracle(capi, g):
    X = g["X"]
    for t in (0, 3, 8, 15):
        u = _window(X, t, 7)
        rows, cols = capi.arps_window(u, 4, 7, t, 7, X.shape[2])
        np.testing.assert_array_equal(rows, g["rows_%d" % t])
        np.testing.assert_array_equal(cols, g["cols_%d" % t])


@pytest.mark.parametrize("bs,mw,T", [(4, 7, 15), (4, 3, 15), (8, 7, 15), (6, 5, 9)])
def test_arps_matches_live_oracle(capi, pkg, oracle, bs, mw, T):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=21, side=48, nt=24)
    ntc, fw, nwin = oracle.window_geometry(T, bs)
    for t in (0, fw - 1, fw + 3, 24 - fw, 23):
        u = _window(noisy, t, fw)
        r0, c0 = oracle.arps_window(u, bs, mw, t, fw, 24)
        r1, c1 = capi.arps_window(u, bs, mw, t, fw, 24)
        np.testing.assert_array_equal(r1, r0)
        np.testing.assert_array_equal(c1, c0)


def test_arps_motion_off(capi, oracle, g):
    u = g["u_8"]
    for compat in (capi.COMPAT_ALL, capi.COMPAT_ALL & ~capi.COMPAT_ZERO_MOTION):
        r0, c0 = oracle.arps_window(u, 4, 7, 8, 7, 16, motion=False, compat=compat)
        r1, c1 = capi.arps_window(u, 4, 7, 8, 7, 16, motion=False, compat=compat)
        np.testing.assert_array_equal(r1, r0)
        np.testing.assert_array_equal(c1, c0)


# ---- SVD: FP32 one-sided Jacobi vs FP64 LAPACK

def test_singular_values(capi, g):
    S0 = np.sort(g["S_8"], axis=1)[:, ::-1]
    S1 = capi.svd_window(g["u_8"], 4, 1, g["rows_8"], g["cols_8"]).astype(np.float64)
    smax = S0[:, :1]
    err = np.abs(S1 - S0)
    # absolute error relative to the patch's largest singular value
    assert (err / smax).max() < 2e-5, (err / smax).max()
    rel = err / np.maximum(S0, 1e-30)
    big = S0 > 1e-3 * smax
    print("singular values: max rel err %.3g, mean rel err %.3g (s > 1e-3 smax)"
          % (rel[big].max(), rel[big].mean()))
    assert rel[big].max() < 1e-3 and rel[big].mean() < 1e-5


@pytest.mark.parametrize("bs,T", [(8, 15), (6, 21), (5, 9)])
def test_singular_values_other_shapes(capi, pkg, oracle, bs, T):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=4, side=24, nt=T)
    ntc, fw, nwin = oracle.window_geometry(T, bs)
    u = _window(noisy, fw, fw)
    rows, cols = oracle.arps_window(u, bs, 5, fw, fw, T)
    S0 = oracle.svd_window(u, bs, 1, rows, cols)
    S1 = capi.svd_window(u, bs, 1, rows, cols).astype(np.float64)
    assert (np.abs(S1 - S0) / S0[:, :1]).max() < 3e-5


# ---- reconstruction at fixed lambda

def test_reconstruct_window(capi, g):
    v1 = capi.reconstruct_window(g["u_8"], 4, 1, g["rows_8"], g["cols_8"], 1.0)
    v0 = g["v_8_l1"]
    assert np.abs(v1 - v0).max() < 2e-5
    assert np.abs(v1 - v0).mean() < 1e-6


@pytest.mark.parametrize("lam,expw", [(0.0, True), (1e12, True), (0.02, False), (5.0, True)])
def test_reconstruct_window_extremes(capi, oracle, g, lam, expw):
    u, rows, cols = g["u_8"], g["rows_8"], g["cols_8"]
    v0 = oracle.reconstruct_window(u, 4, 1, rows, cols, lam, expw=expw)
    v1 = capi.reconstruct_window(u, 4, 1, rows, cols, lam, expw=expw)
    assert np.abs(v1 - v0).max() < 3e-5


# ---- PGURE risk (FP64 accumulation of FP32 factor terms)

@pytest.mark.parametrize("mode", ["compat", "fixed"])
def test_risk(capi, g, mode):
    lams = g["risk_lams"]
    a, m, s = float(g["alpha"]), float(g["mu"]), float(g["sigma"])
    compat = capi.COMPAT_ALL if mode == "compat" else 0
    r1 = capi.risk_window(g["u_8"], 4, 1, g["rows_8"], g["cols_8"], lams, a, m, s, 11, compat)
    r0 = g["risk_8_" + mode]
    scale = np.abs(r0).max()
    print(mode, "risk oracle", r0, "gpu", r1)
    assert np.abs(r1 - r0).max() < 1e-4 * scale + 1e-9


# ---- whole sequence through pgsvt_denoise

def test_denoise_fixed_lambda_matches_oracle(capi, g):
    p = capi.default_params(median_size=-1, optimize_pgure=0, lambda_=0.1)
    Y, est, st = capi.denoise(g["X"], p)
    Y0 = g["Y_fixed"]
    assert np.abs(Y - Y0).max() < 2e-5 * np.abs(Y0).max()
    assert abs(_psnr(Y0, Y)) > 80  # GPU output within FP32 noise of the oracle
    assert np.all(est[:, 0] == 0.1)
    assert st.kernel_launches > 0


def test_denoise_pgure_matches_oracle(capi, oracle, g):
    a, m, s = float(g["alpha"]), float(g["mu"]), float(g["sigma"])
    p = capi.default_params(median_size=-1, random_seed=11, alpha=a, mu=m, sigma=s,
                            search_points=8, search_rounds=2)
    Y, est, st = capi.denoise(g["X"], p)
    Y0, est0 = g["Y_pgure"], g["est_pgure"]
    np.testing.assert_array_equal(est[:, 1:], est0[:, 1:])
    # lambda: same search schedule, FP32 vs FP64 risks; compare the risk the
    # oracle assigns to both choices (risk gap) and the output PSNR
    X = g["X"].astype(np.float64)
    gaps = []
    for t in (0, 8, 15):
        u = _window(X, t, 7)
        rows, cols = oracle.arps_window(u, 4, 7, t, 7, 16)
        r = oracle.risk_window(u, 4, 1, rows, cols, [est[t, 0], est0[t, 0]], a, m, s, 11)
        gaps.append((r[0] - r[1]) / abs(r[1]))
    print("lambda gpu", est[:, 0], "oracle", est0[:, 0], "risk gaps", gaps)
    assert max(gaps) < 0.01
    clean_like = Y0
    assert np.abs(Y - Y0).max() < 5e-3 * np.abs(Y0).max()
    assert st.risk_evals > 0


def test_denoise_is_deterministic(capi, g):
    a, m, s = float(g["alpha"]), float(g["mu"]), float(g["sigma"])
    p = capi.default_params(median_size=-1, random_seed=3, alpha=a, mu=m, sigma=s)
    Y1, e1, _ = capi.denoise(g["X"], p)
    Y2, e2, _ = capi.denoise(g["X"], p)
    np.testing.assert_array_equal(Y1, Y2)
    np.testing.assert_array_equal(e1, e2)


@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32", "float64"])
def test_input_dtypes(capi, oracle, pkg, dtype):
    noisy, _, _ = pkg.synth.workload("plain_64", seed=2, side=32, nt=16)
    X = np.clip(noisy, 0, 255 if dtype == "uint8" else 6e4).astype(dtype)
    kw = dict(median_size=-1, optimize_pgure=0, lambda_=0.3)
    Y, _, _ = capi.denoise(X, capi.default_params(**kw))
    Y0, _, _ = oracle.denoise(X, n_jobs=4, **kw)
    assert np.abs(Y - Y0).max() < 3e-5 * np.abs(Y0).max()


def test_window_batching_does_not_change_results(capi, g):
    kw = dict(median_size=-1, optimize_pgure=0, lambda_=0.1)
    Y1, _, _ = capi.denoise(g["X"], capi.default_params(window_batch=1, **kw))
    Y5, _, _ = capi.denoise(g["X"], capi.default_params(window_batch=5, **kw))
    np.testing.assert_array_equal(Y1, Y5)


def test_svt_estimator_on_gpu(pkg, g):
    s = pkg.SVT(motion_filter=None, noise_alpha=float(g["alpha"]), noise_mu=float(g["mu"]),
                noise_sigma=float(g["sigma"]), random_seed=11)
    s.denoise(np.ascontiguousarray(g["X"]))
    assert s.Y_.shape == g["X"].shape
    assert np.all(s.lambda1s_ > 0) and np.all(s.noise_alphas_ == float(g["alpha"]))


def test_svt_estimator_with_learned_lambda(pkg):
    """The shim with the shipped learned proposal, on the reference's default
    path (median pre-filter 5, noise estimated): fewer risk evaluations than
    the plain search, the same output to within the risk gap's effect."""
    Y, noise = pkg.learned.random_sequence(10 ** 7 + 200, estimated=True)  # held out
    assert noise is None
    plain = pkg.SVT(random_seed=7).denoise(Y)
    learned = pkg.SVT(random_seed=7, learned_lambda=True).denoise(Y)
    print("risk evaluations plain %d learned %d" % (plain.status_.risk_evals,
                                                    learned.status_.risk_evals))
    assert learned.status_.risk_evals < plain.status_.risk_evals
    assert np.all(np.isfinite(learned.lambda1s_)) and np.all(learned.lambda1s_ >= 0)
    err = np.abs(learned.Y_ - plain.Y_).max() / np.abs(plain.Y_).max()
    print("max relative output difference", err)
    assert err < 0.05


def test_errors(capi, pkg):
    X = np.ones((16, 16, 16), np.float32)
    p = capi.default_params(median_size=-1, optimize_pgure=0, lambda_=0.1)
    with pytest.raises(pkg.PgsvtError) as e:
        capi.denoise(np.ones((16, 12, 16), np.float32), p)
    assert e.value.code == capi.ERR_INVALID_ARG
    Xn = X.copy()
    Xn[1, 2, 3] = -1
    with pytest.raises(pkg.PgsvtError) as e:
        capi.denoise(Xn, p)
    assert e.value.code == capi.ERR_NONFINITE
    Xn[1, 2, 3] = np.nan
    with pytest.raises(pkg.PgsvtError) as e:
        capi.denoise(Xn, p)
    assert e.value.code == capi.ERR_NONFINITE
    with pytest.raises(pkg.PgsvtError) as e:  # median window 2*16+1 wider than the frame
        capi.denoise(X, capi.default_params(optimize_pgure=0, lambda_=0.1, median_size=16))
    assert e.value.code == capi.ERR_UNSUPPORTED
    with pytest.raises(pkg.PgsvtError) as e:  # 2*8+1 > 16
        capi.denoise(X, capi.default_params(optimize_pgure=0, lambda_=0.1, median_size=8))
    assert e.value.code == capi.ERR_INVALID_ARG
    with pytest.raises(pkg.PgsvtError) as e:
        capi.denoise(X[:, :, :8], p)  # shorter than the trajectory
    assert e.value.code == capi.ERR_INVALID_ARG
    # the library stays usable after errors
    Y, _, _ = capi.denoise(X, p)
    assert np.isfinite(Y).all()


def test_all_zero_sequence(capi):
    # umax = 0: the reference divides 0/0 and zeroes non-finite voxels
    X = np.zeros((16, 16, 16), np.float32)
    Y, _, _ = capi.denoise(X, capi.default_params(median_size=-1, optimize_pgure=0, lambda_=0.1))
    assert np.all(Y == 0)


def test_frame_range_shards_sum_to_full_run(capi, pkg, g):
    kw = dict(median_size=-1, optimize_pgure=0, lambda_=0.1)
    Y, _, _ = capi.denoise(g["X"], capi.default_params(**kw))
    parts = []
    for r in range(3):
        b, e = pkg.shard.shard_frames(g["X"].shape[2], 3, r)
        Yr, _, _ = capi.denoise(g["X"], capi.default_params(frame_begin=b, frame_end=e, **kw))
        assert not Yr[:, :, :b].any() and not Yr[:, :, e:].any()
        parts.append(Yr)
    np.testing.assert_array_equal(sum(parts), Y)


def test_largest_frames_identity_and_shards(capi, pkg):
    """1024 x 1024 frames (the largest side of the uneven-batch
    configuration), where position and voxel indices reach their widest
    ranges.  A fixed lambda large enough that the exponential weights
    shrink nothing (svt.hpp:137: the threshold smax exp(-lambda s^2 / 2)
    underflows) rebuilds every patch, so the output is the input; and two
    frame ranges give the frames of one full run, bit for bit."""
    noisy, _, _ = pkg.synth.workload("arps_256", seed=31, side=1024, nt=16)
    X = noisy.astype(np.float32)
    kw = dict(median_size=-1, optimize_pgure=0, lambda_=1e12)
    Y, _, st = capi.denoise(X, capi.default_params(**kw))
    assert st.windows == 16
    err = np.abs(Y - X).max() / np.abs(X).max()
    print("max relative difference to the input", err)
    assert err < 1e-5
    kw["lambda_"] = 0.1
    Y, _, _ = capi.denoise(X, capi.default_params(**kw))
    parts = [capi.denoise(X, capi.default_params(frame_begin=b, frame_end=e, **kw))[0]
             for b, e in ((0, 7), (7, 16))]
    np.testing.assert_array_equal(parts[0] + parts[1], Y)


# ---- median pre-filter of the ARPS input

def test_median_filter_matches_reference_fixtures(capi):
    z = np.load(os.path.join(GOLDEN, "median.npz"))
    for k in range(int(z["n"])):
        out = capi.median_filter(z["in_%d" % k], int(z["r_%d" % k]))
        np.testing.assert_array_equal(out, z["out_%d" % k])


def test_denoise_with_median_prefilter_matches_oracle(capi, oracle, g):
    # fixed lambda: the output depends on the filter only through the ARPS
    # trajectories, which must be the oracle's
    X = g["X"].astype(np.float64) * 7.3  # non-integer values: the uint16 conversion truncates
    p = capi.default_params(median_size=5, optimize_pgure=0, lambda_=0.1)
    Y, est, st = capi.denoise(X, p)
    Y0, _, _ = oracle.denoise(X, median_size=5, optimize_pgure=0, lambda_=0.1, n_jobs=4)
    assert np.abs(Y - Y0).max() < 2e-5 * np.abs(Y0).max()
    # and the filter changed the trajectories
    Y1, _, _ = oracle.denoise(X, median_size=-1, optimize_pgure=0, lambda_=0.1, n_jobs=4)
    assert np.abs(Y1 - Y0).max() > 1e-3 * np.abs(Y0).max()


def test_integer_input_arps_ties_match_oracle(capi, oracle, pkg):
    # integer-valued input: ARPS compares exact integer sums of squared
    # differences and settles equal sums as the reference's FP64 costs do;
    # coarse quantisation makes flat regions, hence many exact ties
    clean = pkg.synth.blobs(40, 18, 10, seed=3) / 25.0
    X = np.asfortranarray(np.round(clean).astype(np.uint16))
    p = capi.default_params(median_size=-1, optimize_pgure=0, lambda_=0.1)
    Y, _, st = capi.denoise(X, p)
    Y0, _, _ = oracle.denoise(X.astype(np.float64), median_size=-1, optimize_pgure=0,
                              lambda_=0.1, n_jobs=4)
    print("FP64 tie decisions:", st.arps_exact_steps)
    assert np.abs(Y - Y0).max() < 2e-5 * np.abs(Y0).max()


@pytest.mark.parametrize("bs,T,ov", [(12, 9, 1), (16, 15, 2)])
def test_large_patches_match_oracle(capi, oracle, pkg, bs, T, ov):
    # patch sides 9..16 run the runtime-size ARPS and evaluation kernels and
    # the 8 x 32-lane shared-memory SVD (256 rows for 16 x 16 patches)
    noisy, _, _ = pkg.synth.workload("arps_256", seed=12, side=40, nt=T + 3)
    X = noisy.astype(np.float64)
    fr = (T // 2, T // 2 + 3)
    kw = dict(median_size=-1, optimize_pgure=0, lambda_=0.15, block_size=bs, block_overlap=ov,
              traj_length=T, frame_begin=fr[0], frame_end=fr[1])
    Y, _, _ = capi.denoise(X, capi.default_params(**kw))
    Y0, _, _ = oracle.denoise(X, n_jobs=4, **kw)
    f = slice(*fr)
    err = np.abs(Y[:, :, f] - Y0[:, :, f]).max() / np.abs(Y0[:, :, f]).max()
    print("max relative difference", err)
    assert err < 1e-4


# ---- FP64 decisions of the Jacobi convergence test

def _near_degenerate_window(seed, G=8, bs=4, nwin=15):
    """A window whose kept patches' Casorati matrices are designed: G x G
    disjoint bs x bs blocks, and a trajectory table sending every position
    to a block.  Block b holds orthogonal columns a_k = s_k u_k (random
    orthonormal u_k) in which three pairs have equal norms (s_1 = s_0,
    s_5 = s_4, s_10 = s_9) and are coupled, a_j += d s_j u_i with d in
    [1.5e-6, 3.5e-6]: a first sweep finds only these near-degenerate pairs,
    with inner products between the rotation threshold (1e-6) and four times
    it.  Returns (u, rows, cols)."""
    rng = np.random.default_rng(seed)
    m, S = bs * bs, bs * G
    u = np.zeros((S, S, nwin))
    for b in range(G * G):
        Uq, _ = np.linalg.qr(rng.standard_normal((m, nwin)))
        s = np.sort(rng.uniform(0.05, 1.0, nwin))[::-1]
        B = Uq * s
        for i in (0, 4, 9):
            s[i + 1] = s[i]
            B[:, i + 1] = s[i] * (Uq[:, i + 1] + rng.uniform(1.5e-6, 3.5e-6) * Uq[:, i])
        r0, c0 = bs * (b % G), bs * (b // G)
        for k in range(nwin):  # Casorati row e is pixel (e % bs, e // bs)
            u[r0:r0 + bs, c0:c0 + bs, k] = B[:, k].reshape(bs, bs, order="F")
    u = np.asfortranarray(u / u.max())
    P = (S - bs + 1) ** 2
    blk = np.arange(P) % (G * G)
    rows = np.tile((bs * (blk % G)).astype(np.int32), (nwin, 1))
    cols = np.tile((bs * (blk // G)).astype(np.int32), (nwin, 1))
    return u, rows, cols


def test_jacobi_fp64_convergence_decisions(capi, oracle):
    """Near-degenerate singular pairs whose inner products sit at the FP32
    noise level of the rotation threshold: when a sweep's only rotations are
    of such pairs, the kernel decides convergence from FP64 inner products of
    the FP32 entries.  The decisions are taken (counted) and the singular
    values stay within the tolerance of FP64 LAPACK, the pairs' close values
    included."""
    u, rows, cols = _near_degenerate_window(17)
    S1, st = capi.svd_window(u, 4, 1, rows, cols, status=True)
    S0 = oracle.svd_window(u, 4, 1, rows, cols)
    S1 = S1.astype(np.float64)
    err = np.abs(S1 - S0) / S0[:, :1]
    print("FP64 convergence tests %d over %d matrices, %.2f sweeps per warp, max err %.3g"
          % (st.svd_fp64_tests, st.svd_matrices, st.svd_warp_sweeps / max(1, st.svd_matrices / 8),
             err.max()))
    assert st.svd_fp64_tests > 0
    assert err.max() < 2e-5
    # the close pairs are resolved as two values, in order
    d0 = S0[:, 0] - S0[:, 1]
    d1 = S1[:, 0] - S1[:, 1]
    assert np.all(d1 >= 0)
    assert np.abs(d1 - d0).max() < 2e-5


# ---- the lambda search against a dense grid of the oracle's risk

@pytest.mark.parametrize("noise", ["counts", "normalised", "estimated"])
def test_lambda_search_within_1pct_of_dense_grid(capi, oracle, pkg, noise):
    """The dense-grid minimum of the FP64 oracle's risk is the arbiter of the
    search: on sampled windows the GPU's plain search and the learned
    proposal + narrow search both return a lambda whose oracle risk is within
    1% of the minimum over 256 lambda values spanning [0, upper].  Noise
    parameters: the raw counts used on the normalised window (the
    reference's units, whose risk is smallest at a bound), the same divided
    by the sequence maximum, and estimated per window."""
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=5, side=64, nt=20)
    X = noisy.astype(np.float64)
    if noise == "normalised":
        a, m, s = a / X.max(), m / X.max(), s / X.max()
    elif noise == "estimated":
        a = m = s = -1.0
    kw = dict(median_size=-1, random_seed=7, alpha=a, mu=m, sigma=s)
    _, est, _, ex = capi.denoise_ex(X, capi.default_params(**kw))
    model = pkg.learned.load_model()
    _, estl, _, exl = capi.denoise_ex(X, capi.default_params(lambda_model=model.ctypes.data, **kw))
    grid = np.concatenate([[0.0], np.geomspace(1e-4, 100.0, 255)])
    for t in (7, 10, 19):
        u = _window(X, t, 7)
        rows, cols = oracle.arps_window(u, 4, 7, t, 7, 20)
        na, nm_, ns = est[t, 1], est[t, 2], est[t, 3]  # caller-side values used
        r = oracle.risk_window(u, 4, 1, rows, cols, np.concatenate([grid, [est[t, 0],
                               estl[t, 0]]]), na, nm_, ns, 7)
        rmin, rg, rl = r[:-2].min(), r[-2], r[-1]
        gp, gl = (rg - rmin) / abs(rmin), (rl - rmin) / abs(rmin)
        print("%s t=%d grid min %.6g at %.4g; plain %.4g (%d evals) gap %.2e; learned %.4g "
              "(%d evals) gap %.2e" % (noise, t, rmin, grid[np.argmin(r[:-2])], est[t, 0],
                                       ex["evals"][t], gp, estl[t, 0], exl["evals"][t], gl))
        assert gp <= 0.01
        assert gl <= 0.01


def test_narrow_search_sentinels_match_oracle(capi, oracle, g):
    """A given proposal far from the risk minimum (which lies at the bottom of
    the plain grid): GPU and oracle both see a sentinel beat the narrow grid,
    fall back to the plain search, and spend the same evaluations."""
    a, m, s = float(g["alpha"]), float(g["mu"]), float(g["sigma"])
    kw = dict(median_size=-1, random_seed=11, alpha=a, mu=m, sigma=s, frame_begin=6, frame_end=10,
              lambda_hint=1.0)
    _, est, _, ex = capi.denoise_ex(g["X"], capi.default_params(**kw))
    _, est0, rep = oracle.denoise(g["X"], n_jobs=2, **kw)
    f = slice(6, 10)
    np.testing.assert_array_equal(ex["evals"][f], rep.evals[f])
    assert np.all(ex["evals"][f] > 6)
    np.testing.assert_allclose(est[f, 0], est0[f, 0], rtol=1e-12)
