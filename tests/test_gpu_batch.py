"""Batches of uneven sequences (pgsvt_denoise_batch) and the SVD kernel
shapes of the autotuner, against single-sequence calls and the FP64 oracle.

Tolerances: a batch runs every sequence through the same kernels as a
single call, so its outputs are identical; risks at fixed lambdas are FP64
sums of FP32 terms and are compared with the oracle at 1e-4 relative (as the
component risk tests); the two SVD kernel shapes round differently in FP32
and agree to 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _seq(pkg, side, nt, seed, bs, T, lams=None):
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=seed, side=side, nt=nt)
    return dict(X=noisy, bs=bs, T=T, noise=(a, m, s), lambdas=lams)


def _params(capi, q, **kw):
    a, m, s = q["noise"]
    return capi.default_params(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s,
                               block_size=q["bs"], traj_length=q["T"], **kw)


def _batch(pkg, capi):
    lam = np.array([0.01, 0.1, 1.0, 10.0])
    return [_seq(pkg, 48, 20, 1, 4, 15, lam), _seq(pkg, 40, 12, 2, 6, 9, lam * 3),
            _seq(pkg, 36, 24, 3, 8, 21, lam / 2), _seq(pkg, 32, 16, 4, 4, 15)]


def test_batch_matches_single_calls(capi, pkg):
    seqs = _batch(pkg, capi)
    inp = [dict(X=q["X"], params=_params(capi, q), lambdas=q["lambdas"]) for q in seqs]
    res, st = capi.denoise_batch(inp, slots=3)
    assert st.code == 0 and st.windows == sum(q["X"].shape[2] for q in seqs)
    for q, r in zip(inp, res):
        one, _ = capi.denoise_batch([q], slots=1)
        np.testing.assert_array_equal(r["Y"], one[0]["Y"])
        np.testing.assert_array_equal(r["est"], one[0]["est"])
        if q["lambdas"] is not None:
            np.testing.assert_array_equal(r["risks"], one[0]["risks"])
            # the output lambda is the list's value of least risk
            best = np.asarray(q["lambdas"])[np.argmin(r["risks"], axis=1)]
            np.testing.assert_array_equal(r["est"][:, 0], best)
            assert r["status"].risk_evals == q["X"].shape[2] * len(q["lambdas"])


def test_batch_fixed_lambda_risks_match_oracle(capi, pkg, oracle):
    q = _batch(pkg, capi)[0]
    res, _ = capi.denoise_batch([dict(X=q["X"], params=_params(capi, q),
                                      lambdas=q["lambdas"])])
    X = q["X"].astype(np.float64)
    a, m, s = q["noise"]
    for t in (0, 10, 19):
        s0 = 0 if t < 7 else (X.shape[2] - 15 if t >= X.shape[2] - 7 else t - 7)
        u = X[:, :, s0:s0 + 15]
        u = u / u.max()
        rows, cols = oracle.arps_window(u, 4, 7, t, 7, X.shape[2])
        r0 = oracle.risk_window(u, 4, 1, rows, cols, q["lambdas"], a, m, s, 5)
        np.testing.assert_allclose(res[0]["risks"][t], r0, rtol=1e-4, atol=1e-7)


def test_batch_reports_errors_per_sequence(capi, pkg):
    seqs = _batch(pkg, capi)[:2]
    bad = dict(X=seqs[1]["X"][:, :20, :], params=_params(capi, seqs[1]))  # not square
    good = dict(X=seqs[0]["X"], params=_params(capi, seqs[0]))
    with pytest.raises(capi.PgsvtError, match="square"):
        capi.denoise_batch([good, bad])


@pytest.mark.parametrize("bs,T", [(4, 15), (6, 15), (8, 21)])
def test_alternative_svd_shape_matches_oracle(capi, pkg, oracle, bs, T):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=6, side=40, nt=T + 2)
    X = noisy.astype(np.float64)
    fr = (T // 2, T // 2 + 2)
    base = dict(median_size=0, optimize_pgure=0, lambda_=0.5, block_size=bs, traj_length=T,
                frame_begin=fr[0], frame_end=fr[1])
    Y0, _, st0 = capi.denoise(X, capi.default_params(autotune=0, **base))
    Y1, _, st1 = capi.denoise(X, capi.default_params(autotune=2, **base))
    assert st0.svd_variant == 0 and st1.svd_variant == 1
    Yo, _, _ = oracle.denoise(X, median_size=-1, optimize_pgure=0, lambda_=0.5, block_size=bs,
                              traj_length=T, frame_begin=fr[0], frame_end=fr[1], n_jobs=2)
    f = slice(*fr)
    scale = np.abs(Yo[:, :, f]).max()
    for Y in (Y0, Y1):
        assert np.abs(Y[:, :, f] - Yo[:, :, f]).max() <= 1e-4 * scale
    assert np.abs(Y1[:, :, f] - Y0[:, :, f]).max() <= 1e-4 * scale
    # the shared-memory form applies the register form's rotations in the same
    # order: identical results
    Y2, _, st2 = capi.denoise(X, capi.default_params(autotune=3, **base))
    assert st2.svd_variant == 2
    np.testing.assert_array_equal(Y2[:, :, f], Y0[:, :, f])


@pytest.mark.parametrize("bs,T", [(4, 15), (4, 9), (8, 15), (7, 9)])
def test_eight_rows_per_lane_shape_matches_oracle(capi, pkg, oracle, bs, T):
    noisy, _, _ = pkg.synth.workload("arps_256", seed=9, side=40, nt=T + 2)
    X = noisy.astype(np.float64)
    fr = (T // 2, T // 2 + 2)
    base = dict(median_size=0, optimize_pgure=0, lambda_=0.5, block_size=bs, traj_length=T,
                frame_begin=fr[0], frame_end=fr[1])
    Y0, _, st0 = capi.denoise(X, capi.default_params(autotune=0, **base))
    Y3, _, st3 = capi.denoise(X, capi.default_params(autotune=4, **base))
    assert st0.svd_variant == (4 if bs >= 7 else 0) and st3.svd_variant == 3
    Yo, _, _ = oracle.denoise(X, median_size=-1, optimize_pgure=0, lambda_=0.5, block_size=bs,
                              traj_length=T, frame_begin=fr[0], frame_end=fr[1], n_jobs=2)
    f = slice(*fr)
    scale = np.abs(Yo[:, :, f]).max()
    assert np.abs(Y3[:, :, f] - Yo[:, :, f]).max() <= 1e-4 * scale
    assert np.abs(Y3[:, :, f] - Y0[:, :, f]).max() <= 1e-4 * scale


def test_eight_rows_per_lane_shape_with_pgure(capi, pkg, oracle):
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=8, side=48, nt=18)
    base = dict(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s, frame_begin=6, frame_end=10)
    Y0, e0, _ = capi.denoise(noisy, capi.default_params(autotune=0, **base))
    Y3, e3, st3 = capi.denoise(noisy, capi.default_params(autotune=4, **base))
    assert st3.svd_variant == 3
    f = slice(6, 10)
    np.testing.assert_allclose(e3[f], e0[f], rtol=2e-3)
    scale = np.abs(Y0[:, :, f]).max()
    assert np.abs(Y3[:, :, f] - Y0[:, :, f]).max() <= 1e-3 * scale


@pytest.mark.parametrize("bs,T", [(5, 15), (6, 9), (8, 15), (8, 9), (7, 15)])
def test_qr_preconditioned_shape_matches_oracle(capi, pkg, oracle, bs, T):
    """Jacobi on the triangle of B's Householder QR factorisation (patches of
    17..64 rows): right singular vectors from the sweeps, left ones from B."""
    noisy, _, _ = pkg.synth.workload("arps_256", seed=10, side=40, nt=T + 2)
    X = noisy.astype(np.float64)
    fr = (T // 2, T // 2 + 2)
    base = dict(median_size=0, optimize_pgure=0, lambda_=0.5, block_size=bs, traj_length=T,
                frame_begin=fr[0], frame_end=fr[1])
    Y0, _, st0 = capi.denoise(X, capi.default_params(autotune=0, **base))
    Y4, _, st4 = capi.denoise(X, capi.default_params(autotune=5, **base))
    # the untuned shape of 7x7 and 8x8 patches is the QR form itself
    assert st0.svd_variant == (4 if bs >= 7 else 0) and st4.svd_variant == 4
    Yo, _, _ = oracle.denoise(X, median_size=-1, optimize_pgure=0, lambda_=0.5, block_size=bs,
                              traj_length=T, frame_begin=fr[0], frame_end=fr[1], n_jobs=2)
    f = slice(*fr)
    scale = np.abs(Yo[:, :, f]).max()
    print("max relative difference to the oracle: QR form %.2e, default %.2e"
          % (np.abs(Y4[:, :, f] - Yo[:, :, f]).max() / scale,
             np.abs(Y0[:, :, f] - Yo[:, :, f]).max() / scale))
    assert np.abs(Y4[:, :, f] - Yo[:, :, f]).max() <= 1e-4 * scale
    assert np.abs(Y4[:, :, f] - Y0[:, :, f]).max() <= 1e-4 * scale


def test_qr_preconditioned_shape_with_pgure(capi, pkg, oracle):
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=8, side=48, nt=18)
    base = dict(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s, frame_begin=6,
                frame_end=10, block_size=8)
    Y0, e0, _ = capi.denoise(noisy, capi.default_params(autotune=2, **base))  # 2 x 32 lanes
    Y4, e4, st4 = capi.denoise(noisy, capi.default_params(autotune=5, **base))
    assert st4.svd_variant == 4
    f = slice(6, 10)
    np.testing.assert_allclose(e4[f], e0[f], rtol=2e-3)
    scale = np.abs(Y0[:, :, f]).max()
    assert np.abs(Y4[:, :, f] - Y0[:, :, f]).max() <= 1e-3 * scale


@pytest.mark.parametrize("bs,T", [(4, 9), (3, 7)])
def test_two_kernel_register_form_is_identical(capi, pkg, bs, T):
    """Patches of at most 16 rows run the register form's sweeps and its
    factors in two kernels; the single-kernel shared-memory form applies the
    same rotations in the same order: identical results."""
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=14, side=40, nt=T + 3)
    base = dict(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s, block_size=bs,
                traj_length=T)
    Y0, e0, st0 = capi.denoise(noisy, capi.default_params(autotune=0, **base))
    Y2, e2, st2 = capi.denoise(noisy, capi.default_params(autotune=3, **base))
    assert st0.svd_variant == 0 and st2.svd_variant == 2
    np.testing.assert_array_equal(Y2, Y0)
    np.testing.assert_array_equal(e2, e0)
    assert st2.svd_warp_sweeps == st0.svd_warp_sweeps


def test_shared_memory_svd_form_with_pgure(capi, pkg):
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=8, side=48, nt=18)
    base = dict(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s, frame_begin=6, frame_end=10)
    Y0, e0, st0 = capi.denoise(noisy, capi.default_params(autotune=0, **base))
    Y2, e2, st2 = capi.denoise(noisy, capi.default_params(autotune=3, **base))
    assert st2.svd_variant == 2
    np.testing.assert_array_equal(Y0, Y2)
    np.testing.assert_array_equal(e0, e2)
    assert st0.svd_warp_sweeps == st2.svd_warp_sweeps


def test_autotuner_picks_and_caches(capi, pkg):
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=7, side=64, nt=16)
    p = capi.default_params(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s, autotune=1,
                            block_size=6, traj_length=9)
    Y1, e1, st1 = capi.denoise(noisy, p)
    Y2, e2, st2 = capi.denoise(noisy, p)
    assert st1.svd_tuned == 1 and st2.svd_tuned == 0
    assert st1.svd_variant == st2.svd_variant
    # the tuned call's outputs are those of its chosen shape
    np.testing.assert_array_equal(Y1, Y2)
    np.testing.assert_array_equal(e1, e2)


def test_batch_workers_with_lambda_lists_of_different_sizes(capi, pkg):
    """Sequences on concurrent workers whose rounds need different amounts
    of shared memory (16 lambda values, then the single-lambda final pass)
    all run: a kernel's shared-memory limit is only ever raised."""
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=23, side=64, nt=15)
    p = capi.default_params(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s,
                            frame_begin=7, frame_end=8)
    seqs = [dict(X=noisy, params=p, lambdas=np.geomspace(1e-3, 100.0, 16) * (1 + 0.01 * i))
            for i in range(8)]
    for _ in range(3):
        res, st = capi.denoise_batch(seqs, slots=4)
        assert all(np.isfinite(r["risks"][7]).all() for r in res)


@pytest.mark.parametrize("side,bs,T", [(48, 4, 15), (64, 3, 7)])
def test_tma_staged_factors_are_identical(capi, pkg, side, bs, T):
    """The two-kernel register form with its factors kernel reading
    TMA-staged frame tiles (variant 5, frame sides that are multiples of 16)
    assembles the same Casorati rows and fields as the global-memory gather:
    identical results, PGURE search included."""
    noisy, _, (a, m, s) = pkg.synth.workload("arps_256", seed=31, side=side, nt=T + 4)
    base = dict(median_size=0, random_seed=5, alpha=a, mu=m, sigma=s, block_size=bs,
                traj_length=T)
    Y0, e0, st0 = capi.denoise(noisy, capi.default_params(autotune=0, **base))
    Y5, e5, st5 = capi.denoise(noisy, capi.default_params(autotune=6, **base))
    assert st0.svd_variant == 0 and st5.svd_variant == 5
    np.testing.assert_array_equal(Y5, Y0)
    np.testing.assert_array_equal(e5, e0)
    # fresh probes per window (negative seed: one probe set per window)
    base["random_seed"] = -1
    _, _, st = capi.denoise(noisy, capi.default_params(autotune=6, **base))
    assert st.svd_variant == 5
