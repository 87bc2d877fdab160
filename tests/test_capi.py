"""CPU tests of the C-ABI library and the Python front end (no compute calls)."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "pgsvt.h")).read()
    return sorted(set(re.findall(r"\b(pgsvt_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(capi):
    L = capi.load()
    decl = _declared_symbols()
    assert set(decl) == set(capi.EXPORTS)
    for name in decl:
        assert getattr(L, name) is not None


def test_version_and_defaults(capi):
    assert "sm_103a" in capi.version()
    p = capi.default_params()
    # reference defaults: pguresvt/_pguresvt.pyx:151-168, svt.py:172-191
    assert (p.traj_length, p.block_size, p.block_overlap, p.motion_window) == (15, 4, 1, 7)
    assert (p.median_size, p.noise_method, p.max_iter, p.n_jobs, p.random_seed) == (5, 4, 500, -1, -1)
    assert (p.optimize_pgure, p.exp_weighting, p.motion_estimation) == (1, 1, 1)
    assert (p.lambda_, p.alpha, p.mu, p.sigma, p.tol) == (-1.0, -1.0, -1.0, -1.0, 1e-7)
    assert p.compat_flags == capi.COMPAT_ALL


def test_params_layout_matches_oracle(capi, oracle):
    # the oracle mirrors pgsvt_params field by field, then adds its own
    # per-frame hint and output pointers
    names = [f[0] for f in capi.Params._fields_]
    assert names == [f[0] for f in oracle.OrcParams._fields_][:len(names)]
    for n in names:
        assert getattr(capi.Params, n).offset == getattr(oracle.OrcParams, n).offset


def test_lambda_model_constants(capi):
    text = open(os.path.join(ROOT, "include", "pgsvt.h")).read()
    for name in ("LAMBDA_FEATURES", "LAMBDA_HIDDEN", "LAMBDA_SAMPLES", "LAMBDA_MODEL_FLOATS",
                 "LAMBDA_PARAM_OFFSET", "LAMBDA_PARAMS"):
        m = re.search(r"#define PGSVT_%s (\d+)" % name, text)
        assert m and int(m.group(1)) == getattr(capi, name), name
    H, F = capi.LAMBDA_HIDDEN, capi.LAMBDA_FEATURES
    assert capi.LAMBDA_PARAMS == H * F + H + 2 * (H * H + H) + H + 1
    assert capi.LAMBDA_MODEL_FLOATS == 2 * F + capi.LAMBDA_PARAMS + 2


def test_svt_learned_lambda_parameters(pkg, capi):
    """The SVT shim's keyword-only extras: the shipped (or a given) learned
    model and the SVD shape selection reach pgsvt_params."""
    X = np.ones((32, 32, 16))
    s = pkg.SVT(learned_lambda=True, autotune=1)
    s._check_arguments(X)
    p = s.params()
    assert p.lambda_model and p.autotune == 1
    assert s._model.dtype == np.float32 and s._model.size == capi.LAMBDA_MODEL_FLOATS
    s = pkg.SVT()
    s._check_arguments(X)
    assert not s.params().lambda_model
    s = pkg.SVT(lambda_model=np.zeros(10, np.float32))
    s._check_arguments(X)
    with pytest.raises(ValueError, match="lambda model has 10 floats"):
        s.params()
    s = pkg.SVT(learned_lambda=True, patch_size=8)  # outside the shipped model's range
    s._check_arguments(X)
    with pytest.raises(ValueError, match="covers patch_size 4"):
        s.params()


class TestErrors:
    """pguresvt/tests/test_svt.py:109-164: validation happens before any call."""

    def setup_method(self, method):
        self.X = np.ones((32, 32, 16))

    def test_negative_data(self, pkg):
        with pytest.raises(ValueError, match="Negative values found in data"):
            s = pkg.SVT()
            self.X[0, 0, 0] = -1
            s.denoise(self.X)

    def test_error_patch_overlap(self, pkg):
        with pytest.raises(ValueError, match="Invalid patch_overlap parameter"):
            pkg.SVT(patch_size=10, patch_overlap=11).denoise(self.X)

    def test_error_trajectory_length(self, pkg):
        with pytest.raises(ValueError, match="Invalid trajectory_length parameter"):
            pkg.SVT(trajectory_length=14).denoise(self.X)

    def test_error_motion_window(self, pkg):
        with pytest.raises(ValueError, match="Invalid motion_window parameter"):
            pkg.SVT(motion_estimation=True, motion_window=1).denoise(self.X)
        with pytest.raises(ValueError, match="Invalid motion_window parameter"):
            pkg.SVT(motion_estimation=True, motion_window=8).denoise(self.X)

    def test_error_motion_filter(self, pkg):
        with pytest.raises(ValueError, match="Invalid motion_filter parameter"):
            pkg.SVT(motion_estimation=True, motion_filter=0.5).denoise(self.X)

    def test_error_lambda1(self, pkg):
        with pytest.raises(ValueError, match="Invalid lambda1 parameter"):
            pkg.SVT(optimize_pgure=False, lambda1=-1.0).denoise(self.X)

    def test_error_non_square(self, pkg):
        m, _, _ = self.X.shape
        with pytest.raises(ValueError, match="requires square images"):
            pkg.SVT().denoise(self.X[: m // 2, :, :])

    def test_error_non_power_of_two(self, pkg):
        m, n, _ = self.X.shape
        with pytest.raises(ValueError, match="requires image dimensions 2\\^N"):
            pkg.SVT().denoise(self.X[: m - 1, : n - 1, :])

    def test_error_dtype(self, pkg):
        with pytest.raises(TypeError, match="Invalid dtype"):
            pkg.SVT().denoise((self.X == 0))


def test_params_carry_sentinels(pkg):
    s = pkg.SVT(noise_alpha=0.2, noise_mu=None, random_seed=None, motion_filter=None)
    s._check_arguments(np.ones((8, 8, 4)))
    p = s.params()
    assert (p.alpha, p.mu, p.sigma, p.random_seed, p.median_size) == (0.2, -1.0, -1.0, -1, -1)
