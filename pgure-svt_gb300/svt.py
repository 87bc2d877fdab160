"""SVT estimator with the parameters of the reference's Python API.

Mirrors pguresvt/svt.py:77-337 (same constructor arguments, validation
messages, dtype dispatch, Fortran ordering and result attributes) on top of
the CUDA library through its C ABI.  Arguments this build adds are
keyword-only and default to the reference's behaviour.
"""
import numpy as np

from . import _capi


def _is_power_of_two(n):
    """Checks if n is a power of 2"""
    return (n & (n - 1) == 0) and n != 0


class SVT:
    """Singular value thresholding for denoising image sequences (GB300).

    Parameters are those of the reference ``pguresvt.SVT``; see its
    docstring (pguresvt/svt.py:94-169).  Extra keyword-only arguments:

    compat_flags : int, default=COMPAT_ALL
        Reference behaviours reproduced for parity (see include/pgsvt.h).
    search_points, search_rounds : int
        Lambda values of the search grid (each refinement round places half
        as many) and refinement rounds.
    lambda_hint : float or None
        A proposed lambda (e.g. from the learned proposal): the search
        brackets it first and falls back to the full search.
    learned_lambda : bool, default=False
        Let the shipped learned model (lambda_mlp.npz, trained for 4x4
        patches and 15-frame trajectories) propose each window's lambda; a
        narrow search around the proposal replaces the plain search, which
        remains the fallback.
    lambda_model : ndarray or None
        A model of the same form to use instead of the shipped one.
    autotune : int, default=0
        SVD kernel shape selection (see include/pgsvt.h).
    """

    def __init__(self, trajectory_length=15, patch_size=4, patch_overlap=1,
                 motion_estimation=True, motion_window=7, motion_filter=5,
                 optimize_pgure=True, lambda1=None, exponential_weighting=True,
                 noise_method=4, noise_alpha=None, noise_mu=None, noise_sigma=None,
                 tol=1e-7, max_iter=500, n_jobs=None, random_seed=None, *,
                 compat_flags=_capi.COMPAT_ALL, search_points=8, search_rounds=4,
                 lambda_hint=None, window_batch=0, verbose=False, learned_lambda=False,
                 lambda_model=None, autotune=0):
        self.trajectory_length = trajectory_length
        self.patch_size = patch_size
        self.patch_overlap = patch_overlap
        self.motion_estimation = motion_estimation
        self.motion_window = motion_window
        self.motion_filter = motion_filter
        self.optimize_pgure = optimize_pgure
        self.lambda1 = lambda1
        self.exponential_weighting = exponential_weighting
        self.noise_method = noise_method
        self.noise_alpha = noise_alpha
        self.noise_mu = noise_mu
        self.noise_sigma = noise_sigma
        self.tol = tol
        self.max_iter = max_iter
        self.n_jobs = n_jobs
        self.random_seed = random_seed
        self.compat_flags = compat_flags
        self.search_points = search_points
        self.search_rounds = search_rounds
        self.lambda_hint = lambda_hint
        self.window_batch = window_batch
        self.verbose = verbose
        self.learned_lambda = learned_lambda
        self.lambda_model = lambda_model
        self.autotune = autotune
        self.Y_ = None
        self._model = None

    def _check_arguments(self, X):
        """Sanity-checking of arguments (pguresvt/svt.py:212-271)."""
        if X.min() < 0.0:
            raise ValueError(
                "Negative values found in data. PGURE-SVT "
                "requires strictly non-negative image data."
            )
        self.lambda1_ = -1 if self.lambda1 is None else self.lambda1
        self.motion_filter_ = -1 if self.motion_filter is None else self.motion_filter
        self.noise_alpha_ = -1 if self.noise_alpha is None else self.noise_alpha
        self.noise_mu_ = -1 if self.noise_mu is None else self.noise_mu
        self.noise_sigma_ = -1 if self.noise_sigma is None else self.noise_sigma
        self.n_jobs_ = -1 if self.n_jobs is None else self.n_jobs
        self.random_seed_ = -1 if self.random_seed is None else self.random_seed

        if self.patch_overlap > self.patch_size:
            raise ValueError(
                f"Invalid patch_overlap parameter: got {self.patch_overlap}, "
                f"should not be greater than patch_size ({self.patch_size})"
            )
        if self.trajectory_length % 2 == 0 or self.trajectory_length < 1:
            raise ValueError(
                f"Invalid trajectory_length parameter: got {self.trajectory_length},"
                "but expected a positive, odd-valued integer"
            )
        if self.motion_estimation:
            if self.motion_window < 2 or self.motion_window % 2 == 0:
                raise ValueError(
                    f"Invalid motion_window parameter: got {self.motion_window}, "
                    "should be greater a positive, odd-valued integer > 1 pixel."
                )
            if not isinstance(self.motion_filter_, int):
                raise ValueError(
                    f"Invalid motion_filter parameter: got {type(self.motion_filter)}, "
                    "should be an integer number of pixels or None."
                )
        if not self.optimize_pgure and (self.lambda1 is None or self.lambda1 < 0.0):
            raise ValueError(
                f"Invalid lambda1 parameter: got {self.lambda1}, "
                "should be a float >= 0.0 if optimize_pgure is None."
            )
        if any(v < 0.0 for v in [self.noise_alpha_, self.noise_mu_, self.noise_sigma_]):
            if X.shape[0] != X.shape[1]:
                raise ValueError(
                    f"Quadtree noise estimation requires square images, got {X.shape}"
                )
            if not _is_power_of_two(X.shape[0]):
                raise ValueError("Quadtree noise estimation requires image dimensions 2^N")

    def _model_array(self):
        """The learned model in use (kept alive on the estimator), or None."""
        if self.lambda_model is not None:
            m = np.ascontiguousarray(self.lambda_model, dtype=np.float32)
        elif self.learned_lambda:
            from . import learned
            if self.patch_size != 4 or self.trajectory_length != 15:
                raise ValueError("the shipped lambda model covers patch_size 4 and "
                                 "trajectory_length 15; pass lambda_model= for others")
            m = learned.load_model()
        else:
            return None
        if m.size != _capi.LAMBDA_MODEL_FLOATS:
            raise ValueError("lambda model has %d floats, expected %d"
                             % (m.size, _capi.LAMBDA_MODEL_FLOATS))
        self._model = m
        return m

    def params(self):
        """The pgsvt_params this estimator passes to the library."""
        model = self._model_array()
        return _capi.default_params(
            lambda_model=0 if model is None else model.ctypes.data,
            autotune=int(self.autotune),
            traj_length=self.trajectory_length, block_size=self.patch_size,
            block_overlap=self.patch_overlap, motion_window=self.motion_window,
            median_size=self.motion_filter_, noise_method=self.noise_method,
            max_iter=self.max_iter, n_jobs=self.n_jobs_, random_seed=self.random_seed_,
            optimize_pgure=int(bool(self.optimize_pgure)),
            exp_weighting=int(bool(self.exponential_weighting)),
            motion_estimation=int(bool(self.motion_estimation)),
            verbose=int(bool(self.verbose)), lambda_=float(self.lambda1_),
            alpha=float(self.noise_alpha_), mu=float(self.noise_mu_),
            sigma=float(self.noise_sigma_), tol=float(self.tol),
            compat_flags=self.compat_flags, search_points=self.search_points,
            search_rounds=self.search_rounds, window_batch=self.window_batch,
            lambda_hint=-1.0 if self.lambda_hint is None else float(self.lambda_hint),
        )

    def denoise(self, X):
        """Denoise the data X, shape (nx, ny, nt) (pguresvt/svt.py:273-337)."""
        self._check_arguments(X)
        X_dtype = getattr(X, "dtype", None)
        if X_dtype not in _capi.DTYPES:
            raise TypeError(
                f"Invalid dtype: got {X_dtype}, but only {list(_capi.DTYPES.keys())} are supported"
            )
        if not X.flags.f_contiguous:
            X = np.asfortranarray(X, dtype=X_dtype)
        Y, est, st = _capi.denoise(X, self.params())
        self.Y_ = np.ascontiguousarray(Y)
        self.lambda1s_ = est[:, 0].copy()
        self.noise_alphas_ = est[:, 1].copy()
        self.noise_mus_ = est[:, 2].copy()
        self.noise_sigmas_ = est[:, 3].copy()
        self.status_ = st
        return self
