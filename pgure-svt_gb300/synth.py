"""Seeded synthetic image sequences standing in for microscopy data.

The reference measures on no public dataset (its nanoparticle sequence is
not distributed); these generators build sequences with the shapes, value
ranges and noise model of the benchmark workloads:

* ``blobs``: a sum of isotropic Gaussian blobs (sigma 2-6 px, peak 20-200
  counts) on a 5-count background, translated every frame by a seeded drift
  (integer steps of at most 1 px, or sub-pixel steps of at most 2 px rendered
  exactly at the shifted position), optionally plus a 2-D sinusoidal lattice
  (period 6-10 px, amplitude 15% of the mean);
* ``poisson_gaussian``: y = alpha * Poisson(x / alpha) + N(mu, sigma^2).

``mixed_noise_model`` restates the reference's noise generator
(pguresvt/svt.py:14-74) with the same NumPy RandomState call sequence, so
its outputs match the reference's golden values.
"""
import numpy as np


def mixed_noise_model(X, alpha=1.0, mu=0.0, sigma=0.0, random_state=None):
    """Poisson-Gaussian noise as pguresvt.mixed_noise_model (svt.py:14-74)."""
    if alpha <= 0.0 or alpha > 1.0:
        raise ValueError("alpha should be in range [0, 1]")
    if sigma < 0.0:
        raise ValueError("sigma should be >= 0.0")
    if not isinstance(random_state, np.random.RandomState):
        random_state = np.random.RandomState(random_state)
    X = X.astype(float)
    Xmax = X.max()
    X /= Xmax
    Y = alpha * random_state.poisson(X / alpha) + mu + sigma * random_state.normal(size=X.shape)
    Y *= Xmax
    return Y


def _drift(rng, nt, max_step, integer):
    if integer:
        steps = rng.integers(-max_step, max_step + 1, size=(nt, 2)).astype(float)
    else:
        steps = rng.uniform(-max_step, max_step, size=(nt, 2))
    steps[0] = 0.0
    return np.cumsum(steps, axis=0)


def blobs(side, nt, nblobs, seed, max_step=1.0, integer_drift=True, lattice=False,
          background=5.0, frames=None):
    """Clean (side, side, nt) float64 sequence, column-major like the reference.

    Isotropic Gaussians are separable, so a frame is background +
    Gy diag(peak) Gx^T with Gy[y, b] = exp(-(y - cy_b)^2 / 2s_b^2) (same for x).
    `frames` (indices into the nt-frame sequence) renders only those frames,
    in that order, with the drift of the whole sequence; the lattice
    amplitude then follows the rendered frames' mean.
    """
    rng = np.random.default_rng(seed)
    cy = rng.uniform(0, side, nblobs)
    cx = rng.uniform(0, side, nblobs)
    sg = rng.uniform(2.0, 6.0, nblobs)
    pk = rng.uniform(20.0, 200.0, nblobs)
    off = _drift(rng, nt, max_step, integer_drift)
    r = np.arange(side, dtype=float)[:, None]
    ts = list(range(nt)) if frames is None else [int(t) for t in frames]
    X = np.empty((side, side, len(ts)), dtype=float, order="F")
    if lattice:
        period = rng.uniform(6.0, 10.0, 2)
        phase = rng.uniform(0, 2 * np.pi, 2)
    for n, t in enumerate(ts):
        dy, dx = off[t]
        gy = np.exp(-((r - cy[None, :] - dy) ** 2) / (2 * sg[None, :] ** 2))
        gx = np.exp(-((r - cx[None, :] - dx) ** 2) / (2 * sg[None, :] ** 2))
        X[:, :, n] = background + gy @ (pk[:, None] * gx.T)
    if lattice:
        amp = 0.15 * X.mean()
        for n, t in enumerate(ts):
            dy, dx = off[t]
            ly = np.sin(2 * np.pi * (r[:, 0] - dy) / period[0] + phase[0])
            lx = np.sin(2 * np.pi * (r[:, 0] - dx) / period[1] + phase[1])
            X[:, :, n] += amp * np.outer(ly, lx)
        np.maximum(X, 0.0, out=X)
    return X


def poisson_gaussian(X, alpha, mu, sigma, seed):
    """y = alpha * Poisson(x / alpha) + N(mu, sigma^2), clipped at 0."""
    rng = np.random.default_rng(seed)
    Y = alpha * rng.poisson(X / alpha) + rng.normal(mu, sigma, X.shape)
    return np.asfortranarray(np.maximum(Y, 0.0))


# The workloads (sizes, generators and noise) of the benchmark configurations.
WORKLOADS = {
    "plain_64": dict(side=64, nt=30, nblobs=12, max_step=1, integer_drift=True, lattice=False,
                     alpha=0.1, mu=0.0, sigma=1.0, dtype="float64"),
    "arps_256": dict(side=256, nt=100, nblobs=80, max_step=2.0, integer_drift=False,
                     lattice=False, alpha=0.2, mu=0.5, sigma=2.0, dtype="float32"),
    "lattice_512": dict(side=512, nt=200, nblobs=300, max_step=2.0, integer_drift=False,
                        lattice=True, alpha=0.5, mu=1.0, sigma=3.0, dtype="float32"),
}


def workload(name, seed=0, side=None, nt=None):
    """(noisy, clean, noise params) of a named workload, optionally resized."""
    w = dict(WORKLOADS[name])
    side = side or w["side"]
    nt = nt or w["nt"]
    nb = max(1, int(round(w["nblobs"] * (side / w["side"]) ** 2)))
    clean = blobs(side, nt, nb, seed, w["max_step"], w["integer_drift"], w["lattice"])
    noisy = poisson_gaussian(clean, w["alpha"], w["mu"], w["sigma"], seed + 1)
    return noisy.astype(w["dtype"], order="F"), clean, (w["alpha"], w["mu"], w["sigma"])
