"""The SVD methods of the CUDA kernels, restated in numpy on the CPU (FP64).

These check the mathematics the kernels rely on, not the kernels themselves
(the -m gpu tests compare those with the oracle):

* one-sided Jacobi with the round-robin ordering the register form uses
  (pad column fixed at position NC-1, positions 0..NC-2 shifted by one per
  round) orthogonalises the columns: their norms are the singular values;
* the QR-preconditioned form (svd_split.cu): Jacobi on X = R^T, where
  B = Q R, gives the right singular vectors of B as the normalised rotated
  columns, and u = B v / s the left ones;
* the rotation from the half-angle identities (two reciprocal square roots)
  zeroes the pair's inner product.
"""
import numpy as np


def rotation(al, be, gv):
    """cos/sin of the pair rotation as svd_kernel.cuh computes them."""
    dd = be - al
    ir = 1.0 / np.sqrt(dd * dd + 4.0 * gv * gv)
    hh = 0.5 * abs(dd) * ir + 0.5
    rh = 1.0 / np.sqrt(hh)
    return hh * rh, (gv if dd >= 0 else -gv) * ir * rh


def round_robin_jacobi(A, tol=1e-12, max_sweeps=30):
    """One-sided Jacobi on the columns of A (NC even, last column zero)."""
    A = A.copy()
    nc = A.shape[1]
    pos = list(range(nc))
    for _ in range(max_sweeps):
        rotated = False
        for _ in range(nc - 1):
            for pp in range(1, nc // 2):
                i, j = pos[pp], pos[nc - 1 - pp]
                a, b = A[:, i].copy(), A[:, j].copy()
                al, be, gv = a @ a, b @ b, a @ b
                if gv * gv <= tol * tol * al * be:
                    continue
                cs, sn = rotation(al, be, gv)
                A[:, i], A[:, j] = cs * a - sn * b, sn * a + cs * b
                rotated = True
            pos = pos[1:nc - 1] + [pos[0]] + [pos[nc - 1]]
        if not rotated:
            break
    return A


def householder_r(B):
    """The triangle R of B = Q R by Householder reflections (as k_qr)."""
    B = B.copy()
    m, n = B.shape
    for jj in range(n):
        x = B[jj:, jj]
        ss = x @ x
        xj = B[jj, jj]
        alpha = -np.sqrt(ss) if xj >= 0 else np.sqrt(ss)
        vtv = 2.0 * (ss - xj * alpha)
        if vtv <= 0:
            continue
        v = x.copy()
        v[0] = xj - alpha
        beta = 2.0 / vtv
        B[jj:, jj + 1:] -= beta * np.outer(v, v @ B[jj:, jj + 1:])
        B[jj, jj] = alpha
        B[jj + 1:, jj] = 0.0
    return B[:n, :n]


def test_rotation_zeroes_the_inner_product():
    rng = np.random.default_rng(1)
    for _ in range(100):
        a, b = rng.standard_normal(16), rng.standard_normal(16)
        cs, sn = rotation(a @ a, b @ b, a @ b)
        assert abs(cs * cs + sn * sn - 1) < 1e-12
        na, nb = cs * a - sn * b, sn * a + cs * b
        assert abs(na @ nb) < 1e-12 * np.linalg.norm(na) * np.linalg.norm(nb)


def test_round_robin_jacobi_gives_the_singular_values():
    rng = np.random.default_rng(2)
    B = np.zeros((16, 16))
    B[:, :15] = rng.standard_normal((16, 15)) + 3.0 * rng.standard_normal(16)[:, None]
    A = round_robin_jacobi(B)
    G = A.T @ A
    off = G - np.diag(np.diag(G))
    assert np.abs(off).max() < 1e-10 * np.abs(G).max()
    s = np.sort(np.linalg.norm(A, axis=0))[::-1][:15]
    np.testing.assert_allclose(s, np.linalg.svd(B[:, :15], compute_uv=False), rtol=1e-10)


def test_qr_preconditioned_form_gives_the_factors():
    rng = np.random.default_rng(3)
    m, n = 64, 15  # an 8x8 patch over a 15-frame window
    B = rng.standard_normal((m, n)) + 5.0 * rng.standard_normal(m)[:, None]
    R = householder_r(B)
    np.testing.assert_allclose(R.T @ R, B.T @ B, rtol=1e-10, atol=1e-9)
    X = np.zeros((16, 16))
    X[:n, :n] = R.T  # column k of X = row k of R; pad column 15
    A = round_robin_jacobi(X)
    s = np.linalg.norm(A, axis=0)
    keep = np.argsort(-s)[:n]
    U_ref, s_ref, Vt_ref = np.linalg.svd(B, full_matrices=False)
    np.testing.assert_allclose(s[keep], s_ref, rtol=1e-10)
    for t, k in enumerate(keep):
        v = A[:n, k] / s[k]                 # right singular vector of B
        u = B @ v / s[k]                    # left one, from B itself
        assert abs(abs(v @ Vt_ref[t]) - 1) < 1e-8
        assert abs(abs(u @ U_ref[:, t]) - 1) < 1e-8
        np.testing.assert_allclose(B.T @ u, s[k] * v, atol=1e-9 * s_ref[0])
