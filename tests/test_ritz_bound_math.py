"""The early pass exit's residual bound, restated in numpy (CPU only).

During a Lanczos pass the GPU check (k_ritz_bound) takes theta, the smallest
eigenvalue of the pass's tridiagonal matrix T_k, the last entry y_k of its
normalised eigenvector from the bottom twist of T_k - theta I (the pivots
d_i of its LDL^T factorisation, then z_(k-1) = 1, z_i = -e_i z_(i+1) / d_i
and y_k = |z_(k-1)| / |z|), and ends a group's pass once |b_k y_k| (b_k the
next off-diagonal) is below a fraction of rsb_tol.  These tests check the
restated steps against numpy's symmetric eigensolver, and the bound against
the true residual |L x - theta x| of the Ritz vector x = V_k y on an
orthonormal Lanczos basis, for the dual-graph Laplacian of a small hex box
(weights 4 / 2 / 1 for a shared face / edge / corner).
"""
import numpy as np
import pytest


def box_laplacian(nx, ny, nz):
    """Dual-graph Laplacian of an nx x ny x nz hex box: w = shared vertices."""
    idx = np.arange(nx * ny * nz).reshape(nz, ny, nx)
    n = idx.size
    L = np.zeros((n, n))
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                if dx == dy == dz == 0:
                    continue
                w = 2 ** (3 - abs(dx) - abs(dy) - abs(dz))  # 4 face, 2 edge, 1 corner
                src = idx[max(0, -dz):nz - max(0, dz), max(0, -dy):ny - max(0, dy),
                          max(0, -dx):nx - max(0, dx)]
                dst = idx[max(0, dz):nz - max(0, -dz), max(0, dy):ny - max(0, -dy),
                          max(0, dx):nx - max(0, -dx)]
                L[src.ravel(), dst.ravel()] -= w
    L[np.diag_indices(n)] = -L.sum(axis=1)
    return L


def lanczos(A, v0, k):
    """k steps with full reorthogonalisation: basis V (k + 1 rows), T's
    diagonal a and off-diagonals b (b[k-1] couples step k to the next)."""
    n = len(v0)
    V = np.zeros((k + 1, n))
    a, b = np.zeros(k), np.zeros(k)
    V[0] = v0 / np.linalg.norm(v0)
    for j in range(k):
        w = A @ V[j]
        a[j] = V[j] @ w
        w = w - a[j] * V[j] - (b[j - 1] * V[j - 1] if j else 0.0)
        w -= V[:j + 1].T @ (V[:j + 1] @ w)
        b[j] = np.linalg.norm(w)
        V[j + 1] = w / b[j]
    return V, a, b


def bottom_twist(a, e, theta):
    """Pivots of LDL^T of T - theta I and |y_k| from the bottom twist."""
    k = len(a)
    d = np.empty(k)
    d[0] = a[0] - theta
    for i in range(1, k):
        d[i] = a[i] - theta - e[i - 1] ** 2 / d[i - 1]
    z = np.empty(k)
    z[-1] = 1.0
    for i in range(k - 2, -1, -1):
        z[i] = -e[i] * z[i + 1] / d[i]
    return d, abs(z[-1]) / np.linalg.norm(z)


@pytest.mark.parametrize("k", [4, 8, 16, 30])
def test_bound_equals_ritz_residual(k):
    L = box_laplacian(9, 7, 6)
    rng = np.random.default_rng(5)
    v0 = rng.standard_normal(L.shape[0])
    v0 -= v0.mean()  # orthogonal to the constant vector, as every pass's start
    V, a, b = lanczos(L, v0, k)
    T = np.diag(a) + np.diag(b[:k - 1], 1) + np.diag(b[:k - 1], -1)
    lam, Y = np.linalg.eigh(T)
    theta, y = lam[0], Y[:, 0]
    d, yk = bottom_twist(a, b[:k - 1], theta)
    # the pivots above the last are positive for the smallest eigenvalue
    assert np.all(d[:-1] > 0)
    # the twisted vector's last entry is the eigenvector's
    assert yk == pytest.approx(abs(y[-1]), rel=1e-7, abs=1e-14)
    # and |b_k y_k| is the Ritz vector's residual
    x = V[:k].T @ y
    resid = np.linalg.norm(L @ x - theta * x)
    assert b[k - 1] * yk == pytest.approx(resid, rel=1e-6, abs=1e-12)


def test_bound_falls_with_the_steps():
    """The bound is what ends a pass: it decreases towards the tolerance
    along a pass, and the smallest Ritz value never grows (the check's warm
    multisection bracket [0.99 theta', theta'] relies on the latter)."""
    L = box_laplacian(12, 8, 6)
    rng = np.random.default_rng(9)
    v0 = rng.standard_normal(L.shape[0])
    v0 -= v0.mean()
    V, a, b = lanczos(L, v0, 60)
    bounds, thetas = [], []
    for k in range(3, 61, 3):
        T = np.diag(a[:k]) + np.diag(b[:k - 1], 1) + np.diag(b[:k - 1], -1)
        theta = np.linalg.eigvalsh(T)[0]
        _, yk = bottom_twist(a[:k], b[:k - 1], theta)
        bounds.append(b[k - 1] * yk)
        thetas.append(theta)
    assert all(t2 <= t1 * (1 + 1e-12) for t1, t2 in zip(thetas, thetas[1:]))
    assert bounds[-1] < 1e-3 * bounds[0]
