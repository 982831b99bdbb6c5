"""Nodal-DG reference-element utilities (oracle; test infrastructure only).

Restates the Hesthaven-Warburton helpers the reference carries in
DG_code/core/: JacobiGQ.m:1-30, JacobiGL.m:1-32, JacobiP.m:1-39,
Vandermonde1D.m:1-10, GradJacobiP.m:1-14, GradVandermonde1D.m:1-12,
Dmatrix1D.m:1-9.
"""
import math

import numpy as np


def jacobi_gq(alpha, beta, n):
    """Gauss quadrature of order n for the Jacobi weight (JacobiGQ.m:1-30)."""
    if n == 0:
        return np.array([-(alpha - beta) / (alpha + beta + 2.0)]), np.array([2.0])
    h1 = 2.0 * np.arange(n + 1) + alpha + beta
    with np.errstate(divide="ignore", invalid="ignore"):
        main = -0.5 * (alpha ** 2 - beta ** 2) / (h1 + 2.0) / h1
    i = np.arange(1, n + 1, dtype=float)
    off = 2.0 / (h1[:n] + 2.0) * np.sqrt(
        i * (i + alpha + beta) * (i + alpha) * (i + beta) / (h1[:n] + 1.0) / (h1[:n] + 3.0))
    if alpha + beta < 10 * np.finfo(float).eps:
        main[0] = 0.0
    J = np.diag(main) + np.diag(off, 1)
    J = J + J.T
    d, v = np.linalg.eigh(J)
    w = v[0, :] ** 2 * 2 ** (alpha + beta + 1) / (alpha + beta + 1) * math.gamma(alpha + 1) \
        * math.gamma(beta + 1) / math.gamma(alpha + beta + 1)
    return d, w


def legendre_p(n, x):
    """Legendre polynomial P_n(x) by the three-term recurrence."""
    p0, p1 = 1.0, x
    if n == 0:
        return p0
    for k in range(1, n):
        p0, p1 = p1, ((2 * k + 1) * x * p1 - k * p0) / (k + 1)
    return p1


def jacobi_gl(alpha, beta, n):
    """Gauss-Lobatto nodes and weights of order n (JacobiGL.m:1-32).

    The weights use w_i = 2 / (n (n+1) P_n(x_i)^2), evaluated on the first half
    of the nodes and mirrored, as the reference does.
    """
    if n == 0:
        return np.array([0.0]), np.array([2.0])
    if n == 1:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    xint, _ = jacobi_gq(alpha + 1, beta + 1, n - 2)
    x = np.concatenate(([-1.0], xint, [1.0]))
    m = n + 1
    w = np.zeros(m)
    for i in range(int(math.ceil(m / 2))):
        w[i] = 2.0 / (m * (m - 1)) / legendre_p(m - 1, x[i]) ** 2
        w[m - 1 - i] = w[i]
    return x, w


def jacobi_p(x, alpha, beta, n):
    """Orthonormal Jacobi polynomial of order n at x (JacobiP.m:1-39)."""
    xp = np.asarray(x, dtype=float).ravel()
    gamma0 = 2 ** (alpha + beta + 1) / (alpha + beta + 1) * math.gamma(alpha + 1) \
        * math.gamma(beta + 1) / math.gamma(alpha + beta + 1)
    pl = np.zeros((n + 1, xp.size))
    pl[0] = 1.0 / math.sqrt(gamma0)
    if n == 0:
        return pl[0].copy()
    gamma1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * gamma0
    pl[1] = ((alpha + beta + 2) * xp / 2 + (alpha - beta) / 2) / math.sqrt(gamma1)
    if n == 1:
        return pl[1].copy()
    aold = 2 / (2 + alpha + beta) * math.sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3))
    for i in range(1, n):
        h1 = 2 * i + alpha + beta
        anew = 2 / (h1 + 2) * math.sqrt((i + 1) * (i + 1 + alpha + beta) * (i + 1 + alpha)
                                        * (i + 1 + beta) / (h1 + 1) / (h1 + 3))
        bnew = -(alpha ** 2 - beta ** 2) / h1 / (h1 + 2)
        pl[i + 1] = 1 / anew * (-aold * pl[i - 1] + (xp - bnew) * pl[i])
        aold = anew
    return pl[n].copy()


def vandermonde1d(n, r):
    """V_ij = P_j(r_i) (Vandermonde1D.m:1-10)."""
    r = np.asarray(r, dtype=float).ravel()
    v = np.zeros((r.size, n + 1))
    for j in range(n + 1):
        v[:, j] = jacobi_p(r, 0, 0, j)
    return v


def grad_jacobi_p(r, alpha, beta, n):
    """d/dr of the orthonormal Jacobi polynomial (GradJacobiP.m:1-14)."""
    r = np.asarray(r, dtype=float).ravel()
    if n == 0:
        return np.zeros(r.size)
    return math.sqrt(n * (n + alpha + beta + 1)) * jacobi_p(r, alpha + 1, beta + 1, n - 1)


def grad_vandermonde1d(n, r):
    """Gradient Vandermonde matrix (GradVandermonde1D.m:1-12)."""
    r = np.asarray(r, dtype=float).ravel()
    dv = np.zeros((r.size, n + 1))
    for i in range(n + 1):
        dv[:, i] = grad_jacobi_p(r, 0, 0, i)
    return dv


def dmatrix1d(n, r, v):
    """Differentiation matrix Dr = Vr / V (Dmatrix1D.m:1-9)."""
    vr = grad_vandermonde1d(n, r)
    return np.linalg.solve(v.T, vr.T).T
