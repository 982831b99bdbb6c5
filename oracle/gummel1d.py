"""Restatement of the RTD Gummel loop for the 1D path (oracle; test infrastructure).

Follows, for Ny = 1 and Dirichlet contacts:
  poisson_matrix     RTD/eval_Poisson2D_rtd.m:108-200 (harmonic-mean stencil)
  projection         RTD/project_DG_density_RTD.m:16-61 (exact DG integrals
                     over the dual control volumes)
  poisson_step       RTD/solve_Poisson2D_rtd.m:113-186 (approximate Newton,
                     local Boltzmann screening)
  gummel             RTD/solve2D_rtd_self_consistent.m:88-205 (mixing, unmixed
                     defect / density-change / residual convergence)
Transport is the oracle's direct solve (dg1d) or any callable with its result.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import dg1d

Q = 1.602176634e-19
KB = 1.380649e-23
EPS0 = 8.8541878128e-12


def poisson_matrix(x_nm, eps_r):
    nx = len(x_nm)
    dx = x_nm[1] - x_nm[0]
    cx = EPS0 * 1e18 / dx ** 2
    lo = np.zeros(nx); di = np.zeros(nx); up = np.zeros(nx)
    for i in range(1, nx - 1):
        e0 = eps_r[i]
        cm = cx * (2 * e0 * eps_r[i - 1] / (e0 + eps_r[i - 1]))
        cp = cx * (2 * e0 * eps_r[i + 1] / (e0 + eps_r[i + 1]))
        lo[i], di[i], up[i] = cm, -(cm + cp), cp
    return lo, di, up


def projection(x_nm, p):
    """T (nx x n_el*nK) with T @ n_dg = control-volume averages."""
    x = np.asarray(x_nm, dtype=float)
    nx = len(x)
    n_el, nK = p["N_chi"], p["N_K_chi"]
    r = p["r"]
    edges = np.concatenate(([x[0]], (x[:-1] + x[1:]) / 2, [x[-1]]))
    widths = np.diff(edges)
    nq = int(np.ceil(nK / 2))
    pts, wts = np.polynomial.legendre.leggauss(nq)
    T = np.zeros((nx, n_el * nK))
    for e in range(n_el):
        left, right = x[e * (nK - 1)], x[(e + 1) * (nK - 1)]
        jac = (right - left) / 2
        rows = np.nonzero((edges[:-1] < right) & (edges[1:] > left))[0]
        for row in rows:
            a, b = max(edges[row], left), min(edges[row + 1], right)
            sample = ((a + b) / 2 + (b - a) / 2 * pts - (left + right) / 2) / jac
            basis = np.ones((nq, nK))
            for j in range(nK):
                for k in range(nK):
                    if k != j:
                        basis[:, j] *= (sample - r[k]) / (r[j] - r[k])
            T[row, e * nK:(e + 1) * nK] = (b - a) / 2 * (wts @ basis)
    return T / widths[:, None]


def poisson_step(tri, n, nd, phi0, bias, temp):
    """One approximate-Newton update; returns (candidate, info)."""
    lo, di, up = tri
    nx = len(phi0)
    v = np.array(phi0, dtype=float)
    v[0], v[-1] = 0.0, bias
    free = np.arange(1, nx - 1)
    Av = lo[free] * v[free - 1] + di[free] * v[free] + up[free] * v[free + 1]
    charge = Q * (n - nd)
    F = Av - charge[free]
    scale = max(np.abs(Q * n[free]).max(), np.abs(Q * nd[free]).max(), np.abs(Av).max(), Q)
    g = Q ** 2 * n[free] / (KB * temp)
    J = sp.diags([lo[free][1:], di[free] - g, up[free][:-1]], [-1, 0, 1], format="csc")
    delta = -spla.spsolve(J, F)
    lin = np.abs(J @ delta + F).max() / max(np.abs(F).max(), Q)
    cand = v.copy()
    cand[free] = v[free] + delta
    return cand, {"converged": bool(np.all(np.isfinite(cand)) and lin < 1e-8), "linear_relres": lin,
                  "physical_relres_before": np.abs(F).max() / scale}


def gummel(mat, bias, phi0, *, dy_nm, ef_offset=0.05, mixing=0.1, potential_tol=5e-4, density_tol=5e-4,
           poisson_residual_tol=8e-2, max_iterations=100, transport=None):
    """Fixed point of solve2D_rtd_self_consistent.m:104-187 for one bias."""
    vc = np.asarray(mat["Vc"], dtype=float)
    nd = np.asarray(mat["Nd"], dtype=float)
    x = np.asarray(mat["x"], dtype=float)
    m = np.full(mat["Nx"], float(np.asarray(mat["me_x"]).ravel()[0]) * dg1d.M0_V)
    tri = poisson_matrix(x, np.asarray(mat["eps"], dtype=float))
    phi = np.array(phi0, dtype=float)
    prev = None
    hist = []
    status = "iteration-limit"
    out = None
    for it in range(1, max_iterations + 1):
        V = vc - phi
        efl = vc[0] + ef_offset
        efr = vc[-1] + ef_offset - bias
        p = dg1d.init_params(mat, efl, efr, V, m)
        if transport is None:
            A, rhs = dg1d.get_sysm(mat, p, V)
            rho = spla.spsolve(A.tocsc(), rhs)
        else:
            rho = transport(mat, p, V)
        n_dg, j, _ = dg1d.observables(p, rho, dg1d.node_map(p, m))
        n_dg = n_dg / (dy_nm * 1e-9)
        T = projection(x, p)
        n_cv = T @ n_dg
        dchange = np.inf if prev is None else \
            np.linalg.norm(n_dg - prev) / max(np.linalg.norm(n_dg), np.linalg.norm(prev), np.finfo(float).tiny)
        cand, info = poisson_step(tri, n_cv, nd, phi, bias, float(mat["Temp"]))
        defect = np.abs(cand - phi).max()
        hist.append({"defect": defect, "density_change": dchange, "poisson_relres": info["physical_relres_before"]})
        out = {"phi": phi.copy(), "n": n_dg, "j": j, "rho": rho, "V": V}
        if not info["converged"]:
            status = "poisson-not-converged"
            break
        if defect <= potential_tol and dchange <= density_tol and info["physical_relres_before"] <= poisson_residual_tol:
            status = "fixed-point-converged"
            break
        if it == max_iterations:
            break
        prev = n_dg
        phi = phi + mixing * (cand - phi)
    out.update(status=status, iterations=len(hist), history=hist)
    return out
