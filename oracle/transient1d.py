"""Restatement of the transient self-consistent 1D Wigner solve (oracle; test infrastructure).

Follows DG_code/solve_transport_DG_2D_transient_SC_new.m:124-212 for one mode:
  - the state obeys d rho / dt = s_r rhs - s_A A rho; the reference scales A by
    2e-10 (:148) and uses the rhs handed over in INIT (:21, :153-156)
  - rk4_step: the reference's explicit Runge-Kutta step (:153-158)
  - the operator is rebuilt from the potential before step t when
    (t - 1) % E == 0 or t < F (:131-149, E = 20, F = 50)
  - the potential is re-solved after step t when t % E == 0 or t < F
    (:204-211) by the LINEAR Poisson problem of solve_Poisson2D_transient.m:
    A_poisson V = q (n - N_D) on the free nodes with Dirichlet contacts
  - n and j after every step (:161-185)
The 1D RTD electrostatics (band edge Vc, V = Vc - phi, contact Fermi levels
E_F = Vc + offset at the left and Vc + offset - bias at the right) are those of
RTD/solve2D_rtd_self_consistent.m:104-116, as in gummel1d.  A bias step at t = 0
re-solves the potential for the initial density with the new contact value and
rebuilds the operator and the inflow before the first step (the reference keeps
its INIT rhs, which holds the pre-step contacts; a drain-bias step has to
change the inflow).

cn_step is the Crank-Nicolson step of the GPU transient,
(I + dt/2 s_A A) rho' = (I - dt/2 s_A A) rho + dt s_r rhs, solved directly here.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import dg1d, gummel1d


def rk4_step(A, rhs, rho, dt, scale_a=1.0, scale_rhs=1.0):
    """solve_transport_DG_2D_transient_SC_new.m:153-158."""
    r = scale_rhs * rhs
    f = lambda u: r - scale_a * (A @ u)
    k1 = f(rho)
    k2 = f(rho + dt / 2 * k1)
    k3 = f(rho + dt / 2 * k2)
    k4 = f(rho + dt * k3)
    return rho + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)


def cn_step(A, rhs, rho, dt, scale_a=1.0, scale_rhs=1.0, lu=None):
    """(I + c A) rho' = (I - c A) rho + dt s_r rhs, c = dt s_A / 2."""
    c = dt * scale_a / 2
    n = A.shape[0]
    if lu is None:
        lu = spla.splu((sp.identity(n, dtype=complex, format="csc") + c * A).tocsc())
    b = rho - c * (A @ rho) + dt * scale_rhs * rhs
    return lu.solve(b), lu


def linear_poisson(tri, n_cv, nd, bias):
    """Linear Poisson of solve_Poisson2D_transient.m: A V = q (n - N_D), V(0) = 0, V(end) = bias."""
    lo, di, up = tri
    nx = len(n_cv)
    free = np.arange(1, nx - 1)
    rhs = gummel1d.Q * (n_cv[free] - nd[free])
    rhs[-1] -= up[nx - 2] * bias
    J = sp.diags([lo[free][1:], di[free], up[free][:-1]], [-1, 0, 1], format="csc")
    v = np.zeros(nx)
    v[-1] = bias
    v[free] = spla.spsolve(J, rhs)
    return v


def transient(mat, rho0, phi0, bias, dt, nsteps, *, dy_nm, ef_offset=0.05, method="cn", scale_a=1.0,
              scale_rhs=1.0, refresh_every=20, refresh_first=50, record_every=1, fixed_rhs=None):
    """Bias-step transient from the state (rho0, phi0) to `bias` at t = 0.  fixed_rhs: the
    reference's INIT.rhs, used at every step instead of the inflow of the rebuilt operator
    (solve_transport_DG_2D_transient_SC_new.m:21, 153-156).

    Returns dict(n=[nrec, ncol], j=[nrec, ncol], phi, rho, steps)."""
    vc = np.asarray(mat["Vc"], dtype=float)
    nd = np.asarray(mat["Nd"], dtype=float)
    x = np.asarray(mat["x"], dtype=float)
    m = np.full(mat["Nx"], float(np.asarray(mat["me_x"]).ravel()[0]) * dg1d.M0_V)
    tri = gummel1d.poisson_matrix(x, np.asarray(mat["eps"], dtype=float))
    efl = vc[0] + ef_offset
    efr = vc[-1] + ef_offset - bias
    rho = np.array(rho0, dtype=complex)
    phi = np.array(phi0, dtype=float)

    def build(phi):
        V = vc - phi
        p = dg1d.init_params(mat, efl, efr, V, m)
        A, rhs = dg1d.get_sysm(mat, p, V)
        return p, A.tocsc(), rhs

    def density(p, rho):
        n_dg, j, _ = dg1d.observables(p, rho, dg1d.node_map(p, m))
        return n_dg / (dy_nm * 1e-9), j

    # the bias step: potential for the initial density with the new contact value
    p, A, rhs = build(phi)
    n_dg, _ = density(p, rho)
    T = gummel1d.projection(x, p)
    phi = linear_poisson(tri, T @ n_dg, nd, bias)
    hist_n, hist_j = [], []
    lu = None
    for t in range(1, nsteps + 1):
        if t == 1 or (refresh_every > 0 and ((t - 1) % refresh_every == 0 or t < refresh_first)):
            p, A, rhs = build(phi)
            if fixed_rhs is not None:
                rhs = np.asarray(fixed_rhs, dtype=complex)
            lu = None
        if method == "rk4":
            rho = rk4_step(A, rhs, rho, dt, scale_a, scale_rhs)
        else:
            rho, lu = cn_step(A, rhs, rho, dt, scale_a, scale_rhs, lu)
        n_dg, j = density(p, rho)
        if record_every > 0 and t % record_every == 0:
            hist_n.append(n_dg)
            hist_j.append(j)
        if refresh_every > 0 and (t % refresh_every == 0 or t < refresh_first):
            phi = linear_poisson(tri, T @ n_dg, nd, bias)
    return {"n": np.array(hist_n), "j": np.array(hist_j), "phi": phi, "rho": rho, "steps": nsteps}
