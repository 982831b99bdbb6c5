"""Transient self-consistent solve (bias step, RK4 and Crank-Nicolson).

CPU: the oracle's Crank-Nicolson and the reference's RK4 agree to second order
in dt, and Crank-Nicolson with a fixed potential settles on the stationary
solution A^-1 rhs.

GPU: every transient starts from the device's own stationary state (its Wigner
function and potential after wg_gummel_run), which the oracle then integrates
too.  Tolerances on the n and j histories: RK4 (explicit, operator applies
only) 1e-9 relative; Crank-Nicolson with 1e-12 step solves 1e-8; the mixed
form (1e-10 step solves through FP64 refinement) against the FP64 form 1e-7;
a transient alone and inside a batch 1e-12.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from conftest import small_rtd
from oracle import dg1d, gummel1d, transient1d


def _state(bias=0.05):
    from real_space_dg_gb300 import devices
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=32, order=2)
    dy = devices.density_normalisation_nm(mat)
    g = gummel1d.gummel(mat, bias, bias * mat["ramp"], dy_nm=dy, mixing=0.5, potential_tol=1e-7,
                        density_tol=1e-6, max_iterations=200)
    assert g["status"] == "fixed-point-converged"
    return mat, dy, g


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def test_oracle_cn_matches_rk4_to_second_order():
    mat, dy, g = _state()
    kw = dict(dy_nm=dy, scale_a=2e-10, scale_rhs=2e-10, refresh_every=5, refresh_first=8)
    errs = []
    for dt in (2e-17, 1e-17):
        nsteps = int(round(2.4e-16 / dt))
        a = transient1d.transient(mat, g["rho"], g["phi"], 0.15, dt, nsteps, method="rk4", **kw)
        b = transient1d.transient(mat, g["rho"], g["phi"], 0.15, dt, nsteps, method="cn", **kw)
        errs.append(rel(b["j"][-1], a["j"][-1]))
    assert errs[0] < 1e-4 and errs[1] < errs[0] / 3          # O(dt^2)


def test_oracle_cn_settles_on_the_stationary_solution():
    mat, dy, g = _state()
    r = transient1d.transient(mat, g["rho"], g["phi"], 0.15, 1e-15, 1500, dy_nm=dy, scale_a=2e-10,
                              scale_rhs=2e-10, refresh_every=0, record_every=0)
    vc = np.asarray(mat["Vc"], dtype=float)
    m = np.full(mat["Nx"], float(np.asarray(mat["me_x"]).ravel()[0]) * dg1d.M0_V)
    V = vc - r["phi"]
    p = dg1d.init_params(mat, vc[0] + 0.05, vc[-1] + 0.05 - 0.15, V, m)
    A, rhs = dg1d.get_sysm(mat, p, V)
    assert rel(r["rho"], spla.spsolve(A.tocsc(), rhs)) < 1e-8


def _gpu_sweep(mat, dy, batch, precision="fp64"):
    from real_space_dg_gb300.rtd import RTDSweep
    S = RTDSweep(dict(mat, dy_norm_nm=dy), batch,
                 dict(mixing=0.5, potentialTolerance=1e-7, densityTolerance=1e-6, maxIterations=200,
                      transportTolerance=1e-12, transportMaxCycles=60, precision=precision))
    for b in range(batch):
        S.set(b, 0.05)
    st, info = S.run()
    assert st == 0, info
    return S


@pytest.mark.gpu
@pytest.mark.parametrize("method,dt,tol", [("rk4", 2e-17, 1e-9), ("cn", 1e-15, 1e-8)])
def test_transient_matches_oracle(built_lib, method, dt, tol):
    mat, dy, _ = _state()
    S = _gpu_sweep(mat, dy, 1)
    try:
        rho0 = S.P.rho(0)
        phi0 = S.get(0)[0]
        S.step_bias(0, 0.15)
        st, info, n, j = S.transient(dt, 12, method, scale_a=2e-10, refresh_every=5, refresh_first=8, tol=1e-12,
                                     maxit=40)
    finally:
        S.close()
    # re-solves: the bias step, after t = 1..7 (t < F) and after t = 10 (t % E == 0)
    assert st == 0 and info[0]["steps"] == 12 and info[0]["poisson_solves"] == 1 + 8
    ref = transient1d.transient(mat, rho0, phi0, 0.15, dt, 12, dy_nm=dy, method=method, scale_a=2e-10,
                                scale_rhs=2e-10, refresh_every=5, refresh_first=8)
    for t in range(12):
        assert rel(n[t, 0], ref["n"][t]) < tol, t
        assert rel(j[t, 0], ref["j"][t]) < tol, t


@pytest.mark.gpu
def test_mixed_transient_matches_fp64_and_batch_independence(built_lib):
    mat, dy, _ = _state()
    out = {}
    for precision, batch in (("fp64", 2), ("mixed", 2), ("fp64", 1)):
        S = _gpu_sweep(mat, dy, batch, precision)
        try:
            steps = [0.15, 0.1][:batch]
            for b, v in enumerate(steps):
                S.step_bias(b, v)
            st, info, n, j = S.transient(1e-15, 10, "cn", refresh_every=2, refresh_first=4, tol=1e-10, maxit=40)
        finally:
            S.close()
        assert st == 0, info
        out[(precision, batch)] = (n, j)
    n64, j64 = out[("fp64", 2)]
    nmx, jmx = out[("mixed", 2)]
    assert rel(nmx, n64) < 1e-7 and rel(jmx, j64) < 1e-7
    n1, j1 = out[("fp64", 1)]
    assert rel(n1[:, 0], n64[:, 0]) < 1e-12 and rel(j1[:, 0], j64[:, 0]) < 1e-12


@pytest.mark.gpu
def test_transient_dropin_from_init_matches_oracle(built_lib):
    """solve_transport_DG_2D_transient_SC_new(mat, INIT): the caller's INIT (rho, the fixed
    rhs_INIT, V_total) integrated with the reference's RK4 and refresh schedule; n and j after
    every step, the record strides 1:50:end / 1:5:end and the final rho against the oracle
    with the same fixed right-hand side (1e-9)."""
    from real_space_dg_gb300.rtd import solve_transport_DG_2D_transient_SC_new
    mat, dy, g = _state()
    vc = np.asarray(mat["Vc"], dtype=float)
    m = np.full(mat["Nx"], float(np.asarray(mat["me_x"]).ravel()[0]) * dg1d.M0_V)
    V = vc - g["phi"]
    p = dg1d.init_params(mat, vc[0] + 0.05, vc[-1] + 0.05 - 0.05, V, m)
    _, rhs = dg1d.get_sysm(mat, p, V)
    INIT = dict(rho=[g["rho"]], rhs=[2e-10 * rhs], V_total=-g["phi"], bias=0.05, Ef0=vc[0] + 0.05)
    nt, dt = 60, 2e-17
    mat2 = dict(mat, dy_norm_nm=dy, Nt=nt, dt=dt, Vd=0.15)
    DG = solve_transport_DG_2D_transient_SC_new(mat2, INIT, transient=dict(refreshEvery=5, refreshFirst=8))
    ref = transient1d.transient(mat, g["rho"], g["phi"], 0.15, dt, nt, dy_nm=dy, method="rk4", scale_a=2e-10,
                                scale_rhs=1.0, refresh_every=5, refresh_first=8, fixed_rhs=2e-10 * rhs)
    assert DG["status"] == 0 and DG["info"]["steps"] == nt
    for t in range(nt):
        assert rel(DG["n_all"][:, t], ref["n"][t]) < 1e-9, t
        assert rel(DG["j_all"][:, t], ref["j"][t]) < 1e-9, t
    assert DG["n_over_t"].shape == (ref["n"].shape[1], 1, 2) and DG["j_over_t"].shape == (ref["j"].shape[1], 12)
    assert np.array_equal(DG["n_over_t"][:, 0, 1], DG["n_all"][:, 50])
    assert np.array_equal(DG["j_over_t"][:, 3], DG["j_all"][:, 15])
    assert rel(DG["rho_INIT"][0], ref["rho"]) < 1e-9
