"""GPU parity of the FP64 path against the oracle, through the C ABI.

Tolerances: operator apply / rhs / preconditioner 1e-12 relative (FP64,
different summation order); solution, density and current against the
oracle's sparse LU: density <= 1e-9, current <= 1e-8 relative L2 (the parity
bar of the plain form), with GMRES run to a 1e-12 relative residual.  The same
bars hold with the FP64 transforms emulated on the tensor cores (fp64_tc).
"""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from conftest import small_rtd
from oracle import dg1d, krylov

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "wigner1d_golden.npz")


@pytest.fixture(scope="module")
def lib(built_lib):
    from real_space_dg_gb300 import _lib
    return _lib.load()


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def det_vec(n):
    i = np.arange(1, n + 1, dtype=float)
    return np.sin(i) + 1j * np.cos(i)


def make_problem(spec, batch=1, **kw):
    from real_space_dg_gb300 import Problem1D
    return Problem1D(n_el=spec.n_el, n_local=spec.n_local, nk=spec.nk, n_xi=spec.n_xi or spec.nk,
                     l_xi=spec.l_xi_m, batch=batch, **kw)


CASES = [(12, 32, 2, 0), (10, 16, 1, 20), (8, 24, 3, 0), (9, 20, 2, 26)]


@pytest.mark.parametrize("fp64_tc", [False, True])
@pytest.mark.parametrize("n_el,nk,order,nxi", CASES)
def test_apply_rhs_precond_match_oracle(lib, n_el, nk, order, nxi, fp64_tc):
    spec, mat, E, efl, efr, m = small_rtd(n_el=n_el, nk=nk, order=order, n_xi=nxi)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    op = krylov.Operator1D(mat, p, E)
    pre = krylov.KLinePreconditioner(op, use_drift_diag=False)
    with make_problem(spec, fp64_tc=fp64_tc) as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        x = det_vec(P.N)
        assert rel(P.apply(x), A @ x) < 1e-12
        assert rel(P.rhs(), rhs) < 1e-12
        assert rel(P.precondition(x), pre.apply(x)) < 1e-12


@pytest.mark.parametrize("fp64_tc", [False, True])
@pytest.mark.parametrize("n_el,nk,order,nxi", CASES)
def test_solve_matches_direct_solve(lib, n_el, nk, order, nxi, fp64_tc):
    spec, mat, E, efl, efr, m = small_rtd(n_el=n_el, nk=nk, order=order, n_xi=nxi)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    ref = spla.spsolve(A.tocsc(), rhs)
    n_ref, j_ref, ru_ref = dg1d.observables(p, ref, dg1d.node_map(p, m))
    with make_problem(spec, fp64_tc=fp64_tc) as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        st, info = P.solve(tol=1e-12, maxit=60)
        assert st == 0 and info[0]["flag"] == 0 and info[0]["relres"] <= 1e-12
        n, j = P.observables(0)
        assert rel(P.rho(0), ref) < 1e-9
        assert rel(n, n_ref) < 1e-9
        assert rel(j, j_ref) < 1e-8
        assert rel(P.rho_xi(0), ru_ref.T) < 1e-9


def test_golden_fixtures_on_gpu(lib):
    g = np.load(GOLDEN)
    from golden.make_golden import CASES as GC
    from real_space_dg_gb300 import devices
    for name, (n_el, nk, order, nxi, bias) in GC.items():
        spec, mat, E, efl, efr, m = small_rtd(n_el=n_el, nk=nk, order=order, n_xi=nxi, bias=bias)
        with make_problem(spec) as P:
            P.set_potential(0, g[name + "/x_nm"], g[name + "/E"], g[name + "/m"], spec.m_rel, spec.temp_k,
                            float(g[name + "/efl"]), float(g[name + "/efr"]))
            assert rel(P.apply(det_vec(P.N)), g[name + "/Ax"]) < 1e-12
            assert rel(P.rhs(), g[name + "/rhs"]) < 1e-12
            P.solve(tol=1e-12, maxit=60)
            n, j = P.observables(0)
            assert rel(P.rho(0), g[name + "/rho"]) < 1e-9
            assert rel(n, g[name + "/n_dg"]) < 1e-9
            assert rel(j, g[name + "/j"]) < 1e-8


def test_batch_of_different_devices_is_independent(lib):
    """Three problems with different biases and lengths in one handle give the
    same answer as each alone."""
    specs = []
    for bias, length in [(0.0, 30.0), (0.15, 30.0), (0.3, 34.0)]:
        specs.append(small_rtd(n_el=10, nk=24, order=2, bias=bias, length_nm=length))
    spec0 = specs[0][0]
    with make_problem(spec0, batch=3) as P:
        for b, (spec, mat, E, efl, efr, m) in enumerate(specs):
            P.set_potential(b, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        x = np.concatenate([det_vec(P.N) * (b + 1) for b in range(3)])
        y = P.apply(x)
        st, info = P.solve(tol=1e-12, maxit=60)
        assert st == 0
        for b, (spec, mat, E, efl, efr, m) in enumerate(specs):
            p = dg1d.init_params(mat, efl, efr, E, m)
            A, rhs = dg1d.get_sysm(mat, p, E)
            assert rel(y[b * P.N:(b + 1) * P.N], A @ x[b * P.N:(b + 1) * P.N]) < 1e-12
            assert rel(P.rho(b), spla.spsolve(A.tocsc(), rhs)) < 1e-9


def test_solve_transport_mirror_matches_oracle(lib):
    from real_space_dg_gb300 import solve_transport_DG_2D
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=24, order=2)
    Vsub = np.ones(mat["Nx"])
    ref = dg1d.solve_transport_dg_2d(mat, E, Vsub, efl, efr)
    out = solve_transport_DG_2D(mat, E, Vsub, efl, efr, tol=1e-12, maxit=60)
    assert out["info"][0]["flag"] == 0
    assert rel(out["n"], ref["n"]) < 1e-9
    assert rel(out["j"], ref["j"]) < 1e-8
    assert rel(out["RHO"], ref["RHO"]) < 1e-9
    assert np.allclose(out["chi"], ref["chi"], rtol=1e-14) and np.allclose(out["xi"], ref["xi"], rtol=1e-14)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-12)])
def test_multi_subband_fet_matches_oracle(lib, precision, tol):
    """Two valley types x two modes of a small gated FET through the drop-in: every
    subband is one problem of the batch, n sums the |Vsub|^2-weighted mode densities
    and j the mode currents (solve_transport_DG_2D.m:47-212)."""
    from real_space_dg_gb300 import devices, solve_transport_DG_2D
    spec = devices.FETSpec(length_nm=20.0, sd_nm=6.0, n_el=16, order=2, nk=32, n_modes=2, l_xi_m=12e-9)
    mat, esub, vsub, efl, efr = devices.make_fet(spec, 0.3, 0.2)
    ref = dg1d.solve_transport_dg_2d(mat, esub, vsub, efl, efr)
    out = solve_transport_DG_2D(mat, esub, vsub, efl, efr, tol=tol, maxit=80, precision=precision)
    assert all(i["flag"] == 0 for i in out["info"]), out["info"]
    assert out["RHO"].shape == (2, 2, spec.n_el * spec.n_local, spec.nk)
    assert rel(out["n"], ref["n"]) < 1e-9
    assert rel(out["j"], ref["j"]) < 1e-8
    assert rel(out["RHO"], ref["RHO"]) < 1e-9


def test_warm_start_and_statuses(lib):
    from real_space_dg_gb300 import WignerError, _lib
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=24, order=2)
    with make_problem(spec) as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        st, info = P.solve(tol=1e-12, maxit=60)
        rho = P.rho(0)
        # warm start from the solution: converged at start, zero iterations
        st, info = P.solve(tol=1e-10, maxit=60, rho0=rho)
        assert st == 0 and info[0]["iterations"] == 0 and info[0]["initial_relres"] <= 1e-10
        # forced non-convergence is a status, not an error (iterativeStatus)
        st, info = P.solve(tol=1e-14, maxit=1)
        assert st == _lib.WG_NOT_CONVERGED and info[0]["flag"] == 1
        # non-finite warm start is rejected before any device work (InvalidInitialRho)
        bad = rho.copy(); bad[3] = np.nan
        with pytest.raises(WignerError) as e:
            P.solve(rho0=bad)
        assert e.value.status == _lib.WG_ERR_ARG
        with pytest.raises(WignerError):
            P.set_potential(0, mat["x"][:-1], E[:-1], m[:-1], spec.m_rel, spec.temp_k, efl, efr)
        E2 = E.copy(); E2[5] = np.inf
        with pytest.raises(WignerError):
            P.set_potential(0, mat["x"], E2, m, spec.m_rel, spec.temp_k, efl, efr)
