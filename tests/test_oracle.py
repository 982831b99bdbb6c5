"""CPU tests of the oracle: the pins of the restatement (no GPU)."""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from conftest import small_rtd
from oracle import dg1d, jacobi, krylov

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "wigner1d_golden.npz")


# --- closed-form facts of the DG reference element ------------------------------------
def test_gauss_lobatto_known_values():
    x, w = jacobi.jacobi_gl(0, 0, 2)
    assert np.allclose(x, [-1, 0, 1], atol=1e-15) and np.allclose(w, [1 / 3, 4 / 3, 1 / 3], atol=1e-15)
    x, w = jacobi.jacobi_gl(0, 0, 3)
    assert np.allclose(x, [-1, -1 / np.sqrt(5), 1 / np.sqrt(5), 1], atol=1e-15)
    assert np.allclose(w, [1 / 6, 5 / 6, 5 / 6, 1 / 6], atol=1e-15)
    for n in (1, 2, 3, 4, 9):
        x, w = jacobi.jacobi_gl(0, 0, n)
        assert abs(w.sum() - 2) < 1e-14                 # JacobiGL.m:31 assertion
        # GL with n+1 points integrates degree 2n-1 exactly
        for d in range(2 * n):
            assert abs((w * x ** d).sum() - (2 / (d + 1) if d % 2 == 0 else 0)) < 1e-13


@pytest.mark.parametrize("nK", [2, 3, 4])
def test_mass_and_stiffness_identities(nK):
    r, _ = jacobi.jacobi_gl(0, 0, nK - 1)
    V = jacobi.vandermonde1d(nK - 1, r)
    M = np.linalg.inv(V).T @ np.linalg.inv(V)
    # M_ij = int l_i l_j over [-1,1]: exact 10-point GL quadrature of Lagrange products
    xq, wq = jacobi.jacobi_gl(0, 0, 9)
    W = np.linalg.solve(V.T, jacobi.vandermonde1d(nK - 1, xq).T).T
    assert np.allclose(M, (W * wq[:, None]).T @ W, atol=1e-14)
    Dr = jacobi.dmatrix1d(nK - 1, r, V)
    S = M @ Dr
    # summation-by-parts: S + S^T = diag(-1, 0, ..., 0, 1)
    B = np.zeros((nK, nK)); B[0, 0] = -1; B[-1, -1] = 1
    assert np.allclose(S + S.T, B, atol=1e-13)


def test_golden_gl_nodes():
    g = np.load(GOLDEN)
    for n in (1, 2, 3, 4, 9):
        x, w = jacobi.jacobi_gl(0, 0, n)
        assert np.array_equal(x, g["gl%d/x" % n]) and np.array_equal(w, g["gl%d/w" % n])


# --- the two reference assembly forms of the drift agree ------------------------------
def drift_by_index_tables(mat, p, EM):
    """Literal restatement of the reshape/index-table assembly of
    get_Drift_accel_trial_permutedShell.m:199-333 (hard-coded for N_K_chi=3,
    Nqx=10), with MATLAB column-major reshapes done by order='F'."""
    N_chi, NK, Ny = p["N_chi"], p["N_K_chi"], p["Nk"]
    assert NK == 3
    _, _, G = dg1d.get_drift(mat, p, EM, return_pages=True)     # G[i, j, m], i = (e, q)
    W = dg1d.interp_w(p)
    invM = dg1d.k_blocks(p)["invM"]
    C = G * np.tile(p["w"], N_chi)[:, None, None]                                 # :200
    W_rep = np.tile(np.tile(W, (N_chi, 1)), (Ny * Ny, 1))                        # :202-203
    C = W_rep * C.reshape(-1, order="F")[:, None]                                  # :204-209
    C = C.T.reshape((3, 10, -1), order="F")                                        # :212
    W_rep = W_rep.T.reshape((3, 10, -1), order="F").transpose(1, 0, 2)           # :213-214
    C = np.einsum("aqp,qbp->abp", C, W_rep)                                       # :215 pagemtimes
    C = C.transpose(1, 2, 0).reshape((NK * N_chi * Ny * Ny, NK), order="F")       # :216
    C = np.tile(p["Q_drift"] * invM, (1, N_chi * Ny * Ny)).T * C                  # :219
    # line index (:254-281)
    vspace = np.arange(0, N_chi * NK * Ny, NK * Ny)
    Blockx = np.ones((N_chi, NK, NK)) * vspace[:, None, None]
    XX = np.array([[1, 1, 1], [Ny + 1] * 3, [2 * Ny + 1] * 3], dtype=float)
    XX = np.repeat(XX[:, :, None], N_chi, axis=2).transpose(2, 0, 1)
    T = Blockx + XX
    NN = np.repeat(np.arange(Ny)[:, None], N_chi, axis=1).T.reshape(-1, order="F")
    T = np.tile(T, (Ny, 1, 1))
    Line = T + np.ones((N_chi * Ny, NK, NK)) * NN[:, None, None]
    Line = Line.transpose(1, 0, 2).reshape((-1, NK), order="F")
    Line = np.tile(Line, (Ny, 1))
    # column index (:286-317)
    XC = np.array([[1, Ny + 1, 2 * Ny + 1]] * 3, dtype=float)
    XC = np.repeat(XC[:, :, None], N_chi, axis=2).transpose(2, 0, 1)
    Tc = np.ones((N_chi, NK, NK)) * vspace[:, None, None] + XC
    Tc = np.tile(Tc, (Ny, 1, 1))
    Col = Tc.transpose(1, 0, 2).reshape((-1, NK), order="F")
    Col = np.tile(Col, (Ny, 1))
    spacer = np.tile(np.ones((NK, NK)), (N_chi * Ny * Ny, 1))
    off = np.repeat(np.arange(Ny)[:, None], NK * N_chi * Ny, axis=1).T.reshape(-1, order="F")
    Col = Col + spacer * off[:, None]
    rows = Line.reshape(-1, order="F").astype(np.int64) - 1
    cols = Col.reshape(-1, order="F").astype(np.int64) - 1
    vals = C.reshape(-1, order="F")
    import scipy.sparse as sp
    n = N_chi * NK * Ny
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def test_drift_index_tables_equal_general_form():
    spec, mat, E, efl, efr, m = small_rtd(n_el=5, nk=8, order=2)
    p = dg1d.init_params(mat, efl, efr, E, m)
    G1 = drift_by_index_tables(mat, p, E)
    G2 = dg1d.get_drift(mat, p, E)
    d = (G1 - G2)
    assert abs(d).max() <= 1e-13 * abs(G2).max()


# --- invariants the reference tests for Full-2D, restated for 1D ----------------------
@pytest.mark.parametrize("order,nxi", [(1, 0), (2, 0), (3, 0), (2, 40)])
def test_matrix_free_equals_assembled(order, nxi):
    spec, mat, E, efl, efr, m = small_rtd(n_el=6, nk=32, order=order, n_xi=nxi)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, _ = dg1d.get_sysm(mat, p, E)
    op = krylov.Operator1D(mat, p, E)
    i = np.arange(1, A.shape[0] + 1)
    x = np.sin(i) + 1j * np.cos(i)
    assert np.linalg.norm(op.apply(x) - A @ x) <= 1e-13 * np.linalg.norm(A @ x)


def test_constant_potential_gives_zero_wigner_potential_without_cap(monkeypatch):
    spec, mat, E, efl, efr, m = small_rtd(n_el=6, nk=16, order=2)
    p = dg1d.init_params(mat, efl, efr, E, m)
    monkeypatch.setattr(dg1d, "get_cap", lambda q, L, d: np.zeros_like(np.asarray(q, dtype=float)))
    G = dg1d.get_drift(mat, p, np.full(mat["Nx"], 0.37))
    assert abs(G).max() == 0.0


def test_inflow_only_in_boundary_elements():
    spec, mat, E, efl, efr, m = small_rtd(n_el=6, nk=16, order=2)
    p = dg1d.init_params(mat, efl, efr, E, m)
    rhs = dg1d.inflow_rhs(p).reshape(p["N_chi"], p["N_K_chi"], p["Nk"])
    assert np.all(rhs[1:-1] == 0)
    assert np.all(rhs[0][:, p["k"] < 0] == 0) and np.all(rhs[-1][:, p["k"] > 0] == 0)


def test_oracle_matches_golden_fixtures():
    from golden.make_golden import CASES, make_case
    g = np.load(GOLDEN)
    for name, args in CASES.items():
        out = make_case(name, *args)
        for key in ("Ax", "rhs", "rho", "n_dg", "j", "fnl", "fnr"):
            ref = g[name + "/" + key]
            assert np.linalg.norm(out[key] - ref) <= 1e-12 * np.linalg.norm(ref), (name, key)


def test_oracle_gmres_matches_direct_solve():
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=24, order=2)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    op = krylov.Operator1D(mat, p, E)
    pre = krylov.KLinePreconditioner(op, use_drift_diag=False)
    x, flag, relres, its, _ = krylov.gmres_right(op.apply, pre.apply, rhs, restart=30, tol=1e-12, maxit=30)
    ref = spla.spsolve(A.tocsc(), rhs)
    assert flag == 0 and relres <= 1e-12
    assert np.linalg.norm(x - ref) <= 1e-9 * np.linalg.norm(ref)


def test_kline_preconditioner_inverts_flux_exactly():
    spec, mat, E, efl, efr, m = small_rtd(n_el=7, nk=16, order=3)
    p = dg1d.init_params(mat, efl, efr, E, m)
    op = krylov.Operator1D(mat, p, E)
    pre = krylov.KLinePreconditioner(op, use_drift_diag=False)
    x = np.random.default_rng(1).standard_normal(op.N) + 0j
    assert np.linalg.norm(pre.apply(op.apply_flux(x)) - x) <= 1e-10 * np.linalg.norm(x)


def test_fet_subbands_and_mode_sum():
    """The FET builder's subbands (particle-in-a-box levels of the cross-section per
    valley type) and the oracle's valley x mode loop: n and j of a 2 x 2 subband
    solve are the sums of the single-subband solves."""
    from real_space_dg_gb300 import devices
    spec = devices.FETSpec(length_nm=16.0, sd_nm=5.0, n_el=8, order=1, nk=16, n_modes=2, l_xi_m=10e-9)
    off = devices.fet_subband_offsets(spec)
    hb, m0, q = 6.626e-34 / 2 / np.pi, 9.109e-31, 1.602e-19
    e11 = hb ** 2 * np.pi ** 2 * (1 / (spec.m_t * m0) + 1 / (spec.m_t * m0)) / (2 * (spec.width_nm * 1e-9) ** 2) / q
    assert abs(off[0, 0] - e11) < 1e-12 and np.all(np.diff(off, axis=1) >= 0)
    mat, esub, vsub, efl, efr = devices.make_fet(spec, 0.2, 0.1)
    assert esub.shape == (2, spec.nx, 2) and vsub.shape == (2, spec.nx, 2, 1) and abs(efl - efr - 0.1) < 1e-15
    full = dg1d.solve_transport_dg_2d(mat, esub, vsub, efl, efr)
    n_sum, j_sum = 0, 0
    for iv in range(2):
        for im in range(2):
            one = dict(mat, n_of_valleys=1, n_of_modes=1, me_x=mat["me_x"][iv:iv + 1])
            r = dg1d.solve_transport_dg_2d(one, esub[iv:iv + 1, :, im:im + 1], vsub[iv:iv + 1, :, im:im + 1],
                                           efl, efr)
            n_sum = n_sum + r["n"]
            j_sum = j_sum + r["j"]
    assert np.allclose(full["n"], n_sum, rtol=1e-13, atol=0)
    assert np.allclose(full["j"], j_sum, rtol=1e-13, atol=1e-30)
