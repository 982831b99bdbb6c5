"""Restatement of the reference's 1D phase-space Wigner solve (oracle only).

Test infrastructure: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, never by the product package.

Vector ordering (permute_shell=true, get_Diff.m:66-84): k fastest, then the
local x node, then the x element: index = (e*N_K + a)*Nk + j.

Functions follow, file:line in the reference project:
  init_params          DG_code/initParams.m:58-221 (FV, 1D, DG_MSA_2D branch)
  plane_wave_basis     DG_code/core/Basisfunktionen_Q_m.m:22-33
  verteilung_msa2d     DG_code/core/verteilung.m:118-170 (DG_MSA_2D branch)
  get_diff             DG_code/core/get_Diff.m:1-84 (permute_shell branch)
  v_transient          DG_code/core/V_transient.m:1-8
  get_cap              DG_code/core/get_CAP.m:1-12
  drift_b              get_Drift_accel_trial_permutedShell.m:15-66
  drift_pages          get_Drift_accel_trial_permutedShell.m:95-147
  get_drift            get_Drift_accel_trial_permutedShell.m:183-333 and
                       get_Drift.m:110-153 (general N_K contraction)
  get_sysm             DG_code/core/get_SysM.m:1-16
  observables          DG_code/solve_transport_DG_2D.m:114-156, 203-212
  solve_transport_dg_2d DG_code/solve_transport_DG_2D.m:1-226
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import jacobi

# Physical constants exactly as initParams.m:101-107 states them.
HQUER = 1.054571817e-34
M_ELEKTRON_DEFAULT = 0.041 * 9.1094e-31
Q_E = 1.602176634e-19
KB_P = 1.38064852e-23
# Constants of verteilung.m:161-165 and solve_transport_DG_2D.m:6-8 (they differ
# from initParams.m in the last digits; the reference uses both sets).
H_V = 6.626e-34
M0_V = 9.109e-31
HB_V = H_V / 2 / np.pi
KB_V = 1.38e-23
Q_V = 1.602e-19
NQX = 10
NKZ = 1001


def init_params(mat, EfL, EfR, V, m):
    """Discretisation constants of initParams.m:58-221 for Xi_solver='FV'.

    V is the subband energy on the material grid mat['x'] [eV], m the mass on
    that grid [kg].  Only the quantities used by the FV 1D path are built.
    """
    prm = mat["dg"]["params"]
    p = {}
    p["N_K_chi"] = int(prm["N_K_chi"])
    nx = int(mat["Nx"])
    if (nx - 1) % (p["N_K_chi"] - 1):
        raise ValueError("(Nx-1) must be divisible by N_K_chi-1")
    p["N_chi"] = (nx - 1) // (p["N_K_chi"] - 1)
    p["N_xi"] = int(prm["N_xi"])
    p["Nqx"] = NQX
    p["Nk"] = int(prm["N"])
    p["m_elektron"] = float(prm.get("m_elektron", M_ELEKTRON_DEFAULT))
    p["q"] = Q_E
    p["hquer"] = HQUER
    p["Q_diff"] = HQUER / p["m_elektron"]
    p["Q_drift"] = Q_E / HQUER
    p["U"] = 0.0
    p["L_xi"] = float(prm["Ly"])
    p["L_chi"] = float(mat["L_x"]) * 1e-9
    p["delta_chi"] = p["L_chi"] / p["N_chi"]
    p["disk"] = np.linspace(0.0, p["L_chi"], p["N_chi"] + 1)
    chi = np.zeros(p["N_chi"] * p["N_K_chi"])
    for a in range(p["N_chi"]):
        chi[a * p["N_K_chi"]:(a + 1) * p["N_K_chi"]] = np.linspace(p["disk"][a], p["disk"][a + 1],
                                                                  p["N_K_chi"])
    p["chi_Koord"] = chi
    xi = np.linspace(-p["L_xi"] / 2, p["L_xi"] / 2, p["N_xi"])
    p["delta_xi"] = xi[1] - xi[0]
    p["xi_elem"] = np.linspace(-(p["L_xi"] - p["delta_xi"]) / 2, (p["L_xi"] - p["delta_xi"]) / 2,
                               p["N_xi"])
    p["x"], p["w"] = jacobi.jacobi_gl(0, 0, NQX - 1)
    p["r"], _ = jacobi.jacobi_gl(0, 0, p["N_K_chi"] - 1)
    p["V_tilde"] = jacobi.vandermonde1d(p["N_K_chi"] - 1, p["x"])
    p["V"] = jacobi.vandermonde1d(p["N_K_chi"] - 1, p["r"])
    p["invV"] = np.linalg.inv(p["V"])
    p["M"] = p["invV"].T @ p["invV"]
    p["phi"], p["k"] = plane_wave_basis(p)
    p["fnl"], p["fnr"] = verteilung_msa2d(mat, p, V, m, EfL, EfR)
    return p


def plane_wave_basis(p):
    """Phi(xi_s, k_j) = exp(i k_j xi_s)/sqrt(L_xi) (Basisfunktionen_Q_m.m:22-33)."""
    nk = p["Nk"]
    k = -2 * np.pi / p["L_xi"] * (np.arange(1, nk + 1) - 0.5 * (nk + 1))
    phi = np.exp(1j * np.outer(p["xi_elem"], k)) / np.sqrt(p["L_xi"])
    return phi, k


def fermi_kz_integral(E_k, Ef, me_z, temp, vmax):
    """2/pi * dkz * sum_kz f_FD(E_k + E_kz) over Nkz=1001 kz (verteilung.m:141-152)."""
    kz_max = np.sqrt(2 * 2 * M0_V * me_z * Q_V * (vmax + 0.3)) / HB_V
    kz = np.linspace(0.0, kz_max, NKZ)
    dkz = kz[1] - kz[0]
    ekz = HB_V ** 2 * kz ** 2 / 2 / M0_V / me_z / Q_V
    arg = Q_V * (E_k[:, None] + ekz[None, :] - Ef) / (KB_V * temp)
    with np.errstate(over="ignore"):
        return 2 / np.pi * dkz * np.sum(1.0 / (1.0 + np.exp(arg)), axis=1)


def verteilung_msa2d(mat, p, V, m, EfL, EfR):
    """Contact inflow occupation in the k basis (verteilung.m:118-170, DG_MSA_2D).

    f(k) is the Fermi-Dirac occupation integrated over one transverse kz, cosine
    transformed to the xi cell centres, then projected on Phi by least squares
    (MATLAB's backslash; square Phi when N_xi == Nk).
    """
    V = np.asarray(V, dtype=float).ravel()
    m = np.asarray(m, dtype=float).ravel()
    nx = int(mat["Nx"])
    nk = p["Nk"]
    kf = -2 * np.pi / p["L_xi"] * (np.arange(1, nk + 1) - 0.5 * (nk + 1))
    dk = abs(kf[1] - kf[0])
    me_z = float(mat["me_z_ch"])
    temp = float(mat["Temp"])
    EL = V[0] + HB_V ** 2 * kf ** 2 / 2 / m[0] / Q_V
    ER = V[nx - 1] + HB_V ** 2 * kf ** 2 / 2 / m[nx - 1] / Q_V
    vmax = float(np.max(V))
    fL = fermi_kz_integral(EL, EfL, me_z, temp, vmax)
    fR = fermi_kz_integral(ER, EfR, me_z, temp, vmax)
    y = p["xi_elem"]
    cosm = np.cos(np.outer(y, kf))
    fLn = cosm @ fL * dk / 2 / np.pi
    fRn = cosm @ fR * dk / 2 / np.pi
    fnl = np.linalg.lstsq(p["phi"], fLn.astype(complex), rcond=None)[0]
    fnr = np.linalg.lstsq(p["phi"], fRn.astype(complex), rcond=None)[0]
    return fnl, fnr


def k_blocks(p):
    """Element flux blocks K1..K6 and the scaled inverse mass (get_Diff.m:22-45)."""
    nK = p["N_K_chi"]
    Dr = p["M"] @ jacobi.dmatrix1d(nK - 1, p["r"], p["V"])
    Dr[np.abs(Dr) < 1e-15] = 0.0
    Ms = p["delta_xi"] / 2 * p["M"]
    invM = np.linalg.inv(Ms)
    P1 = np.zeros((nK, nK)); P1[0, 0] = 1
    P2 = np.zeros((nK, nK)); P2[0, nK - 1] = 1
    P3 = np.zeros((nK, nK)); P3[nK - 1, nK - 1] = 1
    P4 = np.zeros((nK, nK)); P4[nK - 1, 0] = 1
    K = {}
    K["K1"] = invM @ (Dr + 0.5 * P1 - 0.5 * P3)
    K["K2L"] = invM @ (0.5 * P1)
    K["K2R"] = invM @ (0.5 * P3)
    K["K3"] = -0.5 * invM @ P2
    K["K4"] = K["K3"]
    K["K5"] = 0.5 * invM @ P4
    K["K6"] = -K["K5"]
    K["invM"] = invM
    return K


def get_diff(p):
    """Upwind x-flux times diag(k) and the contact inflow RHS (get_Diff.m:1-84).

    A = Q_diff * (kron(H1, D) + kron(H2, |D|)) in permuted-shell order with
    alpha == 1 (full upwind), H1/H2 block tridiagonal with blocks scaled 1/detJ.
    """
    n_el, nK, nk = p["N_chi"], p["N_K_chi"], p["Nk"]
    K = k_blocks(p)
    detJ = np.ones(n_el) * p["delta_chi"] / 2
    up = sp.diags(1.0 / detJ[1:], 1, shape=(n_el, n_el))
    lo = sp.diags(1.0 / detJ[1:], -1, shape=(n_el, n_el))
    dg = sp.diags(1.0 / detJ, 0, shape=(n_el, n_el))
    H1 = sp.kron(up, K["K5"]) + sp.kron(lo, K["K3"]) + sp.kron(dg, K["K1"])
    H2 = sp.kron(up, K["K6"]) + sp.kron(lo, K["K4"]) + sp.kron(dg, K["K2L"]) + sp.kron(dg, K["K2R"])
    D = sp.diags(p["k"])
    A = p["Q_diff"] * (sp.kron(H1, D) + sp.kron(H2, abs(D)))
    rhs = inflow_rhs(p, K)
    return sp.csr_matrix(A), rhs


def inflow_rhs(p, K=None):
    """Contact inflow vector Q_diff*(kron(Q1,(k>0)|k|fnl)+kron(Q2,(k<0)|k|fnr))."""
    if K is None:
        K = k_blocks(p)
    n_el, nK, nk = p["N_chi"], p["N_K_chi"], p["Nk"]
    detJ = p["delta_chi"] / 2
    k = p["k"]
    Q1 = np.zeros(n_el * nK); Q1[:nK] = K["invM"][:, 0] / detJ
    Q2 = np.zeros(n_el * nK); Q2[(n_el - 1) * nK:] = K["invM"][:, nK - 1] / detJ
    rhs = np.kron(Q1, (k > 0) * (np.abs(k) * p["fnl"])) + np.kron(Q2, (k < 0) * (np.abs(k) * p["fnr"]))
    return p["Q_diff"] * rhs


def v_transient(x, xg, Ug, Lx):
    """Potential lookup V_transient.m:1-8: linear interpolation inside [0, Lx),
    min(Ug) at x >= Lx and Ug(1) at x < 0."""
    x = np.asarray(x, dtype=float)
    Ug = np.asarray(Ug, dtype=float).ravel()
    out = np.zeros_like(x)
    inside = x < Lx
    out[inside] = np.interp(x[inside], xg, Ug)
    out[x >= Lx] = np.min(Ug)
    out[x < 0] = Ug[0]
    return out


def get_cap(q, L_xi, delta_xi):
    """Complex absorbing potential profile in xi (get_CAP.m:1-12)."""
    W0, n = 1.0, 1.0
    L0 = L_xi / 2 - delta_xi
    weite = L_xi * 0.40
    q = np.asarray(q, dtype=float)
    return (W0 / weite * (q - L0 + weite)) ** (2 * n) * (q >= L0 - weite) \
        + (W0 / weite * (q + L0 - weite)) ** (2 * n) * (q <= -L0 + weite)


def quad_points(p):
    """x quadrature coordinates per element, built as the reference builds them
    (cumulative Gauss-Lobatto spacings, get_Drift_accel_trial_permutedShell.m:16-55)."""
    frac = np.diff(p["x"]) / 2
    chi_gl = np.zeros(NQX)
    for i in range(NQX - 1):
        chi_gl[i + 1] = chi_gl[i] + frac[i] * p["delta_chi"]
    xq = np.zeros(p["N_chi"] * NQX)
    for i in range(p["N_chi"]):
        xq[i * NQX:(i + 1) * NQX] = p["disk"][i] + chi_gl
    return xq


def xi_edges(p):
    """FV xi edge coordinates used by the drift (permutedShell.m:27-28)."""
    return np.linspace(-p["L_xi"] / 2, p["L_xi"] / 2, p["N_xi"] + 1)


def drift_b(mat, p, EM):
    """B(x_q, xi_s) = V(x+xi/2) - V(x-xi/2) - i*CAP(xi) (permutedShell.m:64-66)."""
    xq = quad_points(p)
    ye = xi_edges(p)
    X = xq[:, None] + 0 * ye[None, :]
    Y = ye[None, :] + 0 * xq[:, None]
    xg = np.asarray(mat["x"], dtype=float) * 1e-9
    B = v_transient(X + 0.5 * Y, xg, EM, p["L_chi"]) - v_transient(X - 0.5 * Y, xg, EM, p["L_chi"]) \
        - 1j * get_cap(Y, p["L_xi"], p["delta_xi"])
    return B


def drift_pages(p, B):
    """G_i = 1i * Phi^H C_i Phi with C_i = (dxi/4) tridiag (permutedShell.m:95-147)."""
    phi = p["phi"]
    nq, ne = B.shape
    M = ne - 1
    G = np.empty((nq, p["Nk"], p["Nk"]), dtype=complex)
    for i in range(nq):
        main = B[i, :M] + B[i, 1:M + 1]
        off = B[i, 1:M]
        Cphi = main[:, None] * phi
        Cphi[:-1] += off[:, None] * phi[1:]
        Cphi[1:] += off[:, None] * phi[:-1]
        G[i] = 1j * (phi.conj().T @ (p["delta_xi"] / 4 * Cphi))
    return G


def interp_w(p):
    """W = V_tilde / V: Lagrange interpolation from the DG nodes to the 10 GL points."""
    return np.linalg.solve(p["V"].T, p["V_tilde"].T).T


def get_drift(mat, p, EM, return_pages=False):
    """Assembled Wigner-potential operator in permuted-shell order.

    G_d[(e,a,j),(e,b,m)] = Q_drift*invM(a,b) * sum_q w_q W(q,a) W(q,b) G_{e,q}(j,m)
    (get_Drift.m:128-153 form; the index tables of permutedShell.m:252-333 place
    the same values, invM being symmetric).
    """
    n_el, nK, nk = p["N_chi"], p["N_K_chi"], p["Nk"]
    B = drift_b(mat, p, EM)
    G = drift_pages(p, B)
    W = interp_w(p)
    invM = k_blocks(p)["invM"]
    w = p["w"]
    rows, cols, vals = [], [], []
    jj, mm = np.meshgrid(np.arange(nk), np.arange(nk), indexing="ij")
    for e in range(n_el):
        Ge = G[e * NQX:(e + 1) * NQX]
        for a in range(nK):
            for b in range(nK):
                c = p["Q_drift"] * invM[a, b] * np.einsum("q,qjm->jm", w * W[:, a] * W[:, b], Ge)
                rows.append(((e * nK + a) * nk + jj).ravel())
                cols.append(((e * nK + b) * nk + mm).ravel())
                vals.append(c.ravel())
    n = n_el * nK * nk
    Gd = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(n, n))
    if return_pages:
        return Gd, B, G
    return Gd


def get_sysm(mat, p, EM):
    """A = A_diff + G_drift, rhs from get_Diff (get_SysM.m:1-16, FV branch)."""
    A, rhs = get_diff(p)
    return (A + get_drift(mat, p, EM)).tocsr(), rhs


def node_map(p, values):
    """Material-grid values -> DG nodes: node a of element e is material node
    e*(N_K-1)+a (solve_transport_DG_2D.m:81-87)."""
    values = np.asarray(values)
    n_el, nK = p["N_chi"], p["N_K_chi"]
    idx = (np.arange(n_el)[:, None] * (nK - 1) + np.arange(nK)[None, :]).ravel()
    return values[idx]


def observables(p, rho, m_mod):
    """rho_u = Phi * reshape(rho, Nk, Nxdof); n and j at the centre xi rows
    (solve_transport_DG_2D.m:114-156, FV branch)."""
    nk = p["Nk"]
    R = rho.reshape(-1, nk).T
    rho_u = p["phi"] @ R
    nxi = p["N_xi"]
    if nxi % 2 == 1:
        c = (nxi - 1) // 2
        n_dg = np.real(rho_u[c])
        j = Q_E * HB_V / m_mod * np.imag(rho_u[c + 1] - rho_u[c - 1]) / 2 / p["delta_xi"]
    else:
        c = nxi // 2
        n_dg = (np.real(rho_u[c - 1]) + np.real(rho_u[c])) / 2
        j = Q_E * HB_V / m_mod * np.imag(rho_u[c] - rho_u[c - 1]) / p["delta_xi"]
    return n_dg, j, rho_u


def solve_transport_dg_2d(mat, Esub, Vsub, EfL, EfR, solver="direct", return_systems=False):
    """DG = solve_transport_DG_2D(mat, Esub, Vsub, EfL, EfR) for Xi_solver='FV'.

    Loops valleys x modes, assembles A and rhs, solves A rho = rhs (sparse LU,
    solve_transport_DG_2D.m:101), forms n and j and weights n by |Vsub|^2/dy.
    """
    prm = mat["dg"]["params"]
    nv, nm = int(mat["n_of_valleys"]), int(mat["n_of_modes"])
    ny = int(mat["Ny"])
    Esub = np.asarray(Esub, dtype=float).reshape(nv, int(mat["Nx"]), nm)
    Vsub = np.asarray(Vsub, dtype=float).reshape(nv, int(mat["Nx"]), nm, ny)
    me_x = np.asarray(mat["me_x"], dtype=float).reshape(nv, int(mat["Nx"]), ny)
    mid = int(np.ceil(ny / 2)) - 1
    nT = None
    jT = None
    RHO = []
    systems = []
    for iv in range(nv):
        m = me_x[iv, :, mid] * M0_V
        for im in range(nm):
            EM = Esub[iv, :, im]
            p = init_params(mat, EfL, EfR, EM, m)
            A, rhs = get_sysm(mat, p, EM)
            mpc = float(prm.get("MPC", 1.0))
            if mpc != 1:
                A = mpc * A
                rhs = mpc * rhs
            if solver == "direct":
                rho = spla.spsolve(A.tocsc(), rhs)
            else:
                rho = solver(A, rhs, p)
            if return_systems:
                systems.append((A, rhs, rho, p))
            m_mod = node_map(p, m)
            n_dg, j, rho_u = observables(p, rho, m_mod)
            vs = node_map(p, Vsub[iv, :, im, :])
            n_mode = n_dg[:, None] * np.abs(vs) ** 2 / float(mat["dy"]) / 1e-9
            nT = n_mode if nT is None else nT + n_mode
            jT = j if jT is None else jT + j
            RHO.append(rho_u.T)
    out = {"n": nT, "j": jT, "RHO": np.array(RHO).reshape(nv, nm, *RHO[0].shape),
           "chi": p["chi_Koord"], "xi": p["xi_elem"], "p": p}
    if return_systems:
        out["systems"] = systems
    return out
