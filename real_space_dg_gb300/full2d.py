"""Full-2D (X, Y, rho_x, rho_y) Wigner operator on the GPU: the host side of
``sysInfo.makeGPUApply()`` (DG_code/core/get_SysM_full2D.m:81, 124-139).

As in the reference, the host builds the constant one-dimensional factors once
(DG element matrices, FV derivatives and their characteristic splits, the element
quadrature of the potential term) and hands them to the device; every apply then
runs on the GPU (``wg2d_*`` in libwigner_gb300.so):

  - transport, get_Diff_full2D.m:76-146: every operator part acts on one centre axis
    and the matching relative axis, kron(I_Y, C_X) x kron(I_rho_y, R_x) or
    kron(C_Y, I_X) x kron(R_y, I_rho_x); parts with the same relative factor are merged;
  - potential and CAP, get_Drift_full2D.m:133-364 (FV-consistent form): the vertex
    potential differences are rebuilt on the device from V on the material grid.

Supported: source/drain faces fully open, Y boundaries 'periodic', 'zero-inflow' and
'specular', X/Y fluxes 'upwind', 'rusanov', 'central', constant mass.
"""
import ctypes as C
import math

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import WignerError

HBAR = 1.054571817e-34
M0 = 9.1093837015e-31
QE = 1.602176634e-19


# ---------------------------------------------------------------- reference element (JacobiGL.m etc.)

def _jacobi_gq(alpha, beta, n):
    if n == 0:
        return np.array([-(alpha - beta) / (alpha + beta + 2.0)]), np.array([2.0])
    h1 = 2.0 * np.arange(n + 1) + alpha + beta
    with np.errstate(divide="ignore", invalid="ignore"):
        main = -0.5 * (alpha ** 2 - beta ** 2) / (h1 + 2.0) / h1
    i = np.arange(1, n + 1, dtype=float)
    off = 2.0 / (h1[:n] + 2.0) * np.sqrt(i * (i + alpha + beta) * (i + alpha) * (i + beta) / (h1[:n] + 1.0)
                                         / (h1[:n] + 3.0))
    if alpha + beta < 10 * np.finfo(float).eps:
        main[0] = 0.0
    J = np.diag(main) + np.diag(off, 1)
    d, v = np.linalg.eigh(J + J.T)
    w = v[0, :] ** 2 * 2 ** (alpha + beta + 1) / (alpha + beta + 1) * math.gamma(alpha + 1) * math.gamma(beta + 1) \
        / math.gamma(alpha + beta + 1)
    return d, w


def _legendre(n, x):
    p0, p1 = 1.0, x
    if n == 0:
        return p0
    for k in range(1, n):
        p0, p1 = p1, ((2 * k + 1) * x * p1 - k * p0) / (k + 1)
    return p1


def gauss_lobatto(n):
    """Nodes and weights of order n on [-1, 1] (JacobiGL.m with alpha = beta = 0)."""
    if n == 1:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    xi, _ = _jacobi_gq(1.0, 1.0, n - 2)
    x = np.concatenate(([-1.0], xi, [1.0]))
    m = n + 1
    w = np.array([2.0 / (m * (m - 1)) / _legendre(m - 1, t) ** 2 for t in x])
    return x, w


def _jacobi_p(x, n):
    """Orthonormal Legendre polynomial of degree n (JacobiP.m with alpha = beta = 0)."""
    x = np.asarray(x, dtype=float)
    pl = [np.full_like(x, 1.0 / math.sqrt(2.0))]
    if n == 0:
        return pl[0]
    pl.append(x * math.sqrt(1.5))
    aold = 1.0 / math.sqrt(3.0)
    for i in range(1, n):
        h1 = 2.0 * i
        anew = 2.0 / (h1 + 2.0) * math.sqrt((i + 1) ** 4 / (h1 + 1.0) / (h1 + 3.0))
        pl.append(1.0 / anew * (-aold * pl[i - 1] + x * pl[i]))
        aold = anew
    return pl[n]


def vandermonde(n, r):
    return np.stack([_jacobi_p(r, j) for j in range(n + 1)], axis=1)


def _grad_jacobi_p(r, n):
    return np.zeros_like(r) if n == 0 else math.sqrt(n * (n + 1)) * _jacobi_p_ab(r, 1.0, 1.0, n - 1)


def _jacobi_p_ab(x, alpha, beta, n):
    x = np.asarray(x, dtype=float)
    g0 = 2 ** (alpha + beta + 1) / (alpha + beta + 1) * math.gamma(alpha + 1) * math.gamma(beta + 1) \
        / math.gamma(alpha + beta + 1)
    pl = [np.full_like(x, 1.0 / math.sqrt(g0))]
    if n == 0:
        return pl[0]
    g1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * g0
    pl.append(((alpha + beta + 2) * x / 2 + (alpha - beta) / 2) / math.sqrt(g1))
    aold = 2 / (2 + alpha + beta) * math.sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3))
    for i in range(1, n):
        h1 = 2 * i + alpha + beta
        anew = 2 / (h1 + 2) * math.sqrt((i + 1) * (i + 1 + alpha + beta) * (i + 1 + alpha) * (i + 1 + beta)
                                        / (h1 + 1) / (h1 + 3))
        bnew = -(alpha ** 2 - beta ** 2) / h1 / (h1 + 2)
        pl.append(1 / anew * (-aold * pl[i - 1] + (x - bnew) * pl[i]))
        aold = anew
    return pl[n]


def differentiation_matrix(n, r, V):
    Vr = np.stack([_grad_jacobi_p(r, j) for j in range(n + 1)], axis=1)
    return Vr @ np.linalg.inv(V)


# ---------------------------------------------------------------- one-dimensional factors

def _param(prm, name, default):
    v = prm.get(name, None)
    return default if v is None else v


def dg_axis(coord, n_local, n_el):
    """Element matrices and geometry of one DG axis (initParams_full2D.m:167-214)."""
    r, w = gauss_lobatto(n_local - 1)
    V = vandermonde(n_local - 1, r)
    invV = np.linalg.inv(V)
    M = invV.T @ invV
    Dr = differentiation_matrix(n_local - 1, r, V)
    verts = np.linspace(coord[0], coord[-1], n_el + 1)
    jac = (verts[1:] - verts[:-1]) / 2
    nodes = (0.5 * (verts[:-1] + verts[1:])[:, None] + jac[:, None] * r[None, :]).ravel()
    return dict(nl=n_local, ne=n_el, nd=n_local * n_el, r=r, V=V, M=M, S=M @ Dr, verts=verts, jac=jac, nodes=nodes)


def dg_axis_operators(ax, periodic):
    """H1, H2 interior/boundary and the boundary lifts of one axis as element blocks
    (get_Diff_full2D.m:206-265; close_PeriodicDGAxis_full2D.m when periodic).
    Returns dense nd x nd matrices (small: the element count of one axis)."""
    n, ne, nd = ax["nl"], ax["ne"], ax["nd"]
    invM = np.linalg.inv(ax["M"])
    E = lambda i, j: np.eye(1, n * n, i * n + j).reshape(n, n)   # unit matrix e_i e_j^T
    K1 = invM @ (ax["S"] + 0.5 * E(0, 0) - 0.5 * E(n - 1, n - 1))
    K2 = invM @ (0.5 * E(0, 0) + 0.5 * E(n - 1, n - 1))
    K2L, K2R = invM @ (0.5 * E(0, 0)), invM @ (0.5 * E(n - 1, n - 1))
    K3 = -0.5 * invM @ E(0, n - 1)
    K5 = 0.5 * invM @ E(n - 1, 0)
    ij = 1.0 / ax["jac"]
    H1, H2, HB = (np.zeros((nd, nd)) for _ in range(3))
    for e in range(ne):
        s = slice(e * n, (e + 1) * n)
        H1[s, s] += ij[e] * K1
        H2[s, s] += ij[e] * K2
        if e + 1 < ne:                       # coupling to the right neighbour, scaled by its 1/jacobian
            t = slice((e + 1) * n, (e + 2) * n)
            H1[s, t] += ij[e + 1] * K5
            H2[s, t] += -ij[e + 1] * K5
        if e > 0:
            t = slice((e - 1) * n, e * n)
            H1[s, t] += ij[e] * K3
            H2[s, t] += ij[e] * K3
    HB[:n, :n] += ij[0] * K2L
    HB[nd - n:, nd - n:] += ij[-1] * K2R
    llift = np.zeros(nd); llift[:n] = invM[:, 0] / ax["jac"][0]
    rlift = np.zeros(nd); rlift[nd - n:] = invM[:, n - 1] / ax["jac"][-1]
    left = np.zeros(nd); left[0] = 1
    right = np.zeros(nd); right[-1] = 1
    HI = H2 - HB
    if periodic:
        H1 = H1 - 0.5 * np.outer(llift, right) + 0.5 * np.outer(rlift, left)
        HI = HI + 0.5 * np.outer(llift - rlift, left - right)
        HB = np.zeros_like(HB)
    return dict(H1=H1, HI=HI, HB=HB, lb=np.outer(llift, left), rb=np.outer(rlift, right))


def fv_axis(n_cells, length, periodic=False):
    """Cell centres, edges and the central derivative (initParams_full2D.m:216-230, 90-96)."""
    edges = np.linspace(-length / 2, length / 2, n_cells + 1)
    d = edges[1] - edges[0]
    D = (np.eye(n_cells, k=1) - np.eye(n_cells, k=-1)) / (2 * d)
    if periodic:
        D[0, -1] -= 1 / (2 * d)
        D[-1, 0] += 1 / (2 * d)
    return dict(n=n_cells, length=length, edges=edges, cells=0.5 * (edges[:-1] + edges[1:]), delta=d, D=D)


def characteristic_split(A, tol=1e-12):
    """A+ and A- from the eigen-decomposition (get_Diff_full2D.m:718-730)."""
    lam, Phi = np.linalg.eig(A)
    lp = np.where(lam.real <= tol, 0, lam)
    lm = np.where(lam.real >= -tol, 0, lam)
    Pinv = np.linalg.solve(Phi, np.eye(len(lam)))
    Ap, Am = Phi @ np.diag(lp) @ Pinv, Phi @ np.diag(lm) @ Pinv
    Ap[np.abs(Ap) < 1e-12] = 0
    Am[np.abs(Am) < 1e-12] = 0
    return Ap, Am, lam


def cap_1d(q, length, delta):
    """get_CAP.m: W0 = 1, n = 1, width 0.4 L at both ends."""
    L0 = length / 2 - delta
    wd = length * 0.40
    return ((q - L0 + wd) / wd) ** 2 * (q >= L0 - wd) + ((q + L0 - wd) / wd) ** 2 * (q <= -L0 + wd)


def _flux(prm):
    general = str(_param(prm, "full2D_fluxType", _param(prm, "rho_flux", _param(prm, "fluxType", "rusanov")))).lower()
    general = "rusanov" if general in ("lf", "lax-friedrichs", "rusanov-local") else general

    def norm(v):
        v = str(v).strip().lower()
        return {"lf": "rusanov", "lax-friedrichs": "rusanov", "rusanov-local": "rusanov",
                "matrix-upwind": "upwind", "characteristic-upwind": "upwind"}.get(v, v)
    fx = norm(_param(prm, "full2D_X_flux", general))
    return fx, norm(_param(prm, "full2D_Y_flux", fx))


def _ytype(prm):
    v = str(prm.get("full2D_Y_boundary", "specular")).strip().lower()
    return {"specular-reflection": "specular", "reflection": "specular", "reflecting": "specular",
            "zero_inflow": "zero-inflow", "zeroinflow": "zero-inflow", "zero": "zero-inflow"}.get(v, v)


def _blocks(Cm, nl, ne, periodic):
    """Element blocks [ne][3][nl][nl] of a block-tridiagonal (wrapped when periodic) matrix."""
    out = np.zeros((ne, 3, nl, nl))
    seen = np.zeros(Cm.shape, dtype=bool)
    for e in range(ne):
        rows = slice(e * nl, (e + 1) * nl)
        for k, dirn in enumerate((-1, 0, 1)):
            en = e + dirn
            if en < 0 or en >= ne:
                if not periodic:
                    continue
                en %= ne
            if dirn == 1 and periodic and (e + 1) % ne == (e - 1) % ne:
                continue                     # both neighbours are the same element: kept once, in dir -1
            cols = slice(en * nl, (en + 1) * nl)
            out[e, k] = Cm[rows, cols]
            seen[rows, cols] = True
    if np.any(Cm[~seen] != 0):
        raise WignerError(_lib.WG_ERR_ARG, "centre factor is not block-tridiagonal over the elements")
    return out


def build_factors(mat):
    """The one-dimensional factors of the operator (host set-up, once per shape and
    options): dict(shape, n, x, y, terms=(X terms, Y terms) as [(coef, centre matrix,
    relative 1D matrix)], axes, drift data, nq)."""
    prm = mat["dg"]["params"]
    scale = _param(prm, "full2D_coordinate_scale", 1e-9)
    x = np.asarray(mat["x"], dtype=float) * scale
    y = np.asarray(mat["y"], dtype=float) * scale
    nkd = _param(prm, "N_K_chi", 3)
    nkx, nky = int(_param(prm, "N_K_X", nkd)), int(_param(prm, "N_K_Y", nkd))
    nex = int(_param(prm, "N_el_X", (len(x) - 1) // (nkx - 1)))
    ney = int(_param(prm, "N_el_Y", (len(y) - 1) // (nky - 1)))
    ytype = _ytype(prm)
    if ytype not in ("periodic", "zero-inflow", "specular"):
        raise WignerError(_lib.WG_ERR_ARG, "Full-2D Y boundary %r is not supported on the GPU" % ytype)
    periodic = ytype == "periodic"
    nrx = int(_param(prm, "N_rho_x", _param(prm, "N_xi", 40)))
    nry = int(_param(prm, "N_rho_y", nrx))
    ldef = _param(prm, "Ly", max(abs(y[-1] - y[0]), np.finfo(float).eps))
    lrx = float(_param(prm, "L_rho_x", ldef))
    lry = float(_param(prm, "L_rho_y", 2 * (y[-1] - y[0]) if periodic else ldef))
    AX, AY = dg_axis(x, nkx, nex), dg_axis(y, nky, ney)
    RX, RY = fv_axis(nrx, lrx), fv_axis(nry, lry, periodic)
    fx, fy = _flux(prm)

    def me(m):                           # massToKg of get_Diff_full2D.m:757-767
        mk = m * M0 if abs(m) > 1e-25 else m
        return mk if mk > 0 else 0.041 * M0
    mex = mat.get("me_x_ch", 0.041)
    mey = mat.get("me_y_ch", mex)
    fsc = _param(prm, "full2D_diff_scale", _param(prm, "rho_diff_scale", 1.0))
    sx = fsc * _param(prm, "full2D_Q_diff_x", _param(prm, "full2D_transportScaleX", HBAR / me(mex)))
    sy = fsc * _param(prm, "full2D_Q_diff_y", _param(prm, "full2D_transportScaleY", HBAR / me(mey)))
    ox, oy = dg_axis_operators(AX, False), dg_axis_operators(AY, periodic)
    tol = _param(prm, "full2D_characteristicTol", 1e-12)
    Ax, Ay = -1j * RX["D"], -1j * RY["D"]
    Apx, Amx, lx = characteristic_split(Ax, tol)
    Apy, Amy, ly = characteristic_split(Ay, tol)
    absx, absy = Apx - Amx, Apy - Amy

    def theta(f, name):
        return _param(prm, name, _param(prm, "full2D_thetaLF", _param(prm, "thetaLF", 0.01))) if f == "rusanov" else 0.0
    bx = theta(fx, "full2D_thetaLF_X") * _param(prm, "full2D_alphaLF_X", np.max(np.abs(lx)))
    by = theta(fy, "full2D_thetaLF_Y") * _param(prm, "full2D_alphaLF_Y", np.max(np.abs(ly)))
    tx = [(sx, ox["H1"], Ax)]
    if fx == "upwind":
        tx.append((sx, ox["HI"], absx))
    elif bx != 0:
        tx.append((sx, ox["HI"], bx * np.eye(nrx)))
    tx.append((sx, ox["HB"], absx))
    ty = [(sy, oy["H1"], Ay)]
    if fy == "upwind":
        ty.append((sy, oy["HI"], absy))
    elif by != 0:
        ty.append((sy, oy["HI"], by * np.eye(nry)))
    if ytype != "periodic":
        ty.append((sy, oy["HB"], absy))
    if ytype == "specular":
        flip = np.fliplr(np.eye(nry))
        ty.append((-sy, oy["lb"], Apy @ flip))
        ty.append((sy, oy["rb"], Amy @ flip))
    drift, nq = _drift_setup(prm, AX, AY, RX, RY, periodic)
    return dict(shape=dict(n_el_x=nex, nk_x=nkx, n_el_y=ney, nk_y=nky, n_rho_x=nrx, n_rho_y=nry,
                           periodic_y=int(periodic)),
                n=nrx * nry * nex * nkx * ney * nky, x=x, y=y, terms=(_merge(tx), _merge(ty)), axes=(AX, AY),
                rel=(RX, RY), scales=(sx, sy), drift=drift, nq=nq, split=(Apx, Amx, Apy, Amy), ytype=ytype,
                scale=scale)


def _bilinear(gx, gy, V, qx, qy, periodic):
    """V at (qx, qy): X clamped, Y clamped or wrapped, linear in both (get_Drift_full2D.m:650-666)."""
    qx = np.clip(qx, gx[0], gx[-1])
    qy = gy[0] + np.mod(qy - gy[0], gy[-1] - gy[0]) if periodic else np.clip(qy, gy[0], gy[-1])
    ix = np.clip(np.searchsorted(gx, qx, side="right") - 1, 0, len(gx) - 2)
    iy = np.clip(np.searchsorted(gy, qy, side="right") - 1, 0, len(gy) - 2)
    tx = (qx - gx[ix]) / (gx[ix + 1] - gx[ix])
    ty = (qy - gy[iy]) / (gy[iy + 1] - gy[iy])
    return ((1 - tx) * (1 - ty) * V[ix, iy] + tx * (1 - ty) * V[ix + 1, iy] + (1 - tx) * ty * V[ix, iy + 1]
            + tx * ty * V[ix + 1, iy + 1])


def _transverse_reference(mat, V, ix):
    """Frozen-X transverse transport K and potential V blocks at material column ix: the
    (rho_x cell 0, X dof 0) block of a strip with 2 rho_x cells, 2 X elements of 2 nodes, no X
    transport and no CAP (transverseReference, get_LineTransversePreconditioner_full2D.m:127-175)."""
    prm = dict(mat["dg"]["params"])
    prm.update(N_rho_x=2, N_K_X=2, N_el_X=2, full2D_Q_diff_x=0.0, full2D_cap_scale=0.0)
    strip = dict(mat)
    strip["dg"] = dict(mat["dg"], params=prm)
    fs = build_factors(strip)
    s, (AX, AY), (RX, RY) = fs["shape"], fs["axes"], fs["rel"]
    nry, nY = s["n_rho_y"], AY["nd"]
    periodic = bool(s["periodic_y"])
    K = np.zeros((nry * nY, nry * nY), dtype=complex)
    for c, Cm, R in fs["terms"][1]:
        K += c * np.kron(Cm, R)
    for c, Cm, R in fs["terms"][0]:
        if c != 0:
            raise WignerError(_lib.WG_ERR_ARG, "strip with X transport")
    d = fs["drift"]
    Vr = np.repeat(np.asarray(V, dtype=float)[ix:ix + 1, :], len(fs["x"]), axis=0)
    nq, nvx = fs["nq"], RX["n"] + 1
    nvy = nry if periodic else nry + 1
    # vertex sums P: (rho_x cell 0 touches vertices 0, 1 in x); cells of rho_y around each vertex
    Ex = np.zeros((nvx, RX["n"])); Ex[np.arange(RX["n"]), np.arange(RX["n"])] = 1; Ex[np.arange(1, nvx), np.arange(RX["n"])] = 1
    if periodic:                                      # vertex j touches cells j and j - 1 (mod n)
        Ey = np.eye(nry); Ey[np.arange(nry), (np.arange(nry) - 1) % nry] += 1
    else:
        Ey = np.zeros((nry + 1, nry)); Ey[np.arange(nry), np.arange(nry)] = 1; Ey[np.arange(1, nry + 1), np.arange(nry)] = 1
    P = np.kron(Ey, Ex)
    sel = 2 * np.arange(nry)                          # rel = 0 + 2 ry
    nkx, nky = AX["nl"], AY["nl"]
    Vb = np.zeros_like(K)
    for ey in range(AY["ne"]):
        e = 0 + 2 * ey                                # element (ex = 0, ey)
        X = d["xq"][e][None, :]
        Yq = d["yq"][e][None, :]
        hx, hy = 0.5 * d["vx"][:, None], 0.5 * d["vy"][:, None]
        dV = _bilinear(fs["x"], fs["y"], Vr, X + hx, Yq + hy, periodic) - \
            _bilinear(fs["x"], fs["y"], Vr, X - hx, Yq - hy, periodic)          # [n_vert, nq]
        for ly in range(nky):
            for ly2 in range(nky):
                l, l2 = 0 + nkx * ly, 0 + nkx * ly2
                acc = np.zeros((nry, nry), dtype=complex)
                for q in range(nq):
                    Hq = d["proj"][q, l] * d["interp"][q, l2]
                    if Hq == 0:
                        continue
                    C = (P.T * dV[:, q]) @ P
                    acc += Hq * C[np.ix_(sel, sel)]
                Y1, Y2 = ey * nky + ly, ey * nky + ly2
                Vb[Y1 * nry:(Y1 + 1) * nry, Y2 * nry:(Y2 + 1) * nry] += d["pot"] / 16 * acc
    return K, 2.0 * Vb                                 # the rho_x diagonal of P_x' P_x / 4 is 1/2


def build_preconditioner(mat, V, f, ix=0):
    """Host factors of the line-transverse preconditioner (get_LineTransversePreconditioner_full2D.m:17-113):
    modes U of -i D_rho_x, the shift sigma, X-line factors per mode and element, dense inverses of
    the shifted transverse blocks per mode."""
    prm = mat["dg"]["params"]
    s, (AX, AY), (RX, RY) = f["shape"], f["axes"], f["rel"]
    nm, nry, nY = s["n_rho_x"], s["n_rho_y"], AY["nd"]
    nT = nry * nY
    lam, U = np.linalg.eigh(-1j * RX["D"])
    lam = lam.real.copy()
    lam[np.abs(lam) < 100 * np.spacing(np.max(np.abs(lam)))] = 0
    K, Vt = _transverse_reference(mat, V, ix)
    d = f["drift"]
    wx = cap_1d(RX["cells"], RX["length"], RX["delta"])
    wy = np.zeros(nry) if s["periodic_y"] else cap_1d(RY["cells"], RY["length"], RY["delta"])
    capY = np.tile(wy, nY) * d["capc"]
    capX = np.real(np.sum(np.conj(U) * (wx[:, None] * U), axis=0)) * d["capc"]
    Pm = np.zeros((nm + 1, nm)); Pm[np.arange(nm), np.arange(nm)] = 1; Pm[np.arange(1, nm + 1), np.arange(nm)] = 1
    pw = np.real(np.sum(np.conj(U) * ((Pm.T @ Pm / 4) @ U), axis=0))
    sx = f["scales"][0]
    x_rate = abs(sx) * np.max(np.abs(lam)) / np.min(AX["jac"])
    t_rate = np.max(np.abs(K).sum(1)) + np.max(np.abs(Vt).sum(1)) + np.max(np.abs(capY)) + np.max(np.abs(capX))
    sigma = float(_param(prm, "full2D_lineShift", _param(prm, "full2D_lineRelativeShift", 0.003)
                         * max(x_rate, t_rate, np.finfo(float).tiny)))
    n, ne = AX["nl"], AX["ne"]
    Minv = np.linalg.inv(AX["M"])
    E = lambda i, j: np.eye(1, n * n, i * n + j).reshape(n, n)
    K1 = Minv @ (AX["S"] + 0.5 * E(0, 0) - 0.5 * E(n - 1, n - 1))
    K2 = Minv @ (0.5 * E(0, 0) + 0.5 * E(n - 1, n - 1))
    speeds = sx * lam
    fwd = (speeds >= 0).astype(np.int32)
    xinv = np.zeros((nm, ne, n, n), dtype=complex)
    xcpl = np.zeros_like(xinv)
    for e in range(ne):
        a = speeds / (sigma * AX["jac"][e])
        for k in range(nm):
            xinv[k, e] = np.linalg.inv(np.eye(n) + a[k] * K1 + abs(a[k]) * K2)
            xcpl[k, e] = -a[k] * (Minv @ E(0, n - 1)) if fwd[k] else a[k] * (Minv @ E(n - 1, 0))
    tinv = np.empty((nm, nT, nT), dtype=complex)
    for k in range(nm):
        B = (K + pw[k] * Vt + np.diag(capY + capX[k])) / sigma + np.eye(nT)
        tinv[k] = np.linalg.inv(B)
    return dict(U=U, lam=lam, sigma=sigma, xinv=xinv, xcpl=xcpl, fwd=fwd, tinv=tinv)


def _merge(terms):
    """Merge terms with the same coefficient and relative factor (their centre factors add)."""
    out = []
    for c, Cm, R in terms:
        for i, (c2, C2, R2) in enumerate(out):
            if c2 == c and R2.shape == R.shape and np.array_equal(R2, R):
                out[i] = (c, C2 + Cm, R)
                break
        else:
            out.append((c, np.array(Cm, dtype=float), np.array(R, dtype=complex)))
    return [t for t in out if np.any(t[1]) and np.any(t[2])]


def _drift_setup(prm, AX, AY, RX, RY, periodic):
    """Element quadrature and relative vertices of the FV-consistent potential
    (get_Drift_full2D.m:133-300)."""
    nlx, nly = AX["nl"], AY["nl"]
    common = prm.get("full2D_potentialQuadratureOrder", None)
    nqx = _param(prm, "full2D_potentialQuadratureX", max(4, 2 * nlx - 1)) if common is None else common
    nqy = _param(prm, "full2D_potentialQuadratureY", max(4, 2 * nly - 1)) if common is None else common
    nqx, nqy = max(nlx, int(round(nqx))), max(nly, int(round(nqy)))
    qx, wx = gauss_lobatto(nqx - 1)
    qy, wy = gauss_lobatto(nqy - 1)
    Ix = vandermonde(nlx - 1, qx) @ np.linalg.inv(AX["V"])
    Iy = vandermonde(nly - 1, qy) @ np.linalg.inv(AY["V"])
    interp = np.kron(Iy, Ix)
    w = np.kron(wy, wx)
    MXY = np.kron(AY["M"], AX["M"])
    proj = (interp * w[:, None]) @ np.linalg.solve(MXY, np.eye(MXY.shape[0])).T
    xq, yq = [], []
    for ey in range(AY["ne"]):
        yc = 0.5 * (AY["verts"][ey] + AY["verts"][ey + 1]) + AY["jac"][ey] * qy
        for ex in range(AX["ne"]):
            xc = 0.5 * (AX["verts"][ex] + AX["verts"][ex + 1]) + AX["jac"][ex] * qx
            Xq, Yq = np.meshgrid(xc, yc, indexing="ij")
            xq.append(Xq.ravel(order="F"))
            yq.append(Yq.ravel(order="F"))
    ey_edges = RY["edges"][:-1] if periodic else RY["edges"]
    VX, VY = np.meshgrid(RX["edges"], ey_edges, indexing="ij")
    wxc = cap_1d(RX["cells"], RX["length"], RX["delta"])
    wyc = np.zeros(RY["n"]) if periodic else cap_1d(RY["cells"], RY["length"], RY["delta"])
    qd = _param(prm, "full2D_Q_drift", QE / HBAR)
    ds = _param(prm, "full2D_drift_scale", 1.0)
    cs = _param(prm, "full2D_cap_scale", 1.0)
    drift = dict(interp=np.ascontiguousarray(interp), proj=np.ascontiguousarray(proj),
                 xq=np.ascontiguousarray(np.array(xq)), yq=np.ascontiguousarray(np.array(yq)),
                 vx=np.ascontiguousarray(VX.ravel(order="F")), vy=np.ascontiguousarray(VY.ravel(order="F")),
                 pot=1j * ds * qd, capc=ds * cs * qd,
                 cap=np.ascontiguousarray(np.tile(wxc, RY["n"]) + np.repeat(wyc, RX["n"])))
    return drift, len(w)


class Full2DOperator:
    """A = A_diff + G_drift of the reference's Full-2D solver, applied on the GPU.

    ``mat`` carries x, y (nm), dg.params (N_K_X/Y, N_el_X/Y, N_rho_x/y, L_rho_x/y, flux
    and boundary options as in the reference) and optionally me_x_ch; ``V`` is the
    potential [Nx x Ny] on the material grid (V), like get_SysM_full2D(mat, p, Vxy).
    ``tensor_cores``: the dense characteristic |A_x| factor as an FP64 GEMM emulated on
    the tensor cores (default) instead of FP64 CUDA-core kernels.
    """

    def __init__(self, mat, V=None, tensor_cores=True):
        self.lib = _lib.load()
        f = build_factors(mat)
        self.factors = f
        self.mat = mat
        self.V = None
        self.x, self.y, self.n, self.nq = f["x"], f["y"], f["n"], f["nq"]
        self.shape, self.terms, self.drift = f["shape"], f["terms"], f["drift"]
        s = f["shape"]
        AX, AY = f["axes"]
        periodic = bool(s["periodic_y"])
        nrx, nry = s["n_rho_x"], s["n_rho_y"]
        st = _lib.Wg2dShape(s["n_el_x"], s["nk_x"], s["n_el_y"], s["nk_y"], nrx, nry, int(periodic), self.nq,
                            1 if tensor_cores else 0)
        h = C.c_void_p()
        rc = self.lib.wg2d_create(C.byref(st), C.byref(h))
        if rc != _lib.WG_OK:
            raise WignerError(rc, "wg2d_create failed")
        self.h = h
        try:
            for axis, (terms, ax, nr) in enumerate(((self.terms[0], AX, nrx), (self.terms[1], AY, nry))):
                self._set_axis(axis, terms, ax, nr, periodic and axis == 1)
            d = self.drift
            pot = np.array([d["pot"].real, d["pot"].imag])
            self._check(self.lib.wg2d_set_drift(self.h, _lib.dptr(d["interp"]), _lib.dptr(d["proj"]),
                                                _lib.dptr(d["xq"]), _lib.dptr(d["yq"]), _lib.dptr(d["vx"]),
                                                _lib.dptr(d["vy"]), _lib.dptr(pot), float(d["capc"]),
                                                _lib.dptr(d["cap"])))
            if V is not None:
                self.set_potential(V)
        except Exception:
            self.close()
            raise

    def _set_axis(self, axis, terms, ax, nr, periodic):
        if not terms:
            self._check(self.lib.wg2d_set_transport(self.h, axis, 0, None, None, None, None, None))
            return
        coef = np.array([t[0] for t in terms], dtype=float)
        blocks = np.ascontiguousarray(np.stack([_blocks(t[1], ax["nl"], ax["ne"], periodic) for t in terms]))
        rps, cols, vals = [], [], []
        for _, _, R in terms:
            Rs = sp.csr_matrix(R)
            Rs.eliminate_zeros()
            Rs.sort_indices()
            rps.append(Rs.indptr.astype(np.int32))
            cols.append(Rs.indices.astype(np.int32))
            vals.append(Rs.data.astype(complex))
        rp = np.ascontiguousarray(np.concatenate(rps))
        col = np.ascontiguousarray(np.concatenate(cols))
        val = np.ascontiguousarray(np.concatenate(vals)).view(np.float64)
        self._check(self.lib.wg2d_set_transport(self.h, axis, len(terms), _lib.dptr(coef), _lib.dptr(blocks),
                                                rp.ctypes.data_as(C.POINTER(C.c_int)),
                                                col.ctypes.data_as(C.POINTER(C.c_int)), _lib.dptr(val)))

    def observables(self, rho):
        """(n [X nDof x material Ny] m^-3, j [X nDof], nDG, jxDG) of a state
        (get_Observables_full2D.m:19-78): n = real(rho) at zero relative separation (the
        rho_x = 0 cell; the two rho_y cells around 0 weighted linearly), j_x = q hbar / m_x
        imag(d rho / d rho_x) at zero (the central-difference row), projected onto the material
        Y grid (DG values at shared interface nodes averaged, linear interpolation), j the
        trapezoid integral over Y."""
        f = self.factors
        RX, RY = f["rel"]
        AX, AY = f["axes"]
        nrx, nry, nX, nY = RX["n"], RY["n"], AX["nd"], AY["nd"]
        r4 = np.asarray(rho).reshape(nY, nX, nry, nrx)                   # [Y, X, rho_y, rho_x]

        def zero(cells):
            i = int(np.argmin(np.abs(cells)))
            if abs(cells[i]) <= max(1e-14, 1e-12 * max(1.0, np.abs(cells).max())):
                return np.array([i]), np.array([1.0])
            lo, hi = np.flatnonzero(cells < 0)[-1], np.flatnonzero(cells > 0)[0]
            h = cells[hi] - cells[lo]
            return np.array([lo, hi]), np.array([cells[hi] / h, -cells[lo] / h])
        ax_, wx = zero(RX["cells"])
        ay_, wy = zero(RY["cells"])
        at0 = np.einsum("yxab,a,b->xy", r4[:, :, ay_][:, :, :, ax_], wy, wx)   # rho at (0, 0)
        nDG = at0.real
        ix0 = ax_[0] if ax_.size == 1 else None
        if ix0 is not None:
            drow = RX["D"][ix0]
        else:
            drow = np.zeros(nrx)
            h = RX["cells"][ax_[1]] - RX["cells"][ax_[0]]
            drow[ax_[0]], drow[ax_[1]] = -1 / h, 1 / h
        d = np.einsum("yxba,a,b->xy", r4[:, :, ay_, :], drow, wy)
        mex = self.mat.get("me_x_ch", 0.041)
        mkg = mex * M0 if abs(mex) > 1e-25 else mex
        mkg = mkg if mkg > 0 else 0.041 * M0
        jxDG = QE * HBAR / mkg * d.imag
        target = np.asarray(self.mat["y"], dtype=float) * f["scale"]
        ydg = AY["nodes"]
        order = np.argsort(ydg, kind="stable")
        tol = 1e-12 * max(abs(ydg.max() - ydg.min()), 1e-300)
        uy, cols = [], []
        for i in order:
            if uy and ydg[i] - uy[-1] <= tol:
                cols[-1].append(i)
            else:
                uy.append(ydg[i])
                cols.append([i])
        uy = np.asarray(uy)

        def to_y(v):
            a = np.stack([v[:, c].mean(axis=1) for c in cols], axis=1)
            if uy.size == 1:
                return np.repeat(a, target.size, axis=1)
            k = np.clip(np.searchsorted(uy, target, side="right") - 1, 0, uy.size - 2)
            t = (target - uy[k]) / (uy[k + 1] - uy[k])
            return a[:, k] * (1 - t) + a[:, k + 1] * t
        n, jx = to_y(nDG), to_y(jxDG)
        j = np.sum(0.5 * (jx[:, 1:] + jx[:, :-1]) * np.diff(target), axis=1) if target.size > 1 else jx[:, 0]
        return n, j, nDG, jxDG

    def reservoir_rhs(self, EfL, EfR, Vxy=None):
        """The system's right-hand side from the Source/Drain reservoirs (get_SysM_full2D.m's rhs:
        get_InflowBoundary_full2D + the inflow parts of get_Diff_full2D.m:405-430), for the model
        mat.dg.params.full2D_reservoirModel; Vxy defaults to the potential set last.  Returns
        (rhs, inflow) with inflow[side] = (rhoBoundary, info)."""
        from . import reservoir
        V = self.V if Vxy is None else Vxy
        if V is None:
            V = self.mat.get("V", np.zeros((len(self.x), len(self.y))))
        inflow = reservoir.get_InflowBoundary_full2D(self.mat, self.factors, EfL, EfR, V)
        return reservoir.inflow_rhs(self.factors, inflow), inflow

    def set_potential(self, V):
        """Rebuild the potential differences from V [Nx x Ny] on the material grid (device)."""
        V = np.asarray(V, dtype=float)
        if V.ndim == 1:
            V = np.repeat(V[:, None], len(self.y), axis=1) if V.size == len(self.x) else \
                np.repeat(V[None, :], len(self.x), axis=0)
        if V.shape != (len(self.x), len(self.y)):
            raise WignerError(_lib.WG_ERR_ARG, "V must be Nx x Ny")
        Vc = np.ascontiguousarray(V.ravel(order="F"))
        self._check(self.lib.wg2d_set_potential(self.h, len(self.x), len(self.y), _lib.dptr(self.x),
                                                _lib.dptr(self.y), _lib.dptr(Vc)))
        self.V = V

    def set_preconditioner(self, ix=0, fp32=True):
        """Build the line-transverse preconditioner for the current potential (reference
        column ix of the material grid) and hand it to the device; fp32: apply it in FP32
        (the flexible GMRES keeps the solve's FP64 accuracy)."""
        pre = build_preconditioner(self.mat, self.V, self.factors, ix)
        self.pre = pre
        U = np.ascontiguousarray(pre["U"], dtype=complex)
        xi = np.ascontiguousarray(pre["xinv"], dtype=complex)
        xc = np.ascontiguousarray(pre["xcpl"], dtype=complex)
        ti = np.ascontiguousarray(pre["tinv"], dtype=complex)
        fw = np.ascontiguousarray(pre["fwd"], dtype=np.int32)
        self._check(self.lib.wg2d_set_preconditioner(self.h, _lib.dptr(U.view(np.float64)), float(pre["sigma"]),
                                                     _lib.dptr(xi.view(np.float64)), _lib.dptr(xc.view(np.float64)),
                                                     fw.ctypes.data_as(C.POINTER(C.c_int)),
                                                     _lib.dptr(ti.view(np.float64)), 1 if fp32 else 0))

    def precondition(self, r):
        r = np.ascontiguousarray(np.asarray(r, dtype=complex).reshape(-1))
        out = np.empty_like(r)
        self._check(self.lib.wg2d_precondition(self.h, r.view(np.float64).ctypes.data_as(_lib._D),
                                               out.view(np.float64).ctypes.data_as(_lib._D)))
        return out

    def solve(self, rhs, x0=None, tol=1e-8, maxit=50, restart=40, mixed=False, inner_tol=1e-3):
        """rho = A \\ rhs by right-preconditioned flexible GMRES(restart) on the device; mixed: FP64
        refinement around FP32 inner solves (FP32 preconditioner required).  Returns (status, info, rho)."""
        b = np.ascontiguousarray(np.asarray(rhs, dtype=complex).reshape(-1))
        x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(np.asarray(x0, dtype=complex).reshape(-1))
        if b.size != self.n or x.size != self.n:
            raise WignerError(_lib.WG_ERR_ARG, "rhs and x0 need %d entries" % self.n)
        opts = _lib.Wg2dSolveOpts(float(tol), int(maxit), int(restart), 0 if x0 is None else 1, 1 if mixed else 0,
                                  float(inner_tol))
        info = _lib.Wg2dSolveInfo()
        st = self.lib.wg2d_solve(self.h, b.view(np.float64).ctypes.data_as(_lib._D),
                                 x.view(np.float64).ctypes.data_as(_lib._D), C.byref(opts), C.byref(info))
        if st not in (_lib.WG_OK, _lib.WG_NOT_CONVERGED):
            self._check(st)
        return st, info.as_dict(), x

    def apply(self, u):
        """y = A u (complex vector in the reference's order rho_x, rho_y, X, Y)."""
        u = np.ascontiguousarray(np.asarray(u, dtype=complex).reshape(-1))
        if u.size != self.n:
            raise WignerError(_lib.WG_ERR_ARG, "u needs %d entries" % self.n)
        out = np.empty_like(u)
        self._check(self.lib.wg2d_apply(self.h, u.view(np.float64).ctypes.data_as(_lib._D),
                                        out.view(np.float64).ctypes.data_as(_lib._D)))
        return out

    def apply_time(self, n=10):
        """Mean device time [ms] of one apply and of its (transport, potential) parts."""
        ms = C.c_double()
        parts = np.zeros(2)
        self._check(self.lib.wg2d_apply_repeat(self.h, int(n), C.byref(ms), _lib.dptr(parts)))
        return ms.value, parts

    def _check(self, rc):
        if rc != _lib.WG_OK:
            raise WignerError(rc, self.lib.wg2d_last_error(self.h).decode() if getattr(self, "h", None) else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.wg2d_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
