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

Supported: source/drain faces fully open, Y boundaries 'periodic', 'zero-inflow',
'specular' and 'hard-wall' (the two-point Dirichlet constraint of
constrain_HardWall_full2D.m on the complete operator, its right-hand side and the
preconditioner's transverse blocks), X/Y fluxes 'upwind', 'rusanov', 'central',
constant mass.
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
            "zero_inflow": "zero-inflow", "zeroinflow": "zero-inflow", "zero": "zero-inflow",
            "hardwall": "hard-wall", "hard_wall": "hard-wall", "dirichlet": "hard-wall"}.get(v, v)


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
    if ytype not in ("periodic", "zero-inflow", "specular", "hard-wall"):
        raise WignerError(_lib.WG_ERR_ARG, 'Unknown full2D_Y_boundary "%s". Use "specular" or "zero-inflow", '
                          '"hard-wall" or "periodic".' % ytype, "DG:Full2D:UnknownYBoundaryType")
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
    if ytype not in ("periodic", "hard-wall"):
        ty.append((sy, oy["HB"], absy))
    if ytype == "specular":
        flip = np.fliplr(np.eye(nry))
        ty.append((-sy, oy["lb"], Apy @ flip))
        ty.append((sy, oy["rb"], Amy @ flip))
    drift, nq = _drift_setup(prm, AX, AY, RX, RY, periodic)
    wall = _hard_wall(AX, AY, RX, RY, y, (sx, sy)) if ytype == "hard-wall" else None
    # closed pieces of the outer X faces (get_Diff_full2D.m:393-423): the incoming characteristics there
    # are the rho_x-reflected interior state, a correction on the masked-off Y dofs only
    masks = {side: contact_mask(mat, AY, y, side, scale) for side in ("source", "drain")}
    flip = np.fliplr(np.eye(nrx))
    closed = []
    for side, sign, lift, Ach in (("source", -1.0, ox["lb"], Apx), ("drain", 1.0, ox["rb"], Amx)):
        if not masks[side].all() and sx != 0:
            closed.append((sign * sx, lift, Ach @ flip, ~masks[side]))
    return dict(shape=dict(n_el_x=nex, nk_x=nkx, n_el_y=ney, nk_y=nky, n_rho_x=nrx, n_rho_y=nry,
                           periodic_y=int(periodic)),
                n=nrx * nry * nex * nkx * ney * nky, x=x, y=y, terms=(_merge(tx), _merge(ty)), axes=(AX, AY),
                rel=(RX, RY), scales=(sx, sy), drift=drift, nq=nq, split=(Apx, Amx, Apy, Amy), ytype=ytype,
                scale=scale, wall=wall, contact_masks=masks, closed_terms=closed)


def _nearest(values, grid, target):
    """interp1(grid, values, target, 'nearest', 'extrap'), a target halfway between two grid points
    taking the upper one."""
    grid = np.asarray(grid, dtype=float)
    target = np.asarray(target, dtype=float)
    lo = np.clip(np.searchsorted(grid, target, side="right") - 1, 0, len(grid) - 1)
    hi = np.minimum(lo + 1, len(grid) - 1)
    up = (hi > lo) & (target - grid[lo] >= grid[hi] - target)
    return np.asarray(values)[np.where(up, hi, lo)]


def contact_mask(mat, AY, y, side, scale):
    """The Y dofs of the outer X face at ``side`` that receive reservoir inflow
    (get_ContactMask_full2D.m:14-120); the others are closed.  In order: an explicit
    full2D_<side>ContactMask (per face dof, or per material y point taken to the nearest), the
    doping of the edge column above full2D_contactNdThreshold, the material gap (Eg below the middle
    of Eg_c and Eg_ox) or the W_c / W_cy geometry, the whole face; an empty mask falls back to the
    material / geometry rule."""
    prm = mat["dg"]["params"]
    y_face = AY["nodes"]
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    ix = 0 if side == "source" else nx - 1

    def xy(field):
        a = np.squeeze(np.asarray(field, dtype=float))
        if a.shape == (nx, ny):
            return a
        if a.shape == (ny, nx):
            return a.T
        if a.ndim == 1 and a.size in (nx, ny):
            return np.repeat(a[:, None], ny, axis=1) if a.size == nx else np.repeat(a[None, :], nx, axis=0)
        raise WignerError(_lib.WG_ERR_ARG, "Cannot interpret material field with size %s as an X/Y field."
                          % (a.shape,), "DG:Full2D:InvalidMaterialField")

    def material():
        if mat.get("Eg") is not None and mat.get("Eg_ox") is not None:
            eg = xy(mat["Eg"])
            thr = 0.5 * (float(mat.get("Eg_c", eg.min())) + float(mat["Eg_ox"]))
            return _nearest(eg[ix] < thr, y, y_face).astype(bool)
        for wo, wc in (("W_ox", "W_c"), ("W_oxy", "W_cy")):
            if wo in mat and wc in mat:
                return (y_face >= 0) & (y_face <= float(mat[wc]) * scale)
        return np.ones(y_face.size, dtype=bool)

    explicit = prm.get("full2D_%sContactMask" % side)
    if explicit is not None and np.size(explicit) > 0:
        m = np.ravel(np.asarray(explicit))
        if m.size == y_face.size:
            mask = m.astype(bool)
        elif m.size == ny:
            mask = _nearest(m.astype(float), y, y_face) > 0.5
        else:
            raise WignerError(_lib.WG_ERR_ARG, "Contact mask has %d entries, expected %d face DOFs or mat.Ny "
                              "entries." % (m.size, y_face.size), "DG:Full2D:InvalidContactMask")
    elif mat.get("Nd") is not None and np.size(mat["Nd"]) > 0:
        thr = float(prm.get("full2D_contactNdThreshold", 0.0) or 0.0)
        mask = _nearest((xy(mat["Nd"])[ix] > thr).astype(float), y, y_face) > 0.5
    else:
        mask = material()
    if not mask.any():
        mask = material()
    return np.asarray(mask, dtype=bool)


def wall_project(f, v):
    """T v: the hard-wall projection on the (rho_y, Y) index of a state (applyTransverse of
    constrain_HardWall_full2D.m:52-57)."""
    s = f["shape"]
    ne, nl, nX = s["n_el_y"], s["nk_y"], s["n_el_x"] * s["nk_x"]
    v5 = np.asarray(v, dtype=complex).reshape(ne, nl, nX, s["n_rho_y"], s["n_rho_x"])
    return np.einsum("erAj,ejxrq->eAxrq", f["wall"]["blocks"], v5).reshape(-1)


def _hard_wall(AX, AY, RX, RY, y, scales):
    """Hard-wall geometry (get_HardWallGeometry_full2D.m:15-48, constrain_HardWall_full2D.m:10-18):
    active [n_rho_y, nY] (both particle coordinates Y +- rho_y/2 strictly inside [y0, y1], 64 ulp
    of the largest coordinate as margin), the exact-DG-mass projection per (Y element, rho_y cell)
    as blocks [n_el_y, n_rho_y, nk_y, nk_y] (zero rows for inactive nodes) and the weight of the
    constraint rows."""
    rho, Y = RY["cells"], AY["nodes"]
    big = max(abs(y[0]), abs(y[-1]), float(np.max(np.abs(rho))))
    dist = np.minimum(Y - y[0], y[-1] - Y)
    active = np.abs(rho)[:, None] / 2 < dist[None, :] - 64 * np.spacing(big)
    if not active.any():
        raise WignerError(_lib.WG_ERR_ARG, "No Y/rho_y samples lie inside the hard walls. Refine these grids.",
                          "DG:Full2D:HardWallEmptyDomain")
    nl, ne, nr = AY["nl"], AY["ne"], len(rho)
    M = AY["M"]
    blocks = np.zeros((ne, nr, nl, nl))
    for e in range(ne):
        for ir in range(nr):
            keep = active[ir, e * nl:(e + 1) * nl]
            if keep.any():
                blocks[e, ir][keep] = np.linalg.solve(M[np.ix_(keep, keep)], M[keep, :])
    sx, sy = scales
    g = max(1.0, abs(sx) / (np.min(np.diff(AX["verts"])) * RX["delta"])
            + abs(sy) / (np.min(np.diff(AY["verts"])) * RY["delta"]))
    return dict(active=active, blocks=blocks, scale=g)


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
    wall = f.get("wall")
    if wall is not None:       # get_LineTransversePreconditioner_full2D.m:84-88: T B P + scale (I - P)
        act = wall["active"].T.reshape(-1).astype(float)           # index rho_y + n_rho_y Y
        Tm = np.zeros((nT, nT))
        nl = AY["nl"]
        for e in range(AY["ne"]):
            for ir in range(nry):
                ids = ir + nry * (e * nl + np.arange(nl))
                Tm[np.ix_(ids, ids)] = wall["blocks"][e, ir]
    tinv = np.empty((nm, nT, nT), dtype=complex)
    for k in range(nm):
        B = K + pw[k] * Vt + np.diag(capY + capX[k])
        if wall is not None:
            B = (Tm @ B) * act[None, :] + np.diag(wall["scale"] * (1 - act))
        tinv[k] = np.linalg.inv(B / sigma + np.eye(nT))
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


def _zero_weights(cells):
    """Cells and weights of the value at zero relative separation (zeroInterpolationWeights of
    get_Observables_full2D.m:81-103): the cell at zero, else the two bracketing cells linearly,
    else the nearest cell."""
    cells = np.asarray(cells, dtype=float)
    i = int(np.argmin(np.abs(cells)))
    if abs(cells[i]) <= max(1e-14, 1e-12 * max(1.0, np.abs(cells).max())):
        return [i], [1.0]
    neg, pos = np.flatnonzero(cells < 0), np.flatnonzero(cells > 0)
    if neg.size and pos.size:
        lo, hi = int(neg[-1]), int(pos[0])
        h = cells[hi] - cells[lo]
        return [lo, hi], [cells[hi] / h, -cells[lo] / h]
    return [i], [1.0]


def _derivative_row(cells, D):
    """The derivative at zero relative separation as a sparse row (derivativeRowAtZero of
    get_Observables_full2D.m:105-135): the row of D at a zero cell, else a difference of the
    bracketing (or the nearest one-sided) cells."""
    cells = np.asarray(cells, dtype=float)
    n = cells.size
    i = int(np.argmin(np.abs(cells)))
    row = np.zeros(n)
    if abs(cells[i]) <= max(1e-14, 1e-12 * max(1.0, np.abs(cells).max())):
        row = np.asarray(D[i], dtype=float).ravel().copy()
    else:
        neg, pos = np.flatnonzero(cells < 0), np.flatnonzero(cells > 0)
        if neg.size and pos.size:
            lo, hi = int(neg[-1]), int(pos[0])
        elif i == 0:
            lo, hi = 0, 1
        elif i == n - 1:
            lo, hi = n - 2, n - 1
        else:
            lo, hi = i - 1, i + 1
        h = cells[hi] - cells[lo]
        row[lo], row[hi] = -1 / h, 1 / h
    nz = np.flatnonzero(row)
    return [int(k) for k in nz], [float(row[k]) for k in nz]


def _y_projection(ydg, target):
    """W [n_target x nY] with (W v) = v averaged over duplicate DG Y nodes and linearly
    interpolated (extrapolated) to the target points (projectValuesToY), and the trapezoid
    weights over the target points (integrateOverY; the single point itself when there is one)."""
    ydg = np.asarray(ydg, dtype=float)
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
    A = np.zeros((uy.size, ydg.size))
    for g, c in enumerate(cols):
        A[g, c] = 1.0 / len(c)
    if uy.size == 1:
        W = np.repeat(A, target.size, axis=0)
    else:
        k = np.clip(np.searchsorted(uy, target, side="right") - 1, 0, uy.size - 2)
        t = (target - uy[k]) / (uy[k + 1] - uy[k])
        W = A[k] * (1 - t)[:, None] + A[k + 1] * t[:, None]
    if target.size > 1:
        d = np.diff(target)
        wj = np.zeros(target.size)
        wj[:-1] += 0.5 * d
        wj[1:] += 0.5 * d
    else:
        wj = np.ones(1)
    return np.ascontiguousarray(W), wj


class Full2DOperator:
    """A = A_diff + G_drift of the reference's Full-2D solver, applied on the GPU.

    ``mat`` carries x, y (nm), dg.params (N_K_X/Y, N_el_X/Y, N_rho_x/y, L_rho_x/y, flux
    and boundary options as in the reference) and optionally me_x_ch; ``V`` is the
    potential [Nx x Ny] on the material grid (V), like get_SysM_full2D(mat, p, Vxy).
    ``tensor_cores``: the dense characteristic |A_x| factor as an FP64 GEMM emulated on
    the tensor cores (default) instead of FP64 CUDA-core kernels.
    """

    def __init__(self, mat, V=None, tensor_cores=True, factors=None):
        self.lib = _lib.load()
        f = build_factors(mat) if factors is None else factors
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
            closed = f.get("closed_terms") or []
            xterms = list(self.terms[0]) + [t[:3] for t in closed]
            for axis, (terms, ax, nr) in enumerate(((xterms, AX, nrx), (self.terms[1], AY, nry))):
                self._set_axis(axis, terms, ax, nr, periodic and axis == 1)
            if closed:       # the closed-face corrections act on their masked-off Y dofs only
                masks = np.ones((len(xterms), AY["nd"]), dtype=np.uint8)
                for i, t in enumerate(closed):
                    masks[len(self.terms[0]) + i] = t[3].astype(np.uint8)
                masks = np.ascontiguousarray(masks)
                self._check(self.lib.wg2d_set_transport_masks(self.h, 0, len(xterms),
                                                              masks.ctypes.data_as(C.c_void_p)))
            d = self.drift
            pot = np.array([d["pot"].real, d["pot"].imag])
            self._check(self.lib.wg2d_set_drift(self.h, _lib.dptr(d["interp"]), _lib.dptr(d["proj"]),
                                                _lib.dptr(d["xq"]), _lib.dptr(d["yq"]), _lib.dptr(d["vx"]),
                                                _lib.dptr(d["vy"]), _lib.dptr(pot), float(d["capc"]),
                                                _lib.dptr(d["cap"])))
            w = f.get("wall")
            if w is not None:
                act = np.ascontiguousarray(w["active"].T, dtype=np.uint8)          # [nY][n_rho_y]
                blk = np.ascontiguousarray(w["blocks"], dtype=float)
                self._check(self.lib.wg2d_set_hard_wall(self.h, act.ctypes.data_as(C.c_void_p), _lib.dptr(blk),
                                                        float(w["scale"])))
            self._set_observables()
            if V is not None:
                self.set_potential(V)
        except Exception:
            self.close()
            raise

    def _set_observables(self):
        """Hand the zero-separation weights, derivative rows and the material-Y projection of
        get_Observables_full2D.m to the device (once per handle)."""
        f = self.factors
        RX, RY = f["rel"]
        AX, AY = f["axes"]
        d = _lib.Wg2dObservablesDesc()
        zx, wx = _zero_weights(RX["cells"])
        zy, wy = _zero_weights(RY["cells"])
        dxi, dxv = _derivative_row(RX["cells"], RX["D"])
        dyi, dyv = _derivative_row(RY["cells"], RY["D"])
        if len(dxi) > 8 or len(dyi) > 8:
            raise WignerError(_lib.WG_ERR_ARG, "derivative rows with more than 8 nonzeros")
        d.n_zero_x, d.n_zero_y, d.n_dx, d.n_dy = len(zx), len(zy), len(dxi), len(dyi)
        for i, (a, w) in enumerate(zip(zx, wx)):
            d.zero_x[i], d.w_zero_x[i] = a, w
        for i, (a, w) in enumerate(zip(zy, wy)):
            d.zero_y[i], d.w_zero_y[i] = a, w
        for i, (a, v) in enumerate(zip(dxi, dxv)):
            d.dx_idx[i], d.dx_val[i] = a, v
        for i, (a, v) in enumerate(zip(dyi, dyv)):
            d.dy_idx[i], d.dy_val[i] = a, v

        def kg(m):                          # massToKg
            mk = m * M0 if abs(m) > 1e-25 else m
            return mk if mk > 0 else 0.041 * M0
        mex = self.mat.get("me_x_ch", 0.041)
        d.scale_x = QE * HBAR / kg(mex)
        d.scale_y = QE * HBAR / kg(self.mat.get("me_y_ch", mex))
        target = np.asarray(self.mat["y"], dtype=float) * f["scale"]
        W, wj = _y_projection(AY["nodes"], target)
        d.n_target_y = target.size
        self.target_y = target
        self._check(self.lib.wg2d_set_observables(self.h, C.byref(d), _lib.dptr(W), _lib.dptr(np.ascontiguousarray(wj))))

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

    def observables(self, rho=None):
        """(n [X nDof x material Ny] m^-3, j [X nDof], nDG, jxDG) of a state (get_Observables_full2D.m:19-78),
        computed on the device: n = real(rho) at zero relative separation (the rho_x = 0 cell; the two
        rho_y cells around 0 weighted linearly), j_x = q hbar / m_x imag(d rho / d rho_x) at zero (the
        central-difference row), projected onto the material Y grid (DG values at shared interface
        nodes averaged, linear interpolation), j the trapezoid integral over Y.  rho = None: the
        solution resident on the device (no copy of the state crosses to the host)."""
        o = self.observables_all(rho)
        return o["n"], o["j"], o["nDG"], o["jxDG"]

    def observables_all(self, rho=None):
        """Every observable of get_Observables_full2D.m: n, jx, jy [X nDof x Ny], j, and the DG values
        nDG, jxDG, jyDG [X nDof x Y nDof], y (the material Y points, m); see observables()."""
        AX, AY = self.factors["axes"]
        nX, nY, nty = AX["nd"], AY["nd"], self.target_y.size
        out = {k: np.empty((nX, nY)) for k in ("nDG", "jxDG", "jyDG")}
        out.update({k: np.empty((nX, nty)) for k in ("n", "jx", "jy")})
        out["j"] = np.empty(nX)
        r = None
        if rho is not None:
            r = np.ascontiguousarray(np.asarray(rho, dtype=complex).reshape(-1))
            if r.size != self.n:
                raise WignerError(_lib.WG_ERR_ARG, "rho has %d entries, expected %d" % (r.size, self.n),
                                  "DG:Full2D:InvalidObservableInput")
        self._check(self.lib.wg2d_observables(self.h, None if r is None else r.view(np.float64).ctypes.data_as(_lib._D),
                                              *[_lib.dptr(out[k]) for k in ("nDG", "jxDG", "jyDG", "n", "jx", "jy",
                                                                            "j")]))
        out["y"] = self.target_y
        return out

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
        rhs = reservoir.inflow_rhs(self.factors, inflow)
        if self.factors.get("wall") is not None:
            rhs = wall_project(self.factors, rhs)      # the constrained system's rhs, T b
        return rhs, inflow

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

    def solve(self, rhs, x0=None, tol=1e-8, maxit=50, restart=40, mixed=False, inner_tol=1e-3, resident=False,
              warm=False, inner_basis_fp16=False):
        """rho = A \\ rhs by right-preconditioned flexible GMRES(restart) on the device; mixed: FP64
        refinement around FP32 inner solves (FP32 preconditioner required; the inner basis in FP32, or
        stored in FP16 with inner_basis_fp16).  Returns (status, info, rho).
        resident: the solution stays on the device only (rho is None; observables() and state() read it),
        warm: the warm start is the resident solution of the previous solve (x0 ignored), rhs = None:
        the right-hand side of the previous solve."""
        b = None
        if rhs is not None:
            b = np.ascontiguousarray(np.asarray(rhs, dtype=complex).reshape(-1))
            if b.size != self.n:
                raise WignerError(_lib.WG_ERR_ARG, "rhs needs %d entries" % self.n)
        x = None
        if not warm and (x0 is not None or not resident):
            x = np.zeros(self.n, dtype=complex)
            if x0 is not None:
                x0 = np.asarray(x0, dtype=complex).reshape(-1)
                if x0.size != self.n:
                    raise WignerError(_lib.WG_ERR_ARG, "x0 needs %d entries" % self.n)
                x[:] = x0
        use_x0 = 1 if (warm or x0 is not None) else 0
        opts = _lib.Wg2dSolveOpts(float(tol), int(maxit), int(restart), use_x0, 1 if mixed else 0, float(inner_tol),
                                  1 if inner_basis_fp16 else 0)
        info = _lib.Wg2dSolveInfo()
        st = self.lib.wg2d_solve(self.h, None if b is None else b.view(np.float64).ctypes.data_as(_lib._D),
                                 None if x is None else x.view(np.float64).ctypes.data_as(_lib._D),
                                 C.byref(opts), C.byref(info))
        if st not in (_lib.WG_OK, _lib.WG_NOT_CONVERGED):
            self._check(st)
        if resident:
            return st, info.as_dict(), None
        return st, info.as_dict(), (self.state() if x is None else x)

    def solve_bicgstab(self, rhs, x0=None, tol=1e-8, maxit=100, resident=False):
        """rho = A \\ rhs by preconditioned BiCGSTAB on the device (the line-transverse preconditioner when
        one is set, none otherwise).  Returns (status, info, rho); info["cycles"] counts half steps."""
        b = None
        if rhs is not None:
            b = np.ascontiguousarray(np.asarray(rhs, dtype=complex).reshape(-1))
            if b.size != self.n:
                raise WignerError(_lib.WG_ERR_ARG, "rhs needs %d entries" % self.n)
        x = None if (resident and x0 is None) else np.zeros(self.n, dtype=complex)
        if x0 is not None:
            x[:] = np.asarray(x0, dtype=complex).reshape(-1)
        opts = _lib.Wg2dSolveOpts(float(tol), int(maxit), 0, 1 if x0 is not None else 0, 0, 0.0)
        info = _lib.Wg2dSolveInfo()
        st = self.lib.wg2d_solve_bicgstab(self.h, None if b is None else b.view(np.float64).ctypes.data_as(_lib._D),
                                          None if x is None else x.view(np.float64).ctypes.data_as(_lib._D),
                                          C.byref(opts), C.byref(info))
        if st not in (_lib.WG_OK, _lib.WG_NOT_CONVERGED):
            self._check(st)
        return st, info.as_dict(), (None if resident else x)

    def state(self):
        """The resident solution of the last solve (host copy)."""
        x = np.empty(self.n, dtype=complex)
        self._check(self.lib.wg2d_get_state(self.h, x.view(np.float64).ctypes.data_as(_lib._D)))
        return x

    def resvec(self):
        """Residual norms of the last solve: the initial true residual, then the GMRES estimate after
        every inner iteration (DG.info.solve.resvec)."""
        n = C.c_int()
        self._check(self.lib.wg2d_solve_resvec(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        if n.value:
            self._check(self.lib.wg2d_solve_resvec(self.h, _lib.dptr(out), n.value, C.byref(n)))
        return out

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


_SOLVE_ON = ("true", "yes", "on", "solve", "always")
_SOLVE_OFF = ("false", "no", "off", "operator-only", "skip", "never")


def _should_solve(mode, n, max_auto):
    """shouldSolve of solve_transport_DG_full2D.m:1249-1279: (solve?, status when skipped)."""
    if isinstance(mode, (bool, np.bool_)):
        return bool(mode), "operator-ready-solve-disabled"
    if isinstance(mode, (int, float, np.number)):
        return mode != 0, "operator-ready-solve-disabled"
    m = str(mode).strip().lower()
    if m == "auto":
        return n <= max_auto, "operator-ready-solve-skipped-size"
    if m in _SOLVE_ON:
        return True, ""
    if m in _SOLVE_OFF:
        return False, "operator-ready-solve-disabled"
    raise WignerError(_lib.WG_ERR_ARG, 'Unknown full2D_solve mode "%s".' % mode, "DG:Full2D:UnknownSolveMode")


def _store_rho_array(prm, n):
    """shouldStoreRHOArray (solve_transport_DG_full2D.m:1309-1330)."""
    mode = prm.get("full2D_storeRHOArray", "auto")
    if isinstance(mode, (bool, np.bool_, int, float, np.number)):
        return bool(mode)
    m = str(mode).strip().lower()
    if m == "auto":
        return n <= float(prm.get("full2D_maxStoredRHOArrayDof", 2e6))
    if m in ("true", "yes", "on", "store", "always"):
        return True
    if m in ("false", "no", "off", "never"):
        return False
    raise WignerError(_lib.WG_ERR_ARG, 'Unknown full2D_storeRHOArray mode "%s".' % mode,
                      "DG:Full2D:UnknownStorageMode")


def _initial_rho(rho0, n):
    """validateInitialRho (solve_transport_DG_full2D.m:508-527)."""
    if rho0 is None:
        return None
    r = np.asarray(rho0)
    if r.size == 0:
        return None
    if r.dtype.kind not in "fc" or (r.ndim > 1 and sum(d > 1 for d in r.shape) > 1) or r.size != n:
        raise WignerError(_lib.WG_ERR_ARG, "rho0 must be a full single/double vector with %d entries in "
                          "rho_x,rho_y,X,Y order." % n, "DG:Full2D:InvalidInitialRho")
    r = r.reshape(-1).astype(complex)
    if not np.all(np.isfinite(r)):
        raise WignerError(_lib.WG_ERR_ARG, "rho0 must contain only finite values.", "DG:Full2D:InvalidInitialRho")
    return r


def solve_transport_DG_full2D(mat, Vxy=None, EfL=None, EfR=None, rho0=None):
    """DG = solve_transport_DG_full2D(mat, Vxy, EfL, EfR, rho0) (DG_code/solve_transport_DG_full2D.m:1-130)
    with the operator, the preconditioner, the Krylov solve and the observables on the GPU.

    Follows solveStationarySystem (:132-346): the full2D_solve mode (auto: solve up to
    full2D_maxAutoSolveDof unknowns), full2D_solverTol (default 1e-4) relative to |rhs|,
    full2D_solverMaxIt (default 1400; restart cycles for GMRES, iterations for BiCGSTAB), the
    GMRES restart full2D_gmresRestart (default full2D_gpuGmresRestart, 20), the basis-memory guard
    (DG:Full2D:GmresMemoryLimit, full2D_gmresMaxBasisBytes, default 9 GiB), the warm start rho0 as
    a right-preconditioned correction (GMRES only, DG:Full2D:InitialRhoSolver otherwise), the
    independent true-residual check and iterativeStatus.  Solvers: 'gmres' (flexible GMRES,
    right-preconditioned) and 'bicgstab'; 'auto' selects GMRES with the line-transverse
    preconditioner (the reference's GPU default is BiCGSTAB with the Jacobi diagonal, which is not
    built); 'direct' raises DG:Full2D:GPUDirectSolverUnsupported as the reference does on the GPU.
    Preconditioners: 'line-transverse' (and 'auto'), 'none'; the host-side ones (jacobi, rowabs,
    blockjacobi) raise DG:Full2D:UnsupportedPreconditioner.  Returns a dict with the reference's
    DG fields: status, rho, RHO (when stored), n, jx, jy, j, nDG, jxDG, jyDG, y, chi, yDG, rho_x,
    rho_y, xi, and info.solve (flag, relres, trueRelres, reportedRelres, iterations, resvec,
    initialGuess, rhsNormalization, tolerance, maxIterations, solver, preconditioner, status, ...).
    """
    import time
    prm = mat["dg"]["params"]
    V = mat.get("V") if Vxy is None else Vxy
    if V is None:
        V = np.zeros((len(np.asarray(mat["x"])), len(np.asarray(mat["y"]))))
    f = build_factors(mat)
    n = f["n"]
    # every argument and option is checked before the device operator is built (validateInitialRho
    # runs before get_SysM_full2D in the reference)
    rho0 = _initial_rho(rho0, n)
    info = dict(requestedMode=prm.get("full2D_solve", "auto"), nTotal=n, matrixAssembled=False,
                matrixFreeAvailable=True, tolerance=float(prm.get("full2D_solverTol", 1e-4)),
                maxIterations=int(prm.get("full2D_solverMaxIt", 1400)))
    do, skip = _should_solve(info["requestedMode"], n, float(prm.get("full2D_maxAutoSolveDof", 1e7)))
    if do and n > float(prm.get("full2D_maxMatrixFreeSolveDof", 2e7)):
        do, skip = False, "operator-ready-solve-skipped-matrix-free-limit"
    solver = pmode = None
    restart = int(prm.get("full2D_gmresRestart", prm.get("full2D_gpuGmresRestart", 20)))
    if do:
        solver = str(prm.get("full2D_solver", "auto")).strip().lower()
        solver = "gmres" if solver == "auto" else solver
        if solver == "direct":
            raise WignerError(_lib.WG_ERR_ARG, "full2D_gpu=true supports full2D_solver='bicgstab' or 'gmres'. "
                              "Select one of these matrix-free Krylov solvers.", "DG:Full2D:GPUDirectSolverUnsupported")
        if solver not in ("gmres", "bicgstab"):
            raise WignerError(_lib.WG_ERR_ARG, 'Unknown full2D_solver "%s". Use auto, direct, bicgstab or gmres.'
                              % solver, "DG:Full2D:UnknownSolver")
        if rho0 is not None and solver != "gmres":
            raise WignerError(_lib.WG_ERR_ARG, "A supplied rho0 currently requires full2D_solver='gmres'.",
                              "DG:Full2D:InitialRhoSolver")
        info["solver"] = solver
        pmode = str(prm.get("full2D_preconditioner", "auto")).strip().lower().replace("_", "-")
        if pmode in ("auto", "line-transverse", "linetransverse"):
            pmode = "line-transverse"
        elif pmode in ("none", "off", "false", "no"):
            pmode = "none"
        elif pmode in ("jacobi", "diagonal", "rowabs", "rowsum", "row-sum", "row-scaling", "blockjacobi",
                       "block-jacobi", "rho-block-jacobi", "relative-block-jacobi", "rho-blockjacobi"):
            raise WignerError(_lib.WG_ERR_ARG, "full2D_preconditioner '%s' is a host-side preconditioner of the "
                              "CPU path; the device path offers line-transverse and none" % pmode,
                              "DG:Full2D:UnsupportedPreconditioner")
        else:
            raise WignerError(_lib.WG_ERR_ARG, 'Unknown full2D_preconditioner "%s".' % pmode,
                              "DG:Full2D:UnknownPreconditioner")
        if solver == "gmres":
            info["gmresBasisBytesEstimate"] = 16.0 * n * (min(restart, n) + 1)
            limit = float(prm.get("full2D_gmresMaxBasisBytes", 9 * 1024 ** 3))
            if info["gmresBasisBytesEstimate"] > limit:
                raise WignerError(_lib.WG_ERR_OOM, "Estimated GMRES basis %.3g GiB exceeds full2D_gmresMaxBasisBytes. "
                                  "Reduce restart or explicitly increase the memory budget."
                                  % (info["gmresBasisBytesEstimate"] / 1024 ** 3), "DG:Full2D:GmresMemoryLimit")
            info["gmresRestart"] = restart
            info["preconditionerSide"] = "right"
    AX, AY = f["axes"]
    RX, RY = f["rel"]
    fx, fy = _flux(prm)
    DG = dict(basis="rho-full2D", flux=fx, fluxX=fx, fluxY=fy, yBoundaryType=f["ytype"], massModel="constant",
              coordinates=("rho_x", "rho_y", "X", "Y"), chi=AX["nodes"].copy(), yDG=AY["nodes"].copy(),
              rho_x=RX["cells"].copy(), rho_y=RY["cells"].copy(), xi=RX["cells"].copy(),
              arraySize=(RX["n"], RY["n"], AX["nd"], AY["nd"]))
    op = Full2DOperator(mat, V, tensor_cores=bool(prm.get("full2D_tensorCores", True)), factors=f)
    try:
        rho = None
        if not do:
            info["status"] = skip
            info["reason"] = "Operator is ready but no solve was run. nTotal=%d." % n
        else:
            t0 = time.perf_counter()
            fp32 = str(prm.get("full2D_preconditionerPrecision", "single")).lower() in ("single", "fp32", "float")
            if pmode == "line-transverse":
                op.set_preconditioner(fp32=fp32)
            info["preconditioner"] = dict(method=pmode, enabled=pmode != "none", executionDevice="gpu",
                                          precision="fp32" if fp32 else "fp64")
            info["preconditionerSetupSeconds"] = time.perf_counter() - t0
            rhs, inflow = op.reservoir_rhs(EfL, EfR, V)
            DG["boundary"] = {side: {"rhoBoundary": rb, "info": inf} for side, (rb, inf) in inflow.items()}
            bnorm = float(np.linalg.norm(rhs))
            t0 = time.perf_counter()
            if solver == "gmres":
                st, sinfo, rho = op.solve(rhs, x0=rho0, tol=info["tolerance"], maxit=info["maxIterations"],
                                          restart=restart, mixed=bool(prm.get("full2D_mixedPrecision", False)))
            else:
                st, sinfo, rho = op.solve_bicgstab(rhs, tol=info["tolerance"], maxit=info["maxIterations"])
            info["iterationSeconds"] = time.perf_counter() - t0
            resvec = op.resvec()
            flag = int(sinfo["flag"])
            r0 = sinfo["initial_relres"]
            init = dict(provided=rho0 is not None, used=rho0 is not None, basis="physical-rho",
                        strategy="zero-start", initialTrueRelres=r0, convergedAtStart=False,
                        correctionTolerance=float("nan"))
            if rho0 is not None:
                if r0 <= info["tolerance"]:
                    init["convergedAtStart"] = True
                    init["strategy"] = "native-x0"
                else:
                    init["strategy"] = "right-preconditioned-correction"
                    init["correctionTolerance"] = max(np.finfo(float).tiny, info["tolerance"] / r0)
            if bnorm == 0:
                init["used"] = False
                init["strategy"] = "homogeneous-rhs-zero-solution"
            info["initialGuess"] = init
            info["rhsNormalization"] = bnorm if bnorm > 0 else 1.0
            info["trueRelres"] = sinfo["relres"]
            info["reportedRelres"] = float(resvec[-1] / bnorm) if bnorm > 0 and resvec.size else sinfo["relres"]
            info["krylovFlag"] = flag
            info["flag"] = flag
            info["relres"] = sinfo["relres"]
            if solver == "gmres":
                info["iterations"] = [int(sinfo["cycles"]), int(sinfo["iterations"])]
            else:
                info["iterations"] = sinfo["cycles"] / 2.0
            info["resvec"] = resvec
            info["status"] = ("solved-" if flag == 0 else "iterative-") + solver + ("" if flag == 0 else
                                                                                     "-not-converged")
            info["gpu"] = dict(requested=True, enabled=True, resultGathered=True,
                               note="operator, preconditioner, Krylov vectors and observables on the GPU")
        DG["status"] = info["status"]
        DG["info"] = {"solve": info}
        DG["rho"] = rho
        if rho is None:
            DG.update(n=None, j=None, jx=None, jy=None, RHO=None)
            return DG
        o = op.observables_all()
        DG.update(n=o["n"], jx=o["jx"], jy=o["jy"], j=o["j"], nDG=o["nDG"], jxDG=o["jxDG"], jyDG=o["jyDG"],
                  y=o["y"])
        if _store_rho_array(prm, n):
            DG["RHO"] = rho.reshape(DG["arraySize"], order="F")
        else:
            DG["RHO"] = None
            info["RHONote"] = ("RHO array was not duplicated; use DG.rho and reshape with DG.arraySize, ordered as "
                               "rho_x,rho_y,X,Y, if needed.")
        return DG
    finally:
        op.close()
