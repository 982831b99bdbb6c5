"""CPU restatement of the reference's Full-2D (X, Y, rho_x, rho_y) operator -- ORACLE.

Test infrastructure only: imported by tests/ (and nothing in the product).  It
restates, with scipy.sparse, how the reference assembles and applies the
stationary Full-2D Wigner operator A = A_diff + G_drift:

  - grids and element matrices: DG_code/initParams_full2D.m:27-118 (makeRectDGAxis
    :167-214, makeFVRelativeAxis :216-230), the periodic rho_y derivative :90-96;
  - transport: DG_code/core/get_Diff_full2D.m:76-146 (operator parts), :206-265
    (oneDimensionalDGOperators), :268-293 (liftCenterOperators), :295-347
    (relativeTransportOperators), :718-730 (splitCharacteristicMatrix), :732-755
    (transportScales), :618-639 (applyKronOperator), :486-493 (assembly),
    core/close_PeriodicDGAxis_full2D.m (periodic Y seam), core/get_SpecularReflection_full2D.m
    and get_Diff_full2D.m:433-444 (specular Y walls);
  - potential and CAP: DG_code/core/get_Drift_full2D.m:133-170 (driftData),
    :172-209 (addFVConsistentData), :211-300 (centerProjectionData), :331-364
    (applyFVConsistentDrift), :413-451 (assembly), :620-666 (potential differences
    with independent clamping / periodic wrapping, linear interpolation),
    core/get_CAP_full2D.m, core/get_CAP.m.

Scope: the source/drain faces with their contact masks (core/get_ContactMask_full2D.m;
the closed pieces reflect rho_x, get_Diff_full2D.m:393-423); Y boundaries 'periodic', 'zero-inflow',
'specular' or 'hard-wall' (core/get_HardWallGeometry_full2D.m,
core/constrain_HardWall_full2D.m: the two-point Dirichlet constraint of the
complete operator); constant-mass transport; FV-consistent potential.  The reservoir
right-hand side (get_ContactModeReservoirRho_full2D.m) is not part of the operator.
"""
import numpy as np
import scipy.sparse as sp

from .jacobi import dmatrix1d, jacobi_gl, vandermonde1d

HBAR = 1.054571817e-34
M0 = 9.1093837015e-31
QE = 1.602176634e-19


def _param(prm, name, default):
    v = prm.get(name, None)
    return default if v is None else v


def make_rect_dg_axis(coord, n_local, n_elements):
    """initParams_full2D.m:167-214."""
    r, w = jacobi_gl(0.0, 0.0, n_local - 1)
    V = vandermonde1d(n_local - 1, r)
    invV = np.linalg.inv(V)
    M = invV.T @ invV
    Dr = dmatrix1d(n_local - 1, r, V)
    S = M @ Dr
    vertices = np.linspace(coord[0], coord[-1], n_elements + 1)
    jac = (vertices[1:] - vertices[:-1]) / 2
    nodes = ((vertices[:-1] + vertices[1:])[:, None] / 2 + jac[:, None] * r[None, :]).ravel()
    return dict(nLocal=n_local, nElements=n_elements, nDof=n_elements * n_local, r=r, w=w, V=V, M=M, Dr=Dr,
                S=S, vertices=vertices, nodes=nodes, jacobian=jac)


def make_fv_relative_axis(n_cells, length):
    """initParams_full2D.m:216-230: cell centres and the central-difference derivative."""
    edges = np.linspace(-length / 2, length / 2, n_cells + 1)
    cells = 0.5 * (edges[:-1] + edges[1:])
    delta = edges[1] - edges[0]
    D = sp.diags([-np.ones(n_cells - 1) / (2 * delta), np.ones(n_cells - 1) / (2 * delta)], [-1, 1],
                 shape=(n_cells, n_cells), format="csr")
    return dict(nCells=n_cells, length=length, edges=edges, cells=cells, delta=delta, D=D)


def init_params_full2d(mat):
    """The fields of initParams_full2D.m that the operator uses (coordinates in m)."""
    prm = mat["dg"]["params"]
    scale = _param(prm, "full2D_coordinate_scale", 1e-9)
    x = np.asarray(mat["x"], dtype=float) * scale
    y = np.asarray(mat["y"], dtype=float) * scale
    nk_def = _param(prm, "N_K_chi", 3)
    nkx, nky = int(_param(prm, "N_K_X", nk_def)), int(_param(prm, "N_K_Y", nk_def))
    nex = int(_param(prm, "N_el_X", (len(x) - 1) // (nkx - 1)))
    ney = int(_param(prm, "N_el_Y", (len(y) - 1) // (nky - 1)))
    p = {"coordinateScale": scale, "x": x, "y": y}
    p["X"] = make_rect_dg_axis(x, nkx, nex)
    p["Y"] = make_rect_dg_axis(y, nky, ney)
    p["nCenterDof"] = p["X"]["nDof"] * p["Y"]["nDof"]
    nrx = int(_param(prm, "N_rho_x", _param(prm, "N_xi", 40)))
    nry = int(_param(prm, "N_rho_y", nrx))
    ldef = _param(prm, "Ly", max(abs(y[-1] - y[0]), np.finfo(float).eps))
    lrx = float(_param(prm, "L_rho_x", ldef))
    lry = float(_param(prm, "L_rho_y", ldef))
    ytype = y_boundary_type(mat)
    periodic = ytype == "periodic"
    if periodic:
        lry = float(_param(prm, "L_rho_y", 2 * (y[-1] - y[0])))
    p["rhoX"] = make_fv_relative_axis(nrx, lrx)
    p["rhoY"] = make_fv_relative_axis(nry, lry)
    p["rhoY"]["periodic"] = periodic
    if periodic:                      # initParams_full2D.m:90-96
        d = p["rhoY"]["delta"]
        p["rhoY"]["D"] = (p["rhoY"]["D"] + sp.csr_matrix(([-1 / (2 * d), 1 / (2 * d)], ([0, nry - 1], [nry - 1, 0])),
                                                           shape=(nry, nry))).tocsr()
    p["nRelative"] = nrx * nry
    p["nTotal"] = p["nRelative"] * p["nCenterDof"]
    p["Ax1D"] = -1j * p["rhoX"]["D"]
    p["Ay1D"] = -1j * p["rhoY"]["D"]
    p["Ax"] = sp.kron(sp.identity(nry), p["Ax1D"], format="csr")
    p["Ay"] = sp.kron(p["Ay1D"], sp.identity(nrx), format="csr")
    p["ytype"] = ytype
    return p


def y_boundary_type(mat):
    """core/get_YBoundaryType_full2D.m (default 'specular')."""
    v = str(mat["dg"]["params"].get("full2D_Y_boundary", "specular")).strip().lower()
    return {"specular-reflection": "specular", "reflection": "specular", "reflecting": "specular",
            "zero_inflow": "zero-inflow", "zeroinflow": "zero-inflow", "zero": "zero-inflow",
            "hardwall": "hard-wall", "hard_wall": "hard-wall", "dirichlet": "hard-wall"}.get(v, v)


def one_dimensional_dg_operators(ax):
    """get_Diff_full2D.m:206-265."""
    n, ne, nd = ax["nLocal"], ax["nElements"], ax["nDof"]
    invM = np.linalg.inv(ax["M"])
    P1 = np.zeros((n, n)); P1[0, 0] = 1
    P2 = np.zeros((n, n)); P2[0, n - 1] = 1
    P3 = np.zeros((n, n)); P3[n - 1, n - 1] = 1
    P4 = np.zeros((n, n)); P4[n - 1, 0] = 1
    K1 = invM @ (ax["S"] + 0.5 * P1 - 0.5 * P3)
    K2 = invM @ (0.5 * P1 + 0.5 * P3)
    K2L = invM @ (0.5 * P1)
    K2R = invM @ (0.5 * P3)
    K3 = -0.5 * invM @ P2
    K4 = K3
    K5 = 0.5 * invM @ P4
    K6 = -K5
    ij = 1.0 / ax["jacobian"]
    upper = sp.diags([ij[1:]], [1], shape=(ne, ne))       # spdiags(1./jac, 1): (e, e+1) = 1/jac(e+1)
    lower = sp.diags([ij[1:]], [-1], shape=(ne, ne))
    diag = sp.diags([ij], [0], shape=(ne, ne))
    H1 = sp.kron(upper, K5) + sp.kron(lower, K3) + sp.kron(diag, K1)
    H2 = sp.kron(upper, K6) + sp.kron(lower, K4) + sp.kron(diag, K2)
    left_el = sp.csr_matrix(([1.0], ([0], [0])), shape=(ne, ne))
    right_el = sp.csr_matrix(([1.0], ([ne - 1], [ne - 1])), shape=(ne, ne))
    H2B = sp.kron(left_el @ diag, K2L) + sp.kron(right_el @ diag, K2R)
    left_lift = np.zeros(nd); left_lift[:n] = invM[:, 0] / ax["jacobian"][0]
    right_lift = np.zeros(nd); right_lift[nd - n:] = invM[:, n - 1] / ax["jacobian"][-1]
    left_trace = np.zeros(nd); left_trace[0] = 1
    right_trace = np.zeros(nd); right_trace[nd - 1] = 1
    return {"H1": sp.csr_matrix(H1), "H2": sp.csr_matrix(H2), "H2Boundary": sp.csr_matrix(H2B),
            "H2Interior": sp.csr_matrix(H2 - H2B),
            "leftBoundary": sp.csr_matrix(np.outer(left_lift, left_trace)),
            "rightBoundary": sp.csr_matrix(np.outer(right_lift, right_trace)),
            "leftLift": left_lift, "rightLift": right_lift, "nDof": nd}


def close_periodic_dg_axis(ops):
    """core/close_PeriodicDGAxis_full2D.m."""
    n = ops["nDof"]
    left = np.zeros(n); left[0] = 1
    right = np.zeros(n); right[n - 1] = 1
    out = dict(ops)
    out["H1"] = sp.csr_matrix(ops["H1"] - 0.5 * np.outer(ops["leftLift"], right) + 0.5 * np.outer(ops["rightLift"], left))
    seam = 0.5 * np.outer(ops["leftLift"] - ops["rightLift"], left - right)
    out["H2Interior"] = sp.csr_matrix(ops["H2Interior"] + seam)
    out["H2Boundary"] = sp.csr_matrix((n, n))
    out["H2"] = out["H2Interior"]
    return out


def split_characteristic(A, tol=1e-12):
    """get_Diff_full2D.m:718-730: A = Phi Lambda Phi^-1, A+ / A- from the signs of Lambda."""
    lam, Phi = np.linalg.eig(np.asarray(A.todense() if sp.issparse(A) else A))
    lp = lam.copy(); lp[lp.real <= tol] = 0
    lm = lam.copy(); lm[lm.real >= -tol] = 0
    Pinv = np.linalg.solve(Phi, np.eye(Phi.shape[0]))
    Ap = Phi @ np.diag(lp) @ Pinv
    Am = Phi @ np.diag(lm) @ Pinv
    Ap[np.abs(Ap) < 1e-12] = 0
    Am[np.abs(Am) < 1e-12] = 0
    return Ap, Am, lam


def flux_types(mat):
    """get_Diff_full2D.m:54-61 with the normalisations of :349-391."""
    prm = mat["dg"]["params"]
    general = str(_param(prm, "full2D_fluxType", _param(prm, "rho_flux", _param(prm, "fluxType", "rusanov")))).lower()
    general = "rusanov" if general in ("lf", "lax-friedrichs", "rusanov-local") else general

    def norm(v):
        v = str(v).strip().lower()
        if v in ("lf", "lax-friedrichs", "rusanov-local"):
            return "rusanov"
        if v in ("matrix-upwind", "characteristic-upwind"):
            return "upwind"
        return v
    fx = norm(_param(prm, "full2D_X_flux", general))
    fy = norm(_param(prm, "full2D_Y_flux", fx))
    return fx, fy


def transport_scales(mat):
    """get_Diff_full2D.m:732-755 (constant mass)."""
    prm = mat["dg"]["params"]

    def kg(m):
        mk = m * M0 if abs(m) > 1e-25 else m
        return mk if mk > 0 else 0.041 * M0
    mex = mat.get("me_x_ch", 0.041)
    mey = mat.get("me_y_ch", mex)
    sx = _param(prm, "full2D_Q_diff_x", _param(prm, "full2D_transportScaleX", HBAR / kg(mex)))
    sy = _param(prm, "full2D_Q_diff_y", _param(prm, "full2D_transportScaleY", HBAR / kg(mey)))
    f = _param(prm, "full2D_diff_scale", _param(prm, "rho_diff_scale", 1.0))
    return f * sx, f * sy


def _nearest(values, grid, target):
    """interp1(grid, values, target, 'nearest', 'extrap'): the value of the nearest grid point (a
    target halfway between two points takes the upper one)."""
    grid = np.asarray(grid, dtype=float)
    i = np.clip(np.searchsorted(grid, target, side="right") - 1, 0, len(grid) - 1)
    j = np.minimum(i + 1, len(grid) - 1)
    up = (j > i) & (target - grid[i] >= grid[j] - target)
    return np.asarray(values)[np.where(up, j, i)]


def contact_mask(mat, p, side):
    """get_ContactMask_full2D.m:14-120: the face Y dofs that receive Source/Drain inflow (the rest
    of the outer X face is closed).  Explicit full2D_<side>ContactMask (per face dof or per material
    y point), else the doping at the X edge above full2D_contactNdThreshold, else the material gap
    (Eg below the middle of Eg_c and Eg_ox) or the W_c / W_cy geometry, else the whole face; an empty
    mask falls back to the material/geometry rule."""
    prm = mat["dg"]["params"]
    scale = p["coordinateScale"]
    y_face = p["Y"]["nodes"]
    grid = np.asarray(mat["y"], dtype=float) * scale
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    ix = 0 if side == "source" else nx - 1

    def xy(field):
        a = np.squeeze(np.asarray(field, dtype=float))
        if a.shape == (nx, ny):
            return a
        if a.shape == (ny, nx):
            return a.T
        if a.ndim == 1 and a.size == nx:
            return np.repeat(a[:, None], ny, axis=1)
        if a.ndim == 1 and a.size == ny:
            return np.repeat(a[None, :], nx, axis=0)
        raise ValueError("DG:Full2D:InvalidMaterialField")

    def material():
        if mat.get("Eg") is not None and mat.get("Eg_ox") is not None:
            eg = xy(mat["Eg"])
            thr = 0.5 * (float(mat.get("Eg_c", eg.min())) + float(mat["Eg_ox"]))
            return _nearest(eg[ix] < thr, grid, y_face).astype(bool)
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
            mask = _nearest(m.astype(float), grid, y_face) > 0.5
        else:
            raise ValueError("DG:Full2D:InvalidContactMask")
    elif mat.get("Nd") is not None and np.size(mat["Nd"]) > 0:
        thr = float(prm.get("full2D_contactNdThreshold", 0.0) or 0.0)
        mask = _nearest((xy(mat["Nd"])[ix] > thr).astype(float), grid, y_face) > 0.5
    else:
        mask = material()
    if not mask.any():
        mask = material()
    return np.asarray(mask, dtype=bool)


def diff_operator_parts(mat, p):
    """[(name, coefficient, centre matrix, relative matrix)] of get_Diff_full2D.m:76-146, with the
    closed-face reflection parts of :393-423 on the masked-off Y dofs of the outer X faces."""
    prm = mat["dg"]["params"]
    fx, fy = flux_types(mat)
    ox = one_dimensional_dg_operators(p["X"])
    oy = one_dimensional_dg_operators(p["Y"])
    if p["ytype"] == "periodic":
        oy = close_periodic_dg_axis(oy)
    IX, IY = sp.identity(p["X"]["nDof"]), sp.identity(p["Y"]["nDof"])
    nrx, nry = p["rhoX"]["nCells"], p["rhoY"]["nCells"]
    Irx, Iry = sp.identity(nrx), sp.identity(nry)
    tol = _param(prm, "full2D_characteristicTol", 1e-12)
    Apx, Amx, lx = split_characteristic(p["Ax1D"], tol)
    Apy, Amy, ly = split_characteristic(p["Ay1D"], tol)
    theta_def = 0.01
    tx = _param(prm, "full2D_thetaLF_X", _param(prm, "full2D_thetaLF", _param(prm, "thetaLF", theta_def))) \
        if fx == "rusanov" else 0.0
    ty = _param(prm, "full2D_thetaLF_Y", _param(prm, "full2D_thetaLF", _param(prm, "thetaLF", theta_def))) \
        if fy == "rusanov" else 0.0
    bx = tx * _param(prm, "full2D_alphaLF_X", np.max(np.abs(lx)))
    by = ty * _param(prm, "full2D_alphaLF_Y", np.max(np.abs(ly)))
    absx = sp.kron(Iry, sp.csr_matrix(Apx - Amx))
    absy = sp.kron(sp.csr_matrix(Apy - Amy), Irx)
    IR = sp.identity(nrx * nry)
    sx, sy = transport_scales(mat)
    parts = [("X central", sx, sp.kron(IY, ox["H1"]), p["Ax"])]
    if fx == "upwind":
        parts.append(("X interior upwind", sx, sp.kron(IY, ox["H2Interior"]), absx))
    elif bx != 0:
        parts.append(("X interior Rusanov", sx, sp.kron(IY, ox["H2Interior"]), bx * IR))
    parts.append(("X boundary penalty", sx, sp.kron(IY, ox["H2Boundary"]), absx))
    # closed pieces of the outer X faces reflect rho_x -> -rho_x (R_x = I_rho_y kron Flip_rho_x)
    Rx = sp.kron(Iry, sp.csr_matrix(np.fliplr(np.eye(nrx))))
    for side, sign, lift, Ach in (("source", -1.0, ox["leftBoundary"], Apx), ("drain", 1.0, ox["rightBoundary"], Amx)):
        closed = ~contact_mask(mat, p, side)
        if closed.any():
            parts.append(("X-%s closed-face reflection correction" % ("left" if side == "source" else "right"),
                          sign * sx, sp.kron(sp.diags(closed.astype(float)), lift),
                          sp.kron(Iry, sp.csr_matrix(Ach)) @ Rx))
    parts.append(("Y central", sy, sp.kron(oy["H1"], IX), p["Ay"]))
    if fy == "upwind":
        parts.append(("Y interior upwind", sy, sp.kron(oy["H2Interior"], IX), absy))
    elif by != 0:
        parts.append(("Y interior Rusanov", sy, sp.kron(oy["H2Interior"], IX), by * IR))
    if p["ytype"] not in ("hard-wall", "periodic"):
        parts.append(("Y boundary penalty", sy, sp.kron(oy["H2Boundary"], IX), absy))
    if p["ytype"] == "specular":
        flip = sp.csr_matrix(np.fliplr(np.eye(nry)))
        Ry = sp.kron(flip, Irx)
        parts.append(("Y bottom specular", -sy, sp.kron(oy["leftBoundary"], IX),
                      sp.kron(sp.csr_matrix(Apy), Irx) @ Ry))
        parts.append(("Y top specular", sy, sp.kron(oy["rightBoundary"], IX),
                      sp.kron(sp.csr_matrix(Amy), Irx) @ Ry))
    return [(n, c, sp.csr_matrix(C), sp.csr_matrix(R)) for n, c, C, R in parts if c != 0 and C.nnz and R.nnz]


def apply_kron(parts, u, n_center, n_relative):
    """applyKronOperator (get_Diff_full2D.m:618-639): Y = sum c (R U) C^T."""
    U = np.asarray(u).reshape(n_center, n_relative).T        # column-major reshape(u, nRel, nCenter)
    Y = np.zeros_like(U, dtype=complex)
    for _, c, C, R in parts:
        Y += c * (C @ (R @ U).T).T
    return Y.T.reshape(-1)


def assemble_kron(parts, n_center, n_relative):
    """assembleKronOperator (get_Diff_full2D.m:486-493): sum c kron(C, R)."""
    A = sp.csr_matrix((n_center * n_relative, n_center * n_relative), dtype=complex)
    for _, c, C, R in parts:
        A = A + c * sp.kron(C, R, format="csr")
    return A


# ----------------------------------------------------------------------------- potential and CAP

def cap_profile(p):
    """core/get_CAP_full2D.m: C_rho = kron(I_y, C_x) + kron(C_y, I_x) (no C_y for periodic rho_y)."""
    from .dg1d import get_cap
    wx = get_cap(p["rhoX"]["cells"], p["rhoX"]["length"], p["rhoX"]["delta"])
    wy = get_cap(p["rhoY"]["cells"], p["rhoY"]["length"], p["rhoY"]["delta"])
    if p["rhoY"]["periodic"]:
        wy = np.zeros_like(wy)
    nrx, nry = len(wx), len(wy)
    return (np.tile(wx, nry) + np.repeat(wy, nrx)).astype(float)


def center_projection_data(mat, p):
    """get_Drift_full2D.m:211-300."""
    prm = mat["dg"]["params"]
    nlx, nly = p["X"]["nLocal"], p["Y"]["nLocal"]
    common = prm.get("full2D_potentialQuadratureOrder", None)
    if common is None:
        nqx = _param(prm, "full2D_potentialQuadratureX", max(4, 2 * nlx - 1))
        nqy = _param(prm, "full2D_potentialQuadratureY", max(4, 2 * nly - 1))
    else:
        nqx = nqy = common
    nqx, nqy = max(nlx, int(round(nqx))), max(nly, int(round(nqy)))
    qx, wx = jacobi_gl(0.0, 0.0, nqx - 1)
    qy, wy = jacobi_gl(0.0, 0.0, nqy - 1)
    Ix = vandermonde1d(nlx - 1, qx) @ np.linalg.inv(p["X"]["V"])
    Iy = vandermonde1d(nly - 1, qy) @ np.linalg.inv(p["Y"]["V"])
    interp = np.kron(Iy, Ix)
    w = np.kron(wy, wx)
    MXY = np.kron(p["Y"]["M"], p["X"]["M"])
    invM = np.linalg.solve(MXY, np.eye(MXY.shape[0]))
    proj = (interp * w[:, None]) @ invM.T
    nex, ney = p["X"]["nElements"], p["Y"]["nElements"]
    ids, XQ, YQ = [], [], []
    for ey in range(ney):
        yq = 0.5 * (p["Y"]["vertices"][ey] + p["Y"]["vertices"][ey + 1]) + p["Y"]["jacobian"][ey] * qy
        yid = ey * nly + np.arange(nly)
        for ex in range(nex):
            xq = 0.5 * (p["X"]["vertices"][ex] + p["X"]["vertices"][ex + 1]) + p["X"]["jacobian"][ex] * qx
            xid = ex * nlx + np.arange(nlx)
            lx_, ly_ = np.meshgrid(xid, yid, indexing="ij")
            ids.append((lx_ + ly_ * p["X"]["nDof"]).ravel(order="F"))
            Xq, Yq = np.meshgrid(xq, yq, indexing="ij")
            XQ.append(Xq.ravel(order="F"))
            YQ.append(Yq.ravel(order="F"))
    return dict(interp=interp, proj=proj, ids=np.array(ids).T, XQ=np.array(XQ).T, YQ=np.array(YQ).T,
                nq=len(w), nlocal=nlx * nly)


def relative_projection(p):
    """get_Drift_full2D.m:175-196: P = kron(Ey, Ex) sums the cells around each vertex."""
    nx, ny = p["rhoX"]["nCells"], p["rhoY"]["nCells"]
    Ex = sp.diags([np.ones(nx), np.ones(nx)], [0, -1], shape=(nx + 1, nx))
    ey_edges = p["rhoY"]["edges"]
    if p["rhoY"]["periodic"]:
        Ey = sp.identity(ny) + sp.csr_matrix((np.ones(ny), (np.arange(ny), np.r_[ny - 1, np.arange(ny - 1)])),
                                             shape=(ny, ny))
        ey_edges = ey_edges[:-1]
    else:
        Ey = sp.diags([np.ones(ny), np.ones(ny)], [0, -1], shape=(ny + 1, ny))
    VX, VY = np.meshgrid(p["rhoX"]["edges"], ey_edges, indexing="ij")
    return sp.csr_matrix(sp.kron(Ey, Ex)), VX.ravel(order="F"), VY.ravel(order="F")


def interp_linear_2d(gx, gy, V, qx, qy):
    """griddedInterpolant({gx, gy}, V, 'linear') inside the grid (queries pre-clamped)."""
    ix = np.clip(np.searchsorted(gx, qx, side="right") - 1, 0, len(gx) - 2)
    iy = np.clip(np.searchsorted(gy, qy, side="right") - 1, 0, len(gy) - 2)
    tx = (qx - gx[ix]) / (gx[ix + 1] - gx[ix])
    ty = (qy - gy[iy]) / (gy[iy + 1] - gy[iy])
    return ((1 - tx) * (1 - ty) * V[ix, iy] + tx * (1 - ty) * V[ix + 1, iy] + (1 - tx) * ty * V[ix, iy + 1]
            + tx * ty * V[ix + 1, iy + 1])


def potential_difference(p, V, cpd, vx, vy):
    """get_Drift_full2D.m:635-666: V(X + rho/2) - V(X - rho/2) at every relative vertex and
    centre quadrature point, X clamped, Y clamped or wrapped.  [nVert, nq, nElements]."""
    gx, gy = p["x"], p["y"]

    def ext(qx, qy):
        qx = np.clip(qx, gx[0], gx[-1])
        if p["rhoY"]["periodic"]:
            qy = gy[0] + np.mod(qy - gy[0], gy[-1] - gy[0])
        else:
            qy = np.clip(qy, gy[0], gy[-1])
        return interp_linear_2d(gx, gy, V, qx, qy)
    X = cpd["XQ"][None, :, :]
    Y = cpd["YQ"][None, :, :]
    rx = 0.5 * vx[:, None, None]
    ry = 0.5 * vy[:, None, None]
    return ext(X + rx, Y + ry) - ext(X - rx, Y - ry)


def drift_data(mat, p, V):
    """The FV-consistent drift's data (driftData + addFVConsistentData)."""
    prm = mat["dg"]["params"]
    qdrift = _param(prm, "full2D_Q_drift", QE / HBAR)
    dscale = _param(prm, "full2D_drift_scale", 1.0)
    cscale = _param(prm, "full2D_cap_scale", 1.0)
    P, vx, vy = relative_projection(p)
    cpd = center_projection_data(mat, p)
    return dict(P=P, cpd=cpd, dV=potential_difference(p, np.asarray(V, dtype=float), cpd, vx, vy),
                pot=1j * dscale * qdrift, capc=dscale * cscale * qdrift, cap=cap_profile(p))


def apply_drift(p, dd, u):
    """applyFVConsistentDrift (get_Drift_full2D.m:331-364)."""
    nrel, nc = p["nRelative"], p["nCenterDof"]
    U = np.asarray(u).reshape(nc, nrel).T
    Y = dd["capc"] * (dd["cap"][:, None] * U)
    cpd = dd["cpd"]
    for e in range(cpd["ids"].shape[1]):
        ids = cpd["ids"][:, e]
        Uq = U[:, ids] @ cpd["interp"].T                       # [nRel, nq]
        vert = dd["P"] @ Uq
        res = dd["P"].T @ (dd["dV"][:, :, e] * vert)
        res = dd["pot"] * (1.0 / 16) * res
        Y[:, ids] += res @ cpd["proj"]
    return Y.T.reshape(-1)


def assemble_drift(p, dd):
    """assembleFVConsistentMatrix (get_Drift_full2D.m:413-451)."""
    nrel, nc = p["nRelative"], p["nCenterDof"]
    cpd = dd["cpd"]
    G = sp.csr_matrix((nrel * nc, nrel * nc), dtype=complex)
    for e in range(cpd["ids"].shape[1]):
        local = sp.csr_matrix((nrel * cpd["nlocal"], nrel * cpd["nlocal"]), dtype=complex)
        for q in range(cpd["nq"]):
            Crel = dd["pot"] / 16 * (dd["P"].T @ sp.diags(dd["dV"][:, q, e]) @ dd["P"])
            H = np.outer(cpd["proj"][q, :], cpd["interp"][q, :])
            local = local + sp.kron(sp.csr_matrix(H), Crel)
        gid = (np.arange(nrel)[:, None] + cpd["ids"][:, e][None, :] * nrel).ravel(order="F")
        coo = local.tocoo()
        G = G + sp.csr_matrix((coo.data, (gid[coo.row], gid[coo.col])), shape=G.shape)
    return G + sp.diags(np.tile(dd["capc"] * dd["cap"], nc))


def system(mat, V):
    """(p, parts, drift data): A = sum of the parts + G_drift (get_SysM_full2D.m:124-127)."""
    p = init_params_full2d(mat)
    return p, diff_operator_parts(mat, p), drift_data(mat, p, V)


def apply_system(p, parts, dd, u):
    return apply_kron(parts, u, p["nCenterDof"], p["nRelative"]) + apply_drift(p, dd, u)


# ----------------------------------------------------------------------------- hard-wall Y boundary

def hard_wall_geometry(p, scales):
    """core/get_HardWallGeometry_full2D.m:15-48 and constrain_HardWall_full2D.m:10-18.

    active [N_rho_y, nYdof]: the samples whose two particle coordinates Y +- rho_y/2 lie strictly
    inside the Y interval (64 ulp of the largest coordinate as margin); T: per Y element and rho_y
    cell, the exact-DG-mass projection M(keep,keep)^-1 M(keep,:) onto the element's active nodes
    (rows of inactive nodes zero), on the (rho_y fastest, Y node) index; scale: the constraint
    row weight max(1, |Qx| / (min dX * d_rho_x) + |Qy| / (min dY * d_rho_y))."""
    rho = p["rhoY"]["cells"]
    Y = p["Y"]["nodes"]
    y0, y1 = p["y"][0], p["y"][-1]
    big = max(abs(y0), abs(y1), float(np.max(np.abs(rho))))
    tol = 64 * np.spacing(big)
    dist = np.minimum(Y - y0, y1 - Y)
    active = np.abs(rho)[:, None] / 2 < dist[None, :] - tol
    if not active.any():
        raise ValueError("DG:Full2D:HardWallEmptyDomain")
    nr, ny, nl = len(rho), len(Y), p["Y"]["nLocal"]
    M = p["Y"]["M"]
    T = sp.lil_matrix((nr * ny, nr * ny))
    for e in range(p["Y"]["nElements"]):
        yids = e * nl + np.arange(nl)
        for ir in range(nr):
            keep = active[ir, yids]
            if keep.any():
                ids = ir + nr * yids
                T[np.ix_(ids[keep], ids)] = np.linalg.solve(M[np.ix_(keep, keep)], M[keep, :])
    sx, sy = scales
    g = max(1.0, abs(sx) / (np.min(np.diff(p["X"]["vertices"])) * p["rhoX"]["delta"])
            + abs(sy) / (np.min(np.diff(p["Y"]["vertices"])) * p["rhoY"]["delta"]))
    return dict(active=active, T=sp.csr_matrix(T), scale=g)


def _wall_order(p):
    """Permutation taking the global index (rho_x, rho_y, X, Y) to (rho_y, Y) x (rho_x, X) blocks."""
    nrx, nry = p["rhoX"]["nCells"], p["rhoY"]["nCells"]
    nx, ny = p["X"]["nDof"], p["Y"]["nDof"]
    idx = np.arange(nrx * nry * nx * ny).reshape(ny, nx, nry, nrx)     # C order: rho_x fastest
    # rows (X, rho_x) with rho_x fastest, columns (Y, rho_y) with rho_y fastest (T's index)
    return idx.transpose(1, 3, 0, 2).reshape(nx * nrx, ny * nry)


def wall_active_mask(p, wall):
    """The active flag of every global unknown (maskInput of constrain_HardWall_full2D.m:46-50)."""
    nrx, nx = p["rhoX"]["nCells"], p["X"]["nDof"]
    nry, ny = p["rhoY"]["nCells"], p["Y"]["nDof"]
    m = np.broadcast_to(wall["active"].T[:, None, :, None], (ny, nx, nry, nrx))
    return m.reshape(-1).astype(float)


def wall_project(p, wall, u):
    """applyTransverse (constrain_HardWall_full2D.m:52-57): T on the (rho_y, Y) index of u."""
    order = _wall_order(p)
    U = np.asarray(u)[order]                           # [(rho_x, X), (rho_y, Y)]
    out = np.empty_like(np.asarray(u), dtype=complex)
    out[order] = (wall["T"] @ U.T).T
    return out


def apply_hard_wall(p, wall, apply_base, u):
    """constrainedApply (constrain_HardWall_full2D.m:40-44): T A (mask u) + scale (u - mask u)."""
    act = wall_active_mask(p, wall)
    um = np.asarray(u) * act
    return wall_project(p, wall, apply_base(um)) + wall["scale"] * (np.asarray(u) - um)


def constrain_hard_wall(p, wall, A):
    """constrainedMatrix (constrain_HardWall_full2D.m:65-72): T A P + scale (I - P), T lifted."""
    n = p["nTotal"]
    act = wall_active_mask(p, wall)
    order = _wall_order(p)
    nb = order.shape[0]
    Tl = sp.kron(wall["T"], sp.identity(nb), format="coo")        # index (rho_y,Y) * nb + (rho_x,X)
    flat = order.T.reshape(-1)                                       # position (rho_y,Y)*nb + (rho_x,X)
    T = sp.csr_matrix((Tl.data, (flat[Tl.row], flat[Tl.col])), shape=(n, n))
    return (T @ A @ sp.diags(act) + wall["scale"] * sp.diags(1 - act)).tocsr()


# ----------------------------------------------------------------------------- line-transverse preconditioner

def transverse_reference(mat, V, ix=0):
    """transverseReference (get_LineTransversePreconditioner_full2D.m:127-175): the frozen-X
    transverse transport K and potential V blocks of a 2-cell, 2-element strip at column ix."""
    prm = dict(mat["dg"]["params"])
    prm.update(N_rho_x=2, N_K_X=2, N_el_X=2, full2D_Q_diff_x=0.0, full2D_cap_scale=0.0)
    ref = dict(mat)
    ref["dg"] = dict(mat["dg"], params=prm)
    V = np.asarray(V, dtype=float)
    Vref = np.repeat(V[ix:ix + 1, :], V.shape[0], axis=0)
    pr = init_params_full2d(ref)
    parts = diff_operator_parts(ref, pr)
    dd = drift_data(ref, pr, Vref)
    Kfull = assemble_kron(parts, pr["nCenterDof"], pr["nRelative"])
    Vfull = assemble_drift(pr, dd)
    nry, nX, nY = pr["rhoY"]["nCells"], pr["X"]["nDof"], pr["Y"]["nDof"]
    ry, Y = np.meshgrid(np.arange(nry), np.arange(nY), indexing="ij")
    ids = (0 + 2 * (ry + nry * (0 + nX * Y))).ravel(order="F")        # ids(1,:,1,:)(:)
    K = Kfull[ids][:, ids].toarray()
    Vt = 2.0 * Vfull[ids][:, ids].toarray()          # the rho_x diagonal of P_x' P_x / 4 is 1/2
    return K, Vt


def x_factors(ax, speeds, sigma):
    """xFactors (get_LineTransversePreconditioner_full2D.m:177-200): [n, n, modes, elements]."""
    n = ax["nLocal"]
    Pl = np.zeros((n, n)); Pl[0, 0] = 1
    Pr = np.zeros((n, n)); Pr[-1, -1] = 1
    PfL = np.zeros((n, n)); PfL[0, -1] = 1
    PfR = np.zeros((n, n)); PfR[-1, 0] = 1
    K1 = np.linalg.solve(ax["M"], ax["S"] + 0.5 * Pl - 0.5 * Pr)
    K2 = np.linalg.solve(ax["M"], 0.5 * Pl + 0.5 * Pr)
    ne, nm = ax["nElements"], len(speeds)
    inv = np.zeros((n, n, nm, ne), dtype=complex)
    cpl = np.zeros_like(inv)
    fwd = speeds >= 0
    for e in range(ne):
        for k in range(nm):
            a = speeds[k] / (sigma * ax["jacobian"][e])
            inv[:, :, k, e] = np.linalg.solve(np.eye(n) + a * K1 + abs(a) * K2, np.eye(n))
            cpl[:, :, k, e] = -a * np.linalg.solve(ax["M"], PfL) if fwd[k] else a * np.linalg.solve(ax["M"], PfR)
    return inv, cpl, fwd


def line_transverse(mat, p, V, dd, ix=0):
    """get_LineTransversePreconditioner_full2D.m:17-113 (dense transverse factors)."""
    prm = mat["dg"]["params"]
    nm, nry, nY = p["rhoX"]["nCells"], p["rhoY"]["nCells"], p["Y"]["nDof"]
    nT = nry * nY
    lam, U = np.linalg.eigh(p["Ax1D"].toarray())        # Hermitian: real eigenvalues, unitary modes
    lam = lam.real.copy()
    lam[np.abs(lam) < 100 * np.spacing(np.max(np.abs(lam)))] = 0
    K, Vt = transverse_reference(mat, V, ix)
    wx = dd["cap"][:nm] - (0 if p["rhoY"]["periodic"] else 0)
    from .dg1d import get_cap
    wxp = get_cap(p["rhoX"]["cells"], p["rhoX"]["length"], p["rhoX"]["delta"])
    wyp = get_cap(p["rhoY"]["cells"], p["rhoY"]["length"], p["rhoY"]["delta"])
    if p["rhoY"]["periodic"]:
        wyp = np.zeros_like(wyp)
    capY = np.tile(wyp, nY) * dd["capc"]
    capX = np.real(np.sum(np.conj(U) * (wxp[:, None] * U), axis=0)) * dd["capc"]
    Pm = sp.diags([np.ones(nm), np.ones(nm)], [0, -1], shape=(nm + 1, nm)).toarray()
    pw = np.real(np.sum(np.conj(U) * ((Pm.T @ Pm / 4) @ U), axis=0))
    sx, _ = transport_scales(mat)
    x_rate = abs(sx) * np.max(np.abs(lam)) / np.min(p["X"]["jacobian"])
    t_rate = np.max(np.abs(K).sum(1)) + np.max(np.abs(Vt).sum(1)) + np.max(np.abs(capY)) + np.max(np.abs(capX))
    sigma = _param(prm, "full2D_lineShift", _param(prm, "full2D_lineRelativeShift", 0.003) * max(x_rate, t_rate,
                                                                                               np.finfo(float).tiny))
    xinv, xcpl, fwd = x_factors(p["X"], sx * lam, sigma)
    wall = hard_wall_geometry(p, transport_scales(mat)) if p["ytype"] == "hard-wall" else None
    Binv = np.zeros((nm, nT, nT), dtype=complex)
    for k in range(nm):
        B = K + pw[k] * Vt + np.diag(capY + capX[k])
        if wall is not None:            # get_LineTransversePreconditioner_full2D.m:84-88
            act = wall["active"].T.reshape(-1).astype(float)        # (rho_y fastest, Y) index
            B = wall["T"].toarray() @ B @ np.diag(act) + wall["scale"] * np.diag(1 - act)
        B = B / sigma + np.eye(nT)
        Binv[k] = np.linalg.solve(B, np.eye(nT))
    return dict(U=U, lam=lam, sigma=sigma, xinv=xinv, xcpl=xcpl, fwd=fwd, Binv=Binv, K=K, Vt=Vt, pw=pw,
                capX=capX, capY=capY)


def line_transverse_apply(p, d, r):
    """applyInverse (get_LineTransversePreconditioner_full2D.m:202-238)."""
    nm, nry, nX, nY = p["rhoX"]["nCells"], p["rhoY"]["nCells"], p["X"]["nDof"], p["Y"]["nDof"]
    n, ne = p["X"]["nLocal"], p["X"]["nElements"]
    R = np.asarray(r).reshape(nY, nX, nry, nm)            # C order: [Y][X][ry][mode]
    W = np.einsum("ik,yxrk->yxri", np.conj(d["U"]).T @ np.eye(nm), R) if False else \
        np.einsum("ki,yxrk->yxri", np.conj(d["U"]), R)   # w = U^H r along rho_x
    Wl = W.reshape(nY, ne, n, nry, nm)                      # X = e n + a
    out = np.zeros_like(Wl)
    for k in range(nm):
        order = range(ne) if d["fwd"][k] else range(ne - 1, -1, -1)
        prev = np.zeros((nY, n, nry), dtype=complex)
        for e in order:
            blk = Wl[:, e, :, :, k] - np.einsum("ab,ybr->yar", d["xcpl"][:, :, k, e], prev)
            prev = np.einsum("ab,ybr->yar", d["xinv"][:, :, k, e], blk)
            out[:, e, :, :, k] = prev
    Vv = out.reshape(nY, nX, nry, nm)
    # transverse solve per mode and X dof over t = ry + nry Y
    T = np.transpose(Vv, (3, 1, 0, 2)).reshape(nm, nX, nY * nry)   # [k][X][Y][ry] -> t = ry + nry Y
    T = np.einsum("kst,kxt->kxs", d["Binv"], T)
    Vv = np.transpose(T.reshape(nm, nX, nY, nry), (2, 1, 3, 0))     # back to [Y][X][ry][k]
    Z = np.einsum("ik,yxrk->yxri", d["U"], Vv) / d["sigma"]
    return Z.reshape(-1)


# ----------------------------------------------------------------------------- observables

def _zero_weights(cells):
    """zeroInterpolationWeights (get_Observables_full2D.m:80-103)."""
    cells = np.asarray(cells, dtype=float)
    nearest = int(np.argmin(np.abs(cells)))
    if abs(cells[nearest]) <= max(1e-14, 1e-12 * max(1, np.abs(cells).max())):
        return [nearest], [1.0]
    left = np.flatnonzero(cells < 0)
    right = np.flatnonzero(cells > 0)
    if left.size and right.size:
        lo, hi = left[-1], right[0]
        h = cells[hi] - cells[lo]
        return [lo, hi], [cells[hi] / h, -cells[lo] / h]
    return [nearest], [1.0]


def _derivative_row(cells, D):
    """derivativeRowAtZero (get_Observables_full2D.m:105-134) for a grid with a cell at or
    bracketing zero."""
    cells = np.asarray(cells, dtype=float)
    nearest = int(np.argmin(np.abs(cells)))
    if abs(cells[nearest]) <= max(1e-14, 1e-12 * max(1, np.abs(cells).max())):
        return np.asarray(D.todense() if sp.issparse(D) else D)[nearest]
    row = np.zeros(cells.size)
    lo, hi = np.flatnonzero(cells < 0)[-1], np.flatnonzero(cells > 0)[0]
    h = cells[hi] - cells[lo]
    row[lo], row[hi] = -1 / h, 1 / h
    return row


def _project_to_y(values, ydg, target):
    """projectValuesToY (get_Observables_full2D.m:154-168): columns at the same Y node (element
    interfaces) averaged, then linear interpolation with extrapolation onto the target Y."""
    order = np.argsort(ydg, kind="stable")
    ys, vals = ydg[order], values[:, order]
    tol = 1e-12 * max(abs(ys[-1] - ys[0]), 1e-300)
    groups = []
    for i in range(ys.size):
        if groups and ys[i] - ys[groups[-1][0]] <= tol:
            groups[-1].append(i)
        else:
            groups.append([i])
    uy = np.array([ys[g[0]] for g in groups])
    avg = np.stack([vals[:, g].mean(axis=1) for g in groups], axis=1)
    if uy.size == 1:
        return np.repeat(avg, target.size, axis=1)
    from scipy.interpolate import interp1d
    return interp1d(uy, avg, axis=1, kind="linear", fill_value="extrapolate")(target)


def observables(p, mat, rho):
    """(n [X nDof x material Ny], j [X nDof], nDG, jxDG) (get_Observables_full2D.m:19-78):
    n = real(rho) at zero relative separation, j_x = q hbar / m_x imag(d rho / d rho_x) at zero,
    both projected onto the material Y grid, j integrated over Y (trapezoid, in m)."""
    nrx, nry = p["rhoX"]["nCells"], p["rhoY"]["nCells"]
    nX, nY = p["X"]["nDof"], p["Y"]["nDof"]
    rho = np.asarray(rho).ravel()
    by_center = rho.reshape(nX * nY, nrx * nry).T                   # reshape(rho, nRel, nCenter)
    r4 = rho.reshape(nY, nX, nry, nrx).transpose(3, 2, 1, 0)          # rho(iRhoX, iRhoY, iX, iY)
    ix_ids, ix_w = _zero_weights(p["rhoX"]["cells"])
    iy_ids, iy_w = _zero_weights(p["rhoY"]["cells"])
    nDG = np.zeros((nX, nY))
    for a, wa in zip(ix_ids, ix_w):
        for b, wb in zip(iy_ids, iy_w):
            nDG += wa * wb * np.real(r4[a, b])
    rowx = _derivative_row(p["rhoX"]["cells"], p["rhoX"]["D"])
    dx = np.zeros(nX * nY, dtype=complex)
    for b, wb in zip(iy_ids, iy_w):
        dx += wb * (rowx @ by_center[b * nrx:(b + 1) * nrx, :])
    mex = mat.get("me_x_ch", 0.041)
    mkg = mex * M0 if abs(mex) > 1e-25 else mex
    mkg = mkg if mkg > 0 else 0.041 * M0
    jxDG = QE * HBAR / mkg * np.imag(dx.reshape(nX, nY, order="F"))
    target = np.asarray(mat["y"], dtype=float) * p["coordinateScale"]
    ydg = p["Y"]["nodes"]
    n = _project_to_y(nDG, ydg, target)
    jx = _project_to_y(jxDG, ydg, target)
    trapz = getattr(np, "trapezoid", None) or np.trapz
    return n, trapz(jx, target, axis=1), nDG, jxDG


def observables_y(p, mat, rho):
    """(jy [X nDof x material Ny], jyDG) (get_Observables_full2D.m:47-58): the rho_y derivative at
    zero relative separation, rho_x interpolated to zero, scaled by q hbar / m_y
    (me_y_ch, default me_x_ch), projected onto the material Y grid."""
    nrx, nry = p["rhoX"]["nCells"], p["rhoY"]["nCells"]
    nX, nY = p["X"]["nDof"], p["Y"]["nDof"]
    by_center = np.asarray(rho).ravel().reshape(nX * nY, nrx * nry).T
    ix_ids, ix_w = _zero_weights(p["rhoX"]["cells"])
    rowy = _derivative_row(p["rhoY"]["cells"], p["rhoY"]["D"])
    dy = np.zeros(nX * nY, dtype=complex)
    for a, wa in zip(ix_ids, ix_w):
        rel_ids = a + np.arange(nry) * nrx
        dy += wa * (rowy @ by_center[rel_ids, :])
    mey = mat.get("me_y_ch", mat.get("me_x_ch", 0.041))
    mkg = mey * M0 if abs(mey) > 1e-25 else mey
    mkg = mkg if mkg > 0 else 0.041 * M0
    jyDG = QE * HBAR / mkg * np.imag(dy.reshape(nX, nY, order="F"))
    target = np.asarray(mat["y"], dtype=float) * p["coordinateScale"]
    return _project_to_y(jyDG, p["Y"]["nodes"], target), jyDG
