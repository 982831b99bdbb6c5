"""2D Poisson step of the Full-2D Gummel loop (oracle; test infrastructure only).

Restates in NumPy/SciPy the material-grid electrostatics that the reference runs on either
side of the Full-2D transport solve:

  eval_poisson2d        RTD/eval_Poisson2D_rtd.m:1-196: the 5-point div(eps grad phi) operator
                        on the (Nx, Ny) material grid (harmonic-mean permittivity at faces,
                        half control volumes at free X ends and non-periodic Y ends, identity
                        rows at Dirichlet nodes, a phi(:,end) = phi(:,1) row per periodic
                        duplicate), the node maps with their ghost frame
  solve_poisson2d       RTD/solve_Poisson2D_rtd.m:1-131: the direct or the approximate-Newton
                        update (J = A_ff - diag(q^2 n / (kB T))) on the unique nodes, its
                        diagnostics (linear and physical residuals, net charge per length)
  project_dg_density    RTD/project_DG_density_RTD.m:1-69: exact element-wise integrals of the
                        DG density polynomial over the Poisson dual volumes
  doping_si, x_boundary RTD/get_RTD_doping_SI.m, RTD/get_RTD_poisson_x_boundary.m

Arrays are [Nx, Ny] as in the reference; node k = ix + iy Nx (MATLAB's column-major order).
The direct sparse solves are the reference's own algorithm (backslash).  Pinned by closed forms
(linear and parabolic profiles, flux continuity across a permittivity step) in the tests.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

EPS0 = 8.8541878128e-12
Q = 1.602176634e-19
KB = 1.380649e-23


def x_boundary(mat):
    """RTD/get_RTD_poisson_x_boundary.m: 'dirichlet' unless mat.poisson.xBoundary says 'neumann'."""
    v = mat.get("poisson", {}).get("xBoundary", "dirichlet")
    v = str(v).lower()
    if v not in ("dirichlet", "neumann"):
        raise ValueError("RTD:PoissonXBoundary")
    return v


def y_boundary(mat):
    """eval_Poisson2D_rtd.m:52-62: periodic when the transport's Y boundary is periodic, else
    Neumann, unless mat.poisson.yBoundary overrides."""
    yb = "neumann"
    if str(mat.get("dg", {}).get("params", {}).get("full2D_Y_boundary", "")).lower() == "periodic":
        yb = "periodic"
    yb = str(mat.get("poisson", {}).get("yBoundary", yb)).lower()
    if yb not in ("periodic", "neumann"):
        raise ValueError("RTD:PoissonYBoundary")
    return yb


def doping_si(mat):
    """RTD/get_RTD_doping_SI.m: (Nd, Na) in m^-3 from Nd/Na (SI) or N_d/N_a (cm^-3)."""
    nx, ny = int(mat["Nx"]), int(mat["Ny"])

    def field(si, legacy, required):
        if si in mat:
            return np.asarray(mat[si], dtype=float).reshape(nx, ny)
        if legacy in mat:
            return np.asarray(mat[legacy], dtype=float).reshape(nx, ny) * 1e6
        if required:
            raise ValueError("RTD:MissingDoping")
        return np.zeros((nx, ny))
    return field("Nd", "N_d", True), field("Na", "N_a", False)


def eval_poisson2d(mat):
    """(M [N x N] csr, node_num, node_type, info) (eval_Poisson2D_rtd.m:24-196)."""
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    dx, dy = float(mat["dx"]), float(mat["dy"])
    er = np.asarray(mat["eps"] if "eps" in mat else mat["Eps"], dtype=float).reshape(nx, ny)
    yb = y_boundary(mat)
    periodic = yb == "periodic"
    if periodic and (ny < 3 or np.max(np.abs(er[:, -1] - er[:, 0])) > 1e-12 * er.max()):
        raise ValueError("RTD:PoissonPeriodicMaterial")
    xb = x_boundary(mat)
    if mat.get("boundary") is not None and np.size(mat["boundary"]) > 0:
        boundary = np.asarray(mat["boundary"]).reshape(nx, ny).astype(bool)
    else:
        boundary = np.zeros((nx, ny), dtype=bool)
        if xb == "dirichlet":
            boundary[[0, nx - 1], :] = True
    if xb == "neumann" and boundary.any():
        raise ValueError("RTD:PoissonBoundaryConflict")
    if xb == "dirichlet" and not boundary.any():
        raise ValueError("Dirichlet mode requires at least one fixed potential node.")
    if periodic and not np.array_equal(boundary[:, 0], boundary[:, -1]):
        raise ValueError("RTD:PoissonPeriodicBoundary")
    N = nx * ny
    ids = np.arange(N).reshape(ny, nx).T          # ids[ix, iy] = ix + iy nx
    node_num = np.zeros((nx + 2, ny + 2), dtype=int)
    node_type = np.zeros((nx + 2, ny + 2), dtype=int)
    node_num[1:nx + 1, 1:ny + 1] = ids + 1        # 1-based as in MATLAB
    node_type[1:nx + 1, 1:ny + 1] = 1 + boundary.astype(int)
    if periodic:
        node_type[1:nx + 1, ny] = 3
    rows, cols, vals = [], [], []
    cx = EPS0 * 1e18 / dx ** 2
    cy = EPS0 * 1e18 / dy ** 2
    for iy in range(ny):
        for ix in range(nx):
            k = ids[ix, iy]
            if periodic and iy == ny - 1:
                rows += [k, k]
                cols += [k, ids[ix, 0]]
                vals += [1.0, -1.0]
                continue
            if boundary[ix, iy]:
                rows.append(k); cols.append(k); vals.append(1.0)
                continue
            diag = 0.0
            e0 = er[ix, iy]
            if ix > 0:
                e1 = er[ix - 1, iy]
                c = cx * (2 * e0 * e1 / (e0 + e1))
                if ix == nx - 1:
                    c = 2 * c
                rows.append(k); cols.append(ids[ix - 1, iy]); vals.append(c)
                diag -= c
            if ix < nx - 1:
                e1 = er[ix + 1, iy]
                c = cx * (2 * e0 * e1 / (e0 + e1))
                if ix == 0:
                    c = 2 * c
                rows.append(k); cols.append(ids[ix + 1, iy]); vals.append(c)
                diag -= c
            if iy > 0 or periodic:
                jm = iy - 1
                if jm < 0:
                    jm = ny - 2
                e1 = er[ix, jm]
                c = cy * (2 * e0 * e1 / (e0 + e1))
                if not periodic and iy == ny - 1:
                    c = 2 * c
                rows.append(k); cols.append(ids[ix, jm]); vals.append(c)
                diag -= c
            if iy < ny - 1:
                jp = iy + 1
                if periodic and jp == ny - 1:
                    jp = 0
                e1 = er[ix, jp]
                c = cy * (2 * e0 * e1 / (e0 + e1))
                if not periodic and iy == 0:
                    c = 2 * c
                rows.append(k); cols.append(ids[ix, jp]); vals.append(c)
                diag -= c
            rows.append(k); cols.append(k); vals.append(diag)
    M = sp.csr_matrix((vals, (rows, cols)), shape=(N, N))
    info = {"xBoundary": xb, "yBoundary": yb, "uniqueYNodes": ny - int(periodic)}
    return M, node_num, node_type, info


def solve_poisson2d(M, node_type, node_num, n, mat, phi0, bias):
    """(phi [Nx x Ny], iter_err, info) (solve_Poisson2D_rtd.m:24-131).  n in m^-3 on the
    material grid, phi0 and phi in V."""
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    N = nx * ny
    Nd, Na = doping_si(mat)
    neumann_x = x_boundary(mat) == "neumann"
    types = node_type[1:nx + 1, 1:ny + 1]
    periodic = bool(np.any(types == 3))
    nu = ny - int(periodic)
    bc = np.zeros((nx, ny))
    bc[-1, :] = bias
    if mat.get("Vbc") is not None:
        bc = np.asarray(mat["Vbc"], dtype=float).reshape(nx, ny)
    col = lambda a: np.asarray(a, dtype=float).reshape(nx, ny)[:, :nu].reshape(-1, order="F")
    ut = types[:, :nu].reshape(-1, order="F")
    free = np.flatnonzero(ut == 1)
    fixed = np.flatnonzero(ut == 2)
    if free.size + fixed.size != nx * nu or (not neumann_x and fixed.size == 0) or (neumann_x and fixed.size):
        raise ValueError("RTD:PoissonNodeMap")
    cmap = np.arange(nx * nu).reshape(nu, nx).T
    if periodic:
        cmap = np.concatenate([cmap, cmap[:, :1]], axis=1)
    expand = sp.csr_matrix((np.ones(N), (np.arange(N), cmap.reshape(-1, order="F"))), shape=(N, nx * nu))
    A = (M[:nx * nu, :] @ expand).tocsr()
    old = col(phi0)
    bcu = col(bc)
    nf = col(n)
    net = col(Nd) - col(Na)
    charge = Q * (nf - net)
    v = old.copy()
    v[fixed] = bcu[fixed]
    Av = A @ v
    F = Av - charge
    scale = max(np.abs(Q * nf[free]).max(initial=0), np.abs(Q * net[free]).max(initial=0),
                np.abs(Av[free]).max(initial=0), Q)
    opt = mat.get("poisson", {}).get("opt", {})
    mode = str(opt.get("solve", "direct")).lower()
    alpha = float(opt.get("alpha", 1.0))
    Aff = A[free][:, free].tocsc()
    if mode == "direct":
        if neumann_x:
            raise ValueError("RTD:NeumannNeedsNewton")
        J = Aff
    elif mode in ("newton-raphson", "newton-rhapson"):
        if neumann_x and (np.any(nf < 0) or not np.any(nf > 0)):
            raise ValueError("RTD:NeumannDensityResponse")
        J = (Aff - sp.diags(Q ** 2 * nf[free] / (KB * float(mat["Temp"])))).tocsc()
    else:
        raise ValueError("RTD:UnknownPoissonMethod")
    delta = -spla.spsolve(J, F[free])
    linear_relres = np.abs(J @ delta + F[free]).max() / max(np.abs(F[free]).max(), Q)
    updated = v.copy()
    updated[free] = v[free] + alpha * delta
    phi = (expand @ updated).reshape(ny, nx).T
    iter_err = float(np.linalg.norm(updated[free] - old[free]))
    after = A @ updated - charge
    wx = np.full(nx, float(mat["dx"]) * 1e-9)
    wx[[0, -1]] /= 2
    wy = np.full(nu, float(mat["dy"]) * 1e-9)
    if not periodic and nu > 1:
        wy[[0, -1]] /= 2
    volumes = np.outer(wx, wy).reshape(-1, order="F")
    net_charge = -np.sum(volumes * charge)
    mag = max(Q * max(np.sum(volumes * np.abs(net)), np.sum(volumes * np.abs(nf))), np.finfo(float).tiny)
    info = {"converged": bool(np.all(np.isfinite(updated)) and np.isfinite(linear_relres) and linear_relres < 1e-8),
            "linearRelres": float(linear_relres), "physicalRelresBefore": float(np.abs(F[free]).max() / scale),
            "physicalRelresAfter": float(np.abs(after[free]).max() / scale),
            "physicalResidualBefore": float(np.abs(F[free]).max()), "residualScale": float(scale),
            "unmixedStep": float(np.abs(delta).max()), "alpha": alpha, "netChargePerLength": float(net_charge),
            "relativeChargeImbalance": float(abs(net_charge) / mag), "method": mode}
    return phi, iter_err, info


def _gauss_legendre(nq):
    """project_DG_density_RTD.m:48-52: Golub-Welsch nodes and weights."""
    if nq == 1:
        return np.array([0.0]), np.array([2.0])
    k = np.arange(1, nq)
    off = k / np.sqrt(4 * k ** 2 - 1)
    vals, vecs = np.linalg.eigh(np.diag(off, 1) + np.diag(off, -1))
    order = np.argsort(vals)
    return vals[order], 2 * vecs[0, order] ** 2


def integration_map(axis, nodes):
    """(T [n_nodes x nDof], widths) (project_DG_density_RTD.m:39-69): T[row] integrates each
    element's Lagrange basis over the dual cell of material node `row` (exactly, by an
    n-point Gauss rule per overlap)."""
    nodes = np.asarray(nodes, dtype=float)
    verts = axis["vertices"]
    if nodes.size < 2 or np.any(np.diff(nodes) <= 0) or \
            max(abs(nodes[0] - verts[0]), abs(nodes[-1] - verts[-1])) > 1e-18:
        raise ValueError("RTD:ChargeGridMismatch")
    edges = np.concatenate([[nodes[0]], (nodes[:-1] + nodes[1:]) / 2, [nodes[-1]]])
    widths = np.diff(edges)
    nl = axis["nLocal"]
    T = np.zeros((nodes.size, axis["nDof"]))
    nq = int(np.ceil(nl / 2))
    pts, wts = _gauss_legendre(nq)
    r = axis["r"]
    for e in range(axis["nElements"]):
        left, right = verts[e], verts[e + 1]
        rows = np.flatnonzero((edges[:-1] < right) & (edges[1:] > left))
        cols = slice(e * nl, (e + 1) * nl)
        for row in rows:
            a, b = max(edges[row], left), min(edges[row + 1], right)
            sample = ((a + b) / 2 + (b - a) / 2 * pts - (left + right) / 2) / axis["jacobian"][e]
            basis = np.ones((nq, nl))
            for j in range(nl):
                for k in range(nl):
                    if k != j:
                        basis[:, j] *= (sample - r[k]) / (r[j] - r[k])
            T[row, cols] = (b - a) / 2 * (wts @ basis)
    return T, widths


def project_dg_density(nDG, p, mat, periodic_y):
    """(density [Nx x Ny'], info) (project_DG_density_RTD.m:1-37): nDG [X nDof x Y nDof] on
    the DG nodes; p holds the axes X, Y (nLocal, nElements, nDof, r, M, vertices, jacobian,
    in m) and coordinateScale."""
    if abs(p["coordinateScale"] - 1e-9) > 1e-20:
        raise ValueError("RTD:PoissonCoordinateUnits")
    Tx, wx = integration_map(p["X"], np.asarray(mat["x"], dtype=float) * 1e-9)
    Ty, wy = integration_map(p["Y"], np.asarray(mat["y"], dtype=float) * 1e-9)
    if periodic_y:
        Ty[0] += Ty[-1]
        wy = wy.copy()
        wy[0] += wy[-1]
        Ty, wy = Ty[:-1], wy[:-1]
    volume = np.outer(wx, wy)
    integral = Tx @ nDG @ Ty.T
    density = integral / volume
    src_x = (p["X"]["M"].sum(axis=0)[None, :] * p["X"]["jacobian"][:, None]).ravel()
    src_y = (p["Y"]["M"].sum(axis=0)[None, :] * p["Y"]["jacobian"][:, None]).ravel()
    source = src_x @ nDG @ src_y
    target = integral.sum()
    if periodic_y:
        density = np.concatenate([density, density[:, :1]], axis=1)
    info = {"sourceIntegral": float(source), "targetIntegral": float(target),
            "relativeConservationError": float(abs(target - source) / max(abs(source), np.finfo(float).tiny)),
            "uniqueVolume": volume}
    return density, info
