"""2D Poisson step of the Full-2D Gummel loop on the GPU.

Host side of ``wg_poisson2d_*`` (libwigner_gb300.so), mirroring the reference's functions:

  eval_Poisson2D_rtd(mat)                      -> (op, node_num, node_type, info)
                                                  (RTD/eval_Poisson2D_rtd.m:1-196; ``op`` is the
                                                  device-resident operator in place of the sparse M)
  solve_Poisson2D_rtd(op, node_type, node_num, n, mat, phi0, bias) -> (phi, iter_err, info)
                                                  (RTD/solve_Poisson2D_rtd.m:1-131)
  project_DG_density_RTD(nDG, p, mat, periodicY) -> (density, info)
                                                  (RTD/project_DG_density_RTD.m:1-37)
  make_RTD_poisson_step(mat, method)           -> (step, setup)
                                                  (RTD/make_RTD_poisson_step.m:1-55; ``step`` runs
                                                  projection + update as one device call)

Arrays are [Nx, Ny] as in the reference (SI densities, potentials in V); a ``Poisson2D`` with
``batch`` > 1 takes and returns a leading bias-point axis.
"""
import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import WignerError

INFO_FIELDS = [f for f, _ in _lib.WgPoisson2dInfo._fields_]


def _ybc(mat):
    """Y boundary of the Poisson grid (eval_Poisson2D_rtd.m:52-62)."""
    yb = "neumann"
    if str(mat.get("dg", {}).get("params", {}).get("full2D_Y_boundary", "")).lower() == "periodic":
        yb = "periodic"
    yb = str(mat.get("poisson", {}).get("yBoundary", yb)).lower()
    if yb not in ("periodic", "neumann"):
        raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonYBoundary: use periodic or neumann")
    return yb


def _xbc(mat):
    """RTD/get_RTD_poisson_x_boundary.m."""
    xb = str(mat.get("poisson", {}).get("xBoundary", "dirichlet")).lower()
    if xb not in ("dirichlet", "neumann"):
        raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonXBoundary")
    return xb


def _doping(mat, nx, ny):
    """RTD/get_RTD_doping_SI.m: Nd/Na in m^-3 (or legacy N_d/N_a in cm^-3)."""
    def field(si, legacy, required):
        if si in mat:
            return np.asarray(mat[si], dtype=float).reshape(nx, ny)
        if legacy in mat:
            return np.asarray(mat[legacy], dtype=float).reshape(nx, ny) * 1e6
        if required:
            raise WignerError(_lib.WG_ERR_ARG, "RTD:MissingDoping: provide mat.Nd [m^-3] or mat.N_d [cm^-3]")
        return np.zeros((nx, ny))
    return field("Nd", "N_d", True), field("Na", "N_a", False)


def _c(a):
    """[Nx, Ny] (or [B, Nx, Ny]) -> C-contiguous x-fastest [.., Ny, Nx]."""
    a = np.asarray(a, dtype=float)
    return np.ascontiguousarray(np.swapaxes(a, -1, -2))


def _axis(ax):
    """A DG axis in either naming (the reference's nLocal/nElements/... or nl/ne/...)."""
    if "nLocal" in ax:
        return dict(nl=ax["nLocal"], ne=ax["nElements"], nd=ax["nDof"], r=np.asarray(ax["r"]), M=np.asarray(ax["M"]),
                    verts=np.asarray(ax["vertices"], dtype=float), jac=np.asarray(ax["jacobian"], dtype=float))
    return dict(nl=ax["nl"], ne=ax["ne"], nd=ax["nd"], r=np.asarray(ax["r"]), M=np.asarray(ax["M"]),
                verts=np.asarray(ax["verts"], dtype=float), jac=np.asarray(ax["jac"], dtype=float))


def integration_map(ax, nodes):
    """(T [n_nodes x nDof] as CSR arrays (rp, col, val), widths, dense T) of the dual cells of the
    material nodes (project_DG_density_RTD.m:39-69): T[row, element dofs] integrates each Lagrange
    basis function of an overlapping element over the overlap exactly (ceil(nl/2)-point Gauss)."""
    nodes = np.asarray(nodes, dtype=float)
    verts = ax["verts"]
    if nodes.size < 2 or np.any(np.diff(nodes) <= 0) or \
            max(abs(nodes[0] - verts[0]), abs(nodes[-1] - verts[-1])) > 1e-18:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:ChargeGridMismatch: DG and Poisson grids must cover the same interval")
    edges = np.concatenate([[nodes[0]], 0.5 * (nodes[:-1] + nodes[1:]), [nodes[-1]]])
    widths = np.diff(edges)
    nl, r = ax["nl"], ax["r"]
    pts, wts = np.polynomial.legendre.leggauss(int(math.ceil(nl / 2)))
    T = np.zeros((nodes.size, ax["nd"]))
    others = [np.delete(np.arange(nl), j) for j in range(nl)]
    for e in range(ax["ne"]):
        left, right = verts[e], verts[e + 1]
        for row in np.flatnonzero((edges[:-1] < right) & (edges[1:] > left)):
            a, b = max(edges[row], left), min(edges[row + 1], right)
            xi = ((a + b) / 2 + (b - a) / 2 * pts - (left + right) / 2) / ax["jac"][e]
            basis = np.stack([np.prod((xi[:, None] - r[others[j]][None, :]) / (r[j] - r[others[j]])[None, :], axis=1)
                              for j in range(nl)], axis=1)
            T[row, e * nl:(e + 1) * nl] = (b - a) / 2 * (wts @ basis)
    return T, widths


def _csr(T):
    rp = [0]
    col, val = [], []
    for row in T:
        nz = np.flatnonzero(row)
        col.extend(nz.tolist())
        val.extend(row[nz].tolist())
        rp.append(len(col))
    return (np.asarray(rp, dtype=np.int32), np.asarray(col, dtype=np.int32), np.asarray(val, dtype=float))


def projection_maps(p, mat, periodic_y):
    """Tx, Ty (dense), wx, wy and the element-integral weights of project_DG_density_RTD.m:16-28
    with the periodic endpoint merged (Ty row 1 += row end, the last row dropped)."""
    if abs(float(p.get("coordinateScale", 1e-9)) - 1e-9) > 1e-20:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonCoordinateUnits: material coordinates must be in nm")
    X, Y = _axis(p["X"]), _axis(p["Y"])
    Tx, wx = integration_map(X, np.asarray(mat["x"], dtype=float) * 1e-9)
    Ty, wy = integration_map(Y, np.asarray(mat["y"], dtype=float) * 1e-9)
    if periodic_y:
        Ty = Ty.copy()
        Ty[0] += Ty[-1]
        wy = wy.copy()
        wy[0] += wy[-1]
        Ty, wy = Ty[:-1], wy[:-1]
    sx = (X["M"].sum(axis=0)[None, :] * X["jac"][:, None]).ravel()
    sy = (Y["M"].sum(axis=0)[None, :] * Y["jac"][:, None]).ravel()
    return Tx, Ty, wx, wy, sx, sy


class Poisson2D:
    """Device-resident 2D Poisson operator and step of one material grid (eval_Poisson2D_rtd's
    M and node maps), for ``batch`` bias points per call."""

    def __init__(self, mat, batch=1):
        self.lib = _lib.load()
        nx, ny = int(mat["Nx"]), int(mat["Ny"])
        self.nx, self.ny, self.batch = nx, ny, int(batch)
        self.ybc, self.xbc = _ybc(mat), _xbc(mat)
        self.periodic = self.ybc == "periodic"
        er = mat["eps"] if "eps" in mat else mat.get("Eps")
        if er is None:
            raise WignerError(_lib.WG_ERR_ARG, "eval_Poisson:MissingEps: mat.eps (relative permittivity) is required")
        for name, n_ in (("x", nx), ("y", ny)):
            if name in mat:
                g = np.asarray(mat[name], dtype=float).ravel()
                step = float(mat["d" + name])
                if g.size != n_ or np.any(np.abs(np.diff(g) - step) > 1e-10 * step):
                    raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonUniformGrid: mat.%s must agree with its uniform "
                                                       "spacing in nm" % name)
        nd, na = _doping(mat, nx, ny)
        bnd = mat.get("boundary")
        bptr = None
        if bnd is not None and np.size(bnd) > 0:
            b = np.asarray(bnd).reshape(nx, ny)
            if not np.all(np.isin(b, [0, 1])):
                raise WignerError(_lib.WG_ERR_ARG, "mat.boundary must contain only 0 (free) and 1 (Dirichlet)")
            self._bnd = np.ascontiguousarray(b.T.astype(np.uint8))
            bptr = self._bnd.ctypes.data_as(C.POINTER(C.c_ubyte))
            fixed = b.astype(bool)
        else:
            fixed = np.zeros((nx, ny), dtype=bool)
            if self.xbc == "dirichlet":
                fixed[[0, -1], :] = True
        self.fixed = fixed
        d = _lib.WgPoisson2dDesc(nx, ny, float(mat["dx"]), float(mat["dy"]), int(self.periodic),
                                 int(self.xbc == "neumann"), float(mat.get("Temp", 300.0)), self.batch)
        eps_c, nd_c, na_c = _c(np.asarray(er, dtype=float).reshape(nx, ny)), _c(nd), _c(na)
        h = _lib._H()
        rc = self.lib.wg_poisson2d_create(C.byref(d), _lib.dptr(eps_c), bptr, _lib.dptr(nd_c), _lib.dptr(na_c),
                                          C.byref(h))
        if rc != _lib.WG_OK:
            raise WignerError(rc, "wg_poisson2d_create rejected the grid (Nx >= 2, unique Ny <= 32, eps > 0, "
                                  "matching periodic endpoints, a Dirichlet node unless Neumann X, none with it)")
        self.h = h
        self.has_projection = False

    def _check(self, rc):
        if rc != _lib.WG_OK:
            raise WignerError(rc, self.lib.wg_poisson2d_last_error(self.h).decode())

    def _batched(self, a, shape):
        a = np.asarray(a, dtype=float)
        return a.reshape((self.batch,) + shape)

    def apply(self, phi):
        """M phi (the reference's operator with all its rows), phi [Nx, Ny] or [B, Nx, Ny]."""
        x = _c(self._batched(phi, (self.nx, self.ny)))
        y = np.empty_like(x)
        self._check(self.lib.wg_poisson2d_apply(self.h, _lib.dptr(x), _lib.dptr(y)))
        out = np.swapaxes(y, -1, -2)
        return out[0] if self.batch == 1 and np.ndim(phi) == 2 else out

    def set_projection(self, p, mat):
        """Hand the DG -> dual-volume maps of the transport axes p['X'], p['Y'] to the device."""
        Tx, Ty, wx, wy, sx, sy = projection_maps(p, mat, self.periodic)
        (a, b, c), (d, e, f) = _csr(Tx), _csr(Ty)
        self._proj = (a, b, c, d, e, f, np.ascontiguousarray(wx), np.ascontiguousarray(wy), sx, sy)
        ip = lambda v: v.ctypes.data_as(C.POINTER(C.c_int))
        self._check(self.lib.wg_poisson2d_set_projection(self.h, Tx.shape[1], ip(a), ip(b), _lib.dptr(c), Ty.shape[1],
                                                         ip(d), ip(e), _lib.dptr(f), _lib.dptr(self._proj[6]),
                                                         _lib.dptr(self._proj[7]), _lib.dptr(sx), _lib.dptr(sy)))
        self.ndx, self.ndy = Tx.shape[1], Ty.shape[1]
        self.has_projection = True

    def solve(self, n, phi0, bias, method="direct", alpha=1.0, vbc=None, dg=False):
        """One update (solve_Poisson2D_rtd.m:64-131): n [Nx, Ny] in m^-3 (or nDG [X nDof, Y nDof]
        with dg=True, projected on the device first), phi0 [Nx, Ny], bias (V, per problem) or
        vbc [Nx, Ny].  Returns (phi, density, info) with the batch axis when batch > 1."""
        method = str(method).lower()
        if method not in ("direct", "newton-raphson", "newton-rhapson"):
            raise WignerError(_lib.WG_ERR_ARG, "RTD:UnknownPoissonMethod: use direct or newton-raphson, not %s"
                              % method)
        if not (0 < alpha <= 1):
            raise WignerError(_lib.WG_ERR_ARG, "opt.alpha must be in (0, 1]")
        B = self.batch
        src = _c(self._batched(n, (self.ndx, self.ndy) if dg else (self.nx, self.ny)))
        p0 = _c(self._batched(phi0, (self.nx, self.ny)))
        bias_a = np.ascontiguousarray(np.broadcast_to(np.asarray(bias, dtype=float), (B,))) if bias is not None \
            else None
        vbc_a = _c(self._batched(vbc, (self.nx, self.ny))) if vbc is not None else None
        phi = np.empty((B, self.ny, self.nx))
        dens = np.empty((B, self.ny, self.nx))
        infos = (_lib.WgPoisson2dInfo * B)()
        self._check(self.lib.wg_poisson2d_solve(self.h, _lib.dptr(src), int(dg), _lib.dptr(p0),
                                                _lib.dptr(bias_a) if bias_a is not None else None,
                                                _lib.dptr(vbc_a) if vbc_a is not None else None,
                                                int(method != "direct"), float(alpha), _lib.dptr(phi),
                                                _lib.dptr(dens), infos))
        info = [{f: getattr(infos[b], f) for f in INFO_FIELDS} for b in range(B)]
        for i in info:
            i["converged"] = bool(i["converged"])
            i["method"] = method
            i["alpha"] = alpha
        phi, dens = np.swapaxes(phi, -1, -2), np.swapaxes(dens, -1, -2)
        if B == 1:
            return phi[0], dens[0], info[0]
        return phi, dens, info

    def buffers(self):
        p = [C.c_void_p() for _ in range(5)]
        self._check(self.lib.wg_poisson2d_buffers(self.h, *[C.byref(x) for x in p]))
        return tuple(x.value for x in p)

    def close(self):
        if getattr(self, "h", None):
            self.lib.wg_poisson2d_destroy(self.h)
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


def eval_Poisson2D_rtd(mat):
    """(op, node_num, node_type, info) (eval_Poisson2D_rtd.m:1-196): ``op`` is the device
    operator (``op.apply(phi)`` = M phi); node_num/node_type carry the reference's ghost frame
    (1-based numbers; types 0 outside, 1 free, 2 Dirichlet, 3 periodic duplicate)."""
    op = Poisson2D(mat)
    nx, ny = op.nx, op.ny
    node_num = np.zeros((nx + 2, ny + 2), dtype=int)
    node_type = np.zeros((nx + 2, ny + 2), dtype=int)
    node_num[1:nx + 1, 1:ny + 1] = np.arange(1, nx * ny + 1).reshape(ny, nx).T
    node_type[1:nx + 1, 1:ny + 1] = 1 + op.fixed.astype(int)
    if op.periodic:
        node_type[1:nx + 1, ny] = 3
    info = {"xBoundary": op.xbc, "yBoundary": op.ybc, "uniqueYNodes": ny - int(op.periodic),
            "potentialUnits": "V", "operator": "div(epsilon*grad(phi))", "interfaceMean": "harmonic",
            "periodicEndpointDuplicated": op.periodic}
    return op, node_num, node_type, info


def solve_Poisson2D_rtd(M, node_type, node_num, n, mat, phi0, bias):
    """(phi, iter_err, info) (solve_Poisson2D_rtd.m:1-131) with ``M`` the operator of
    eval_Poisson2D_rtd; mat.poisson.opt.solve ('direct' / 'newton-raphson') and .alpha as there."""
    opt = mat.get("poisson", {}).get("opt", {})
    phi, dens, info = M.solve(n, phi0, bias, method=opt.get("solve", "direct"), alpha=float(opt.get("alpha", 1.0)),
                              vbc=mat.get("Vbc"))
    return phi, info["iter_err"], info


def project_DG_density_RTD(nDG, p, mat, periodicY):
    """(density [Nx, Ny], info) (project_DG_density_RTD.m:1-37) on the host: Tx nDG Ty^T over the
    dual volumes (the device runs the same contraction inside the Poisson step)."""
    Tx, Ty, wx, wy, sx, sy = projection_maps(p, mat, bool(periodicY))
    nDG = np.asarray(nDG, dtype=float)
    integral = Tx @ nDG @ Ty.T
    density = integral / np.outer(wx, wy)
    if periodicY:
        density = np.concatenate([density, density[:, :1]], axis=1)
    source, target = float(sx @ nDG @ sy), float(integral.sum())
    return density, {"sourceIntegral": source, "targetIntegral": target,
                     "relativeConservationError": abs(target - source) / max(abs(source), np.finfo(float).tiny)}


def make_RTD_poisson_step(mat, method="direct"):
    """(step, setup) (RTD/make_RTD_poisson_step.m:1-55): ``step(state)`` takes
    state['transport']['nDG'], state['transport']['p'], state['phi'], state['bias'] and returns
    (phi, info), the projection and the update in one device call."""
    method = str(method).lower()
    if method not in ("direct", "newton-raphson", "newton-rhapson"):
        raise WignerError(_lib.WG_ERR_ARG, "RTD:UnknownPoissonMethod: use direct or newton-raphson")
    if _xbc(mat) == "neumann" and method == "direct":
        raise WignerError(_lib.WG_ERR_ARG, "RTD:NeumannNeedsNewton: Neumann X requires newton-raphson")
    if mat.get("Vbc") is not None:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonContactModel: the coupled RTD sets contact values from bias")
    op, node_num, node_type, setup = eval_Poisson2D_rtd(mat)
    if mat.get("boundary") is not None and np.size(mat["boundary"]) > 0:
        expected = np.zeros((op.nx, op.ny), dtype=bool)
        if op.xbc == "dirichlet":
            expected[[0, -1], :] = True
        if not np.array_equal(np.asarray(mat["boundary"]).astype(bool).reshape(op.nx, op.ny), expected):
            raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonContactModel: full source/drain contacts only")
    setup = dict(setup, method=method, approximateNewton=method != "direct", operator=op)
    state_p = {}

    def step(state, *_):
        tr = state["transport"]
        if state_p.get("p") is not tr["p"]:
            op.set_projection(tr["p"], mat)
            state_p["p"] = tr["p"]
        phi, dens, info = op.solve(tr["nDG"], state["phi"], state["bias"], method=method, alpha=1.0, dg=True)
        info["electronDensity"] = dens
        info["chargeTransfer"] = {"sourceIntegral": info["source_integral"], "targetIntegral": info["target_integral"]}
        return phi, info

    return step, setup
