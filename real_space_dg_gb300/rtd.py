"""Host-side mirror of the reference's RTD self-consistency driver (1D path).

``solve_rtd_self_consistent(mat, biases, options)`` follows
RTD/solve2D_rtd_self_consistent.m:1-205 (options maxIterations, mixing,
potentialTolerance, densityTolerance, poissonResidualTolerance; results with a
``sweep`` of current, density, potential, phi, converged, iterations, status)
for the 1D transport of solve_transport_DG_2D.  The Gummel loop, the Poisson
step and every transport solve run in libwigner_gb300.so.

Two sweep modes:
  * ``sequential``: the reference's bias continuation, one bias after another,
    each seeded by the converged potential and Wigner function of the last;
  * ``batched``: every bias is an independent problem of one handle and all
    Gummel loops advance together on the GPU (initial phi = bias * ramp).
"""
import ctypes as C

import numpy as np

from . import _lib, devices
from ._lib import WignerError
from .transport import M0, Problem1D, shape_from_mat

DEFAULTS = dict(maxIterations=100, mixing=0.1, potentialTolerance=5e-4, densityTolerance=5e-4,
                poissonResidualTolerance=8e-2, transportTolerance=1e-8, transportMaxCycles=50,
                fermiOffset=0.05, restart=50, precision="fp64", innerRestart=40, innerTol=1e-3,
                inexactFactor=0.0, inexactCap=1e-4)


def _opts(options):
    o = dict(DEFAULTS)
    for k, v in (options or {}).items():
        if k not in o:
            raise WignerError(_lib.WG_ERR_ARG, "RTD:UnknownSelfConsistencyOption %s" % k)
        o[k] = v
    if not (0 < o["mixing"] <= 1):
        raise WignerError(_lib.WG_ERR_ARG, "mixing must be in (0, 1]")
    return o


class RTDSweep:
    """A handle of `batch` RTD problems with their Gummel state resident on the GPU."""

    def __init__(self, mat, batch, options=None):
        self.mat = mat
        self.o = _opts(options)
        shp = shape_from_mat(mat)
        self.P = Problem1D(batch=batch, precision=self.o["precision"], restart=self.o["restart"],
                           inner_restart=self.o["innerRestart"], inner_tol=self.o["innerTol"], **shp)
        self.lib = self.P.lib
        self.nx = int(mat["Nx"])
        self.dy = float(mat.get("dy_norm_nm") or devices.density_normalisation_nm(mat, self.o["fermiOffset"]))
        x = np.ascontiguousarray(mat["x"], dtype=float)
        m = np.ascontiguousarray(np.asarray(mat["me_x"], dtype=float).reshape(-1, self.nx, int(mat["Ny"]))[0, :, 0]
                                 * M0)
        self._keep = [x, m]
        self.dev = _lib.WgDevice(self.nx, _lib.dptr(x), _lib.dptr(m), float(mat["me_z_ch"]), float(mat["Temp"]))
        self.vc = np.ascontiguousarray(mat["Vc"], dtype=float)
        self.nd = np.ascontiguousarray(mat["Nd"], dtype=float)
        self.eps = np.ascontiguousarray(mat["eps"], dtype=float)
        self.ramp = np.asarray(mat["ramp"], dtype=float)

    def close(self):
        self.P.close()

    def set(self, b, bias, phi0=None):
        phi0 = np.ascontiguousarray(bias * self.ramp if phi0 is None else phi0, dtype=float)
        rtd = _lib.WgRtd1D(_lib.dptr(self.vc), _lib.dptr(self.nd), _lib.dptr(self.eps), _lib.dptr(phi0),
                           float(bias), float(self.o["fermiOffset"]), self.dy)
        self.P._check(self.lib.wg_gummel_set(self.P.h, int(b), C.byref(self.dev), C.byref(rtd)))

    def run(self, warm_start=False, restart_from_phi0=False):
        o = self.o
        go = _lib.WgGummelOpts(int(o["maxIterations"]), float(o["mixing"]), float(o["potentialTolerance"]),
                               float(o["densityTolerance"]), float(o["poissonResidualTolerance"]),
                               float(o["transportTolerance"]), int(o["transportMaxCycles"]), 1 if warm_start else 0,
                               1 if restart_from_phi0 else 0, float(o["inexactFactor"]), float(o["inexactCap"]))
        info = (_lib.WgGummelInfo * self.P.batch)()
        st = self.lib.wg_gummel_run(self.P.h, C.byref(go), info)
        self.P._check(st, allow_not_converged=True)
        return st, [i.as_dict() for i in info]

    def get(self, b):
        phi = np.empty(self.nx); n = np.empty(self.P.ncol); j = np.empty(self.P.ncol)
        self.P._check(self.lib.wg_gummel_get(self.P.h, int(b), _lib.dptr(phi), _lib.dptr(n), _lib.dptr(j)))
        return phi, n, j


def solve_rtd_self_consistent(mat, biases, options=None, mode="batched"):
    """results = solve2D_rtd_self_consistent('DG', mat, options) for the 1D path.

    Returns a dict with ``sweep`` (bias, current [Nxdof x nb], density, potential,
    phi, converged, iterations, status, gmres_iterations), ``Id`` (mean current per
    bias, results.Id of the reference) and ``selfConsistency``.
    """
    biases = np.atleast_1d(np.asarray(biases, dtype=float))
    nb = len(biases)
    batch = nb if mode == "batched" else 1
    S = RTDSweep(mat, batch, options)
    sweep = {"bias": biases, "current": [], "density": [], "potential": [], "phi": [], "converged": [],
             "iterations": [], "status": [], "gmres_iterations": [], "transport_relres": []}
    try:
        if mode == "batched":
            for b, v in enumerate(biases):
                S.set(b, v)
            st, info = S.run()
            results = [(info[b], S.get(b)) for b in range(nb)]
        else:
            results = []
            phi_prev = None
            for ib, v in enumerate(biases):
                phi0 = v * S.ramp if ib == 0 else phi_prev + (v - biases[ib - 1]) * S.ramp
                S.set(0, v, phi0)
                st, info = S.run(warm_start=ib > 0)
                results.append((info[0], S.get(0)))
                phi_prev = results[-1][1][0]
                if info[0]["status"] != 0:
                    break                      # no bias continuation from an unconverged state
        for inf, (phi, n, j) in results:
            sweep["current"].append(j)
            sweep["density"].append(n)
            sweep["phi"].append(phi)
            sweep["potential"].append(S.vc - phi)
            sweep["converged"].append(inf["status"] == 0)
            sweep["iterations"].append(inf["iterations"])
            sweep["status"].append(_lib.GUMMEL_STATUS.get(inf["status"], str(inf["status"])))
            sweep["gmres_iterations"].append(inf["gmres_iterations"])
            sweep["transport_relres"].append(inf["transport_relres"])
    finally:
        S.close()
    for k in ("current", "density", "phi", "potential"):
        sweep[k] = np.array(sweep[k]).T
    Id = sweep["current"].mean(axis=0) if len(sweep["current"]) else np.array([])
    return {"sweep": sweep, "Id": Id,
            "selfConsistency": {"converged": bool(all(sweep["converged"]) and len(sweep["converged"]) == nb),
                                "iterations": sweep["iterations"], "status": sweep["status"]}}
