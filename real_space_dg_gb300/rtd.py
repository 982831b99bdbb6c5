"""Host-side mirror of the reference's RTD self-consistency driver (1D path).

``solve_rtd_self_consistent(mat, biases, options)`` follows
RTD/solve2D_rtd_self_consistent.m:1-205 (options maxIterations, mixing,
potentialTolerance, densityTolerance, poissonResidualTolerance; results with a
``sweep`` of current, density, potential, phi, converged, iterations, status)
for the 1D transport of solve_transport_DG_2D.  The Gummel loop, the Poisson
step and every transport solve run in libwigner_gb300.so.

``solve_transient_self_consistent(mat, bias0, steps, options)`` follows
DG_code/solve_transport_DG_2D_transient_SC_new.m:1-221: from the stationary
self-consistent state at bias0 (the reference's INIT) every problem of the
batch takes a drain-bias step at t = 0 and is integrated in time (RK4 or
Crank-Nicolson) with the potential re-solved on the reference's schedule.

Two sweep modes:
  * ``sequential``: the reference's bias continuation, one bias after another,
    each seeded by the converged potential and Wigner function of the last;
  * ``batched``: every bias is an independent problem of one handle and all
    Gummel loops advance together on the GPU (initial phi = bias * ramp).
"""
import atexit
import ctypes as C
import threading

import numpy as np

from . import _lib, devices
from ._lib import WignerError
from .transport import M0, Problem1D, shape_from_mat

DEFAULTS = dict(maxIterations=100, mixing=0.1, potentialTolerance=5e-4, densityTolerance=5e-4,
                poissonResidualTolerance=8e-2, transportTolerance=1e-8, transportMaxCycles=50,
                fermiOffset=0.05, restart=50, precision="fp64", innerRestart=40, innerTol=1e-3,
                inexactFactor=0.0, inexactCap=1e-4, reorth=0.0, innerReorth=0.0, fp64TensorCores=False,
                deferFinal=0, keepHandles=True, innerBasisFP32=False)


def _opts(options):
    o = dict(DEFAULTS)
    for k, v in (options or {}).items():
        if k not in o:
            raise WignerError(_lib.WG_ERR_ARG, "RTD:UnknownSelfConsistencyOption %s" % k)
        o[k] = v
    if not (0 < o["mixing"] <= 1):
        raise WignerError(_lib.WG_ERR_ARG, "mixing must be in (0, 1]")
    return o


def _grid_key(mat):
    """What a handle's device buffers are sized and its operator shape is built from (the node
    positions, masses and potentials are per problem, set by ``set``)."""
    return tuple(sorted(shape_from_mat(mat).items())) + (int(mat["Nx"]), int(mat["Ny"]))


class RTDSweep:
    """A handle of `batch` RTD problems with their Gummel state resident on the GPU."""

    def __init__(self, mat, batch, options=None):
        self.o = _opts(options)
        shp = shape_from_mat(mat)
        self.P = Problem1D(batch=batch, precision=self.o["precision"], restart=self.o["restart"],
                           inner_restart=self.o["innerRestart"], inner_tol=self.o["innerTol"],
                           reorth=self.o["reorth"], inner_reorth=self.o["innerReorth"],
                           fp64_tc=self.o["fp64TensorCores"], inner_basis_fp32=self.o["innerBasisFP32"], **shp)
        self.lib = self.P.lib
        self.nx = int(mat["Nx"])
        self.grid = _grid_key(mat)
        self.bind(mat)

    def bind(self, mat):
        """The device description (band edge, doping, permittivity, masses, ramp) that ``set``
        gives every problem without a ``mat`` of its own; ``mat`` has this handle's grid."""
        if _grid_key(mat) != self.grid:
            raise WignerError(_lib.WG_ERR_ARG, "bind: the device needs the node count and shape of this handle")
        self.mat = mat
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

    def set(self, b, bias, phi0=None, mat=None):
        """Problem b at ``bias``; ``mat`` (same grid) gives it its own device data."""
        if mat is None:
            vc, nd, eps, dev, ramp = self.vc, self.nd, self.eps, self.dev, self.ramp
        else:
            if int(mat["Nx"]) != self.nx:
                raise WignerError(_lib.WG_ERR_ARG, "every problem of a handle needs the same grid")
            x = np.ascontiguousarray(mat["x"], dtype=float)
            m = np.ascontiguousarray(np.asarray(mat["me_x"], dtype=float).reshape(-1, self.nx,
                                                                                  int(mat["Ny"]))[0, :, 0] * M0)
            vc = np.ascontiguousarray(mat["Vc"], dtype=float)
            nd = np.ascontiguousarray(mat["Nd"], dtype=float)
            eps = np.ascontiguousarray(mat["eps"], dtype=float)
            dev = _lib.WgDevice(self.nx, _lib.dptr(x), _lib.dptr(m), float(mat["me_z_ch"]), float(mat["Temp"]))
            ramp = np.asarray(mat["ramp"], dtype=float)
        phi0 = np.ascontiguousarray(bias * ramp if phi0 is None else phi0, dtype=float)
        rtd = _lib.WgRtd1D(_lib.dptr(vc), _lib.dptr(nd), _lib.dptr(eps), _lib.dptr(phi0),
                           float(bias), float(self.o["fermiOffset"]), self.dy)
        self.P._check(self.lib.wg_gummel_set(self.P.h, int(b), C.byref(dev), C.byref(rtd)))

    def run(self, warm_start=False, restart_from_phi0=False):
        o = self.o
        go = _lib.WgGummelOpts(int(o["maxIterations"]), float(o["mixing"]), float(o["potentialTolerance"]),
                               float(o["densityTolerance"]), float(o["poissonResidualTolerance"]),
                               float(o["transportTolerance"]), int(o["transportMaxCycles"]), 1 if warm_start else 0,
                               1 if restart_from_phi0 else 0, float(o["inexactFactor"]), float(o["inexactCap"]),
                               int(o["deferFinal"]))
        info = (_lib.WgGummelInfo * self.P.batch)()
        st = self.lib.wg_gummel_run(self.P.h, C.byref(go), info)
        self.P._check(st, allow_not_converged=True)
        return st, [i.as_dict() for i in info]

    def get(self, b):
        phi = np.empty(self.nx); n = np.empty(self.P.ncol); j = np.empty(self.P.ncol)
        self.P._check(self.lib.wg_gummel_get(self.P.h, int(b), _lib.dptr(phi), _lib.dptr(n), _lib.dptr(j)))
        return phi, n, j

    def step_bias(self, b, bias):
        """Drain-bias step of problem b at t = 0 of the next transient()."""
        self.P._check(self.lib.wg_transient_set_bias(self.P.h, int(b), float(bias)))

    def transient(self, dt, nsteps, method="cn", scale_a=0.0, scale_rhs=0.0, refresh_every=0, refresh_first=0,
                  tol=0.0, maxit=0, record_every=1, fixed_rhs=False):
        """Advance every problem by nsteps; returns (status, info, n [nrec, batch, ncol], j).
        fixed_rhs: keep the resident right-hand side at every refresh (the reference's rhs_INIT)."""
        if method not in _lib.TRANSIENT_METHODS:
            raise WignerError(_lib.WG_ERR_ARG, "unknown transient method %r" % (method,))
        o = _lib.WgTransientOpts(float(dt), int(nsteps), _lib.TRANSIENT_METHODS[method], float(scale_a),
                                 float(scale_rhs), int(refresh_every), int(refresh_first), float(tol), int(maxit),
                                 int(record_every), 1 if fixed_rhs else 0)
        nrec = nsteps // record_every if record_every > 0 else 0
        n = np.zeros((nrec, self.P.batch, self.P.ncol))
        j = np.zeros((nrec, self.P.batch, self.P.ncol))
        info = (_lib.WgTransientInfo * self.P.batch)()
        st = self.lib.wg_transient_run(self.P.h, C.byref(o), _lib.dptr(n), _lib.dptr(j), info)
        self.P._check(st, allow_not_converged=True)
        return st, [i.as_dict() for i in info], n, j


def run_concurrent(sweeps, **kw):
    """Run the Gummel loops of several handles at once, one host thread per handle: each handle
    works on its own CUDA stream, so the latency-bound launch chains of the handles overlap on the
    device.  Returns [(status, info)] per handle; an error of any handle is raised."""
    out = [None] * len(sweeps)
    errors = []

    def work(k):
        try:
            out[k] = sweeps[k].run(**kw)
        except Exception as e:            # re-raised on the calling thread
            errors.append(e)
    if len(sweeps) == 1:
        work(0)
    else:
        threads = [threading.Thread(target=work, args=(k,)) for k in range(len(sweeps))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    if errors:
        raise errors[0]
    return out


_KEPT = {"key": None, "sweeps": []}
_KEPT_LOCK = threading.Lock()


def _take_kept(key):
    """The kept handles when they match ``key`` (taken out under the lock, so that a concurrent
    call cannot share them), else None."""
    with _KEPT_LOCK:
        if _KEPT["key"] != key:
            return None
        sweeps = _KEPT["sweeps"]
        _KEPT.update(key=None, sweeps=[])
    return sweeps


def _keep(key, sweeps):
    """Keep ``sweeps`` for the next call; a set kept meanwhile by another thread is closed."""
    with _KEPT_LOCK:
        old = _KEPT["sweeps"]
        _KEPT.update(key=key, sweeps=sweeps)
    for sw in old:
        sw.close()


def release_handles():
    """Close the handles solve_rtd_self_consistent keeps for its next call."""
    with _KEPT_LOCK:
        sweeps = _KEPT["sweeps"]
        _KEPT.update(key=None, sweeps=[])
    for sw in sweeps:
        sw.close()


atexit.register(release_handles)


def solve_rtd_self_consistent(mat, biases, options=None, mode="batched", handles=1):
    """results = solve2D_rtd_self_consistent('DG', mat, options) for the 1D path.

    Returns a dict with ``sweep`` (bias, current [Nxdof x nb], density, potential,
    phi, converged, iterations, status, gmres_iterations), ``Id`` (mean current per
    bias, results.Id of the reference) and ``selfConsistency``.  ``handles`` (batched
    mode): the biases are dealt round-robin to that many handles that run concurrently
    on their own streams (each bias' result is the same as in one handle).

    ``keepHandles`` (option, default on): the handles stay open after the call and serve the
    next call with the same shape, batch layout and options (another device of the same node
    count included), which then skips their allocation and set-up; every problem still starts
    from its own phi0 = bias * ramp with a zero Wigner function, so the results are those of
    fresh handles.  One set is kept; ``release_handles()`` frees it.
    """
    biases = np.atleast_1d(np.asarray(biases, dtype=float))
    nb = len(biases)
    o = _opts(options)
    K = max(1, min(int(handles), nb)) if mode == "batched" else 1
    sizes = [len(range(k, nb, K)) for k in range(K)] if mode == "batched" else [1]
    keep = bool(o["keepHandles"])
    key = (_grid_key(mat), tuple(sizes), repr(sorted((k, v) for k, v in o.items() if k != "keepHandles")))
    sweeps = _take_kept(key) if keep else None
    if sweeps is None:
        release_handles()
        sweeps = []
        try:
            for sz in sizes:
                sweeps.append(RTDSweep(mat, sz, o))
        except BaseException:
            for sw in sweeps:
                sw.close()
            raise
    else:
        for sw in sweeps:
            sw.bind(mat)
    S = sweeps[0]
    sweep = {"bias": biases, "current": [], "density": [], "potential": [], "phi": [], "converged": [],
             "iterations": [], "status": [], "gmres_iterations": [], "transport_relres": []}
    try:
        if mode == "batched":
            for i, v in enumerate(biases):
                sweeps[i % K].set(i // K, v)
            outs = run_concurrent(sweeps)
            results = [(outs[i % K][1][i // K], sweeps[i % K].get(i // K)) for i in range(nb)]
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
    except BaseException:
        for sw in sweeps:
            sw.close()
        raise
    if keep:
        _keep(key, sweeps)
    else:
        for sw in sweeps:
            sw.close()
    for k in ("current", "density", "phi", "potential"):
        sweep[k] = np.array(sweep[k]).T
    Id = sweep["current"].mean(axis=0) if len(sweep["current"]) else np.array([])
    return {"sweep": sweep, "Id": Id,
            "selfConsistency": {"converged": bool(all(sweep["converged"]) and len(sweep["converged"]) == nb),
                                "iterations": sweep["iterations"], "status": sweep["status"]}}


TRANSIENT_DEFAULTS = dict(dt=1e-15, steps=100, method="cn", scaleA=2e-10, scaleRhs=0.0, refreshEvery=20,
                          refreshFirst=50, stepTolerance=1e-10, stepMaxCycles=20, recordEvery=1)


def solve_transient_self_consistent(mat, bias0, steps, options=None, transient=None):
    """DG = solve_transport_DG_2D_transient_SC_new(mat, INIT) for the 1D RTD, batched.

    bias0: the stationary bias of INIT; steps: the bias after the step, one
    transient per entry, all advanced together.  ``options`` are the Gummel
    options of the stationary state (solve_rtd_self_consistent); ``transient``
    overrides TRANSIENT_DEFAULTS.  Returns n_over_t / j_over_t as
    [n_el*n_local, nrec, n_transients] (DG.n_over_t / DG.j_over_t), the time
    axis t, the final potential phi and per-transient info.
    """
    steps = np.atleast_1d(np.asarray(steps, dtype=float))
    T = dict(TRANSIENT_DEFAULTS)
    for k, v in (transient or {}).items():
        if k not in T:
            raise WignerError(_lib.WG_ERR_ARG, "unknown transient option %s" % k)
        T[k] = v
    S = RTDSweep(mat, len(steps), options)
    try:
        for b in range(len(steps)):
            S.set(b, bias0)
        st, ginfo = S.run()
        if st != 0:
            raise WignerError(st, "stationary state at bias0 did not converge: %s" % [g["status"] for g in ginfo])
        for b, v in enumerate(steps):
            S.step_bias(b, v)
        st, info, n, j = S.transient(T["dt"], int(T["steps"]), T["method"], T["scaleA"], T["scaleRhs"],
                                     int(T["refreshEvery"]), int(T["refreshFirst"]), T["stepTolerance"],
                                     int(T["stepMaxCycles"]), int(T["recordEvery"]))
        phi = np.array([S.get(b)[0] for b in range(len(steps))]).T
    finally:
        S.close()
    rec = int(T["recordEvery"])
    t = T["dt"] * rec * np.arange(1, n.shape[0] + 1)
    return {"n_over_t": np.transpose(n, (2, 0, 1)), "j_over_t": np.transpose(j, (2, 0, 1)), "t": t, "phi": phi,
            "status": st, "info": info, "stationary": ginfo}



def solve_transport_DG_2D_transient_SC_new(mat, INIT, options=None, transient=None):
    """DG = solve_transport_DG_2D_transient_SC_new(mat, INIT) (DG_code/solve_transport_DG_2D_transient_SC_new.m:1-221)
    for the 1D RTD (one valley, one mode), from a caller-supplied INIT.

    INIT (:18-25): ``rho`` (the initial Wigner function, a vector in the solver's order or a
    one-entry list of it, INIT.rho{1}), ``rhs`` (INIT.rhs{1}, used as given and never refreshed,
    :153-156), ``V_total`` (the potential added to the band edge, mat.V + V_total at :132;
    here phi = -V_total on the material grid), optional ``bias`` (the drain bias the INIT state
    was computed at, default 0) and ``Ef0`` (unused: the contact Fermi levels follow from the band
    edge and the bias as in the stationary driver); ``Esub``, ``Vsub``, ``A`` and ``p`` are rebuilt
    on the device from the potential.  mat: the RTD description of solve_rtd_self_consistent plus
    ``Nt`` (steps), ``dt`` (s) and ``Vd`` (the drain bias after the step at t = 0).

    The loop follows the reference: d rho/dt = rhs_INIT - 2e-10 A rho with RK4 (:153-158) by
    default (``transient={"method": "cn"}`` for Crank-Nicolson), the operator rebuilt before step t
    when (t-1) % 20 == 0 or t < 50 (:131-149), the Poisson problem solved for the density after
    step t when t % 20 == 0 or t < 50 (:204-211).  Returns n_over_t [Nxdof x Ny x ceil(Nt/50)]
    (steps 1, 51, ...: n_over_t(:,:,1:50:end)), j_over_t [Nxdof x ceil(Nt/5)] (j_over_t(:,1:5:end)),
    rho_INIT (the final state, a one-entry list as the reference's cell), chi, xi, the final phi
    and the per-step solver info.
    """
    nm = int(mat.get("n_of_modes", 1)) * int(mat.get("n_of_valleys", 1))
    if nm != 1:
        raise WignerError(_lib.WG_ERR_ARG, "the 1D RTD transient mirrors one valley and one mode")
    T = dict(TRANSIENT_DEFAULTS, method="rk4", scaleRhs=1.0, recordEvery=1, stepTolerance=1e-10)
    for k, v in (transient or {}).items():
        if k not in T:
            raise WignerError(_lib.WG_ERR_ARG, "unknown transient option %s" % k)
        T[k] = v
    nt = int(mat["Nt"])
    dt = float(mat["dt"])
    rho0 = INIT["rho"]
    rho0 = rho0[0] if isinstance(rho0, (list, tuple)) else rho0
    rhs0 = INIT["rhs"]
    rhs0 = rhs0[0] if isinstance(rhs0, (list, tuple)) else rhs0
    phi0 = -np.asarray(INIT["V_total"], dtype=float).reshape(-1)
    S = RTDSweep(mat, 1, options)
    try:
        if phi0.size != S.nx:
            raise WignerError(_lib.WG_ERR_ARG, "INIT.V_total needs %d values on the material grid" % S.nx)
        S.set(0, float(INIT.get("bias", 0.0)), phi0=phi0)
        S.P.set_rho(0, rho0)
        S.P.set_rhs(0, rhs0)
        S.step_bias(0, float(mat.get("Vd", INIT.get("bias", 0.0))))
        st, info, n, j = S.transient(dt, nt, T["method"], T["scaleA"], T["scaleRhs"], int(T["refreshEvery"]),
                                     int(T["refreshFirst"]), T["stepTolerance"], int(T["stepMaxCycles"]), 1,
                                     fixed_rhs=True)
        rho_end = S.P.rho(0)
        phi = S.get(0)[0]
        shp = shape_from_mat(mat)
    finally:
        S.close()
    n_el, nK = shp["n_el"], shp["n_local"]
    dx = (float(mat["x"][-1]) - float(mat["x"][0])) * 1e-9 / n_el
    chi = np.concatenate([np.linspace(e * dx, (e + 1) * dx, nK) for e in range(n_el)])
    lxi = shp["l_xi"]
    dxi = lxi / (shp["n_xi"] - 1)
    xi = np.linspace(-(lxi - dxi) / 2, (lxi - dxi) / 2, shp["n_xi"])
    n_all = n[:, 0, :].T                                   # [Nxdof x Nt]
    j_all = j[:, 0, :].T
    return {"n_over_t": n_all[:, None, 0::50], "j_over_t": j_all[:, 0::5], "rho_INIT": [rho_end], "chi": chi,
            "xi": xi, "phi": phi, "status": st, "info": info[0], "n_all": n_all, "j_all": j_all}
