"""Full-2D self-consistent bias sweep: ``results = solve2D_rtd_self_consistent('DG', mat, options)``.

Host driver of RTD/solve2D_rtd_self_consistent.m:1-222 around the device pieces:

  transport   Full2DOperator: potential V = Vc - phi set on the device, the contact-mode /
              material-default reservoir right-hand side, flexible GMRES with the line-transverse
              preconditioner (mixed or FP64), warm-started from the previous iterate
  observables Full2DOperator.observables: n on the material grid and nDG at zero separation
  Poisson     poisson2d.make_RTD_poisson_step: projection of nDG and the direct or approximate-
              Newton update, one device call

with the reference's fixed-point logic: phi starts from bias x ramp (or the previous bias point
shifted by the bias step), the unmixed potential defect, the relative density change and the
Poisson residual at the current potential decide convergence, and phi <- phi + mixing
(candidate - phi).  Dirichlet contacts (phi(source) = 0, phi(drain) = bias); the Neumann-contact
variant (prepare_RTD_neumann_contacts.m) is not built.
"""
import time

import numpy as np

from . import _lib
from ._lib import WignerError
from .full2d import Full2DOperator
from .poisson2d import make_RTD_poisson_step

# innerRestart: restart length of the mixed form's FP32 inner FGMRES (each inner cycle ends with an FP64
# residual refinement); None takes mat.dg.params.full2D_gmresRestart (the reference's GMRES(40)).  20 is
# faster on the recorded 3.1M-unknown system (3.42 s vs 3.80 s per solve to 5e-6: 7% more iterations, each
# with less Gram-Schmidt work) and lands on different, equally converged transport states.
DEFAULTS = dict(maxIterations=100, mixing=0.1, potentialTolerance=5e-4, densityTolerance=5e-4,
                poissonResidualTolerance=8e-2, chargeNeutralityTolerance=1e-3, poissonMethod="",
                initialPhi=None, initialRho=None, mixed=True, innerRestart=None)


def _options(options):
    o = dict(DEFAULTS)
    for k, v in (options or {}).items():
        if k not in o:
            raise WignerError(_lib.WG_ERR_ARG, "RTD:UnknownSelfConsistencyOption: %s" % k)
        o[k] = v
    if not (0 < o["mixing"] <= 1):
        raise WignerError(_lib.WG_ERR_ARG, "mixing must be in (0, 1]")
    return o


def _check_phi(phi, mat, bias, periodic):
    tol = 1e-10 * max(1.0, abs(bias))
    if not np.all(np.isfinite(phi)) or phi.shape != (int(mat["Nx"]), int(mat["Ny"])):
        raise WignerError(_lib.WG_ERR_ARG, "RTD:InvalidPoissonPotential")
    if np.abs(phi[0]).max() > tol or np.abs(phi[-1] - bias).max() > tol:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonContactPotential: phi(source) = 0, phi(drain) = bias")
    if periodic and np.abs(phi[:, 0] - phi[:, -1]).max() > tol:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:NonperiodicPoissonPotential")


def solve2D_rtd_self_consistent(solver, mat, options=None, callback=None):
    """The self-consistent sweep over mat['Vdd'] (solve2D_rtd_self_consistent.m).  Returns a dict
    with the reference's sweep fields (bias, current [X nDof x nb], density [X nDof x Ny x nb],
    potential V and phi [Nx x Ny x nb], flag, relres, converged, iterations, status) and the
    per-bias histories (gmresIterations, potentialDefect, densityChange, poissonPhysicalRelres) and the
    wall time per phase (timing: potential, reservoir, transport, observables, poisson seconds).
    ``callback(bias_index, iteration, history_entry)`` is called after every Poisson step."""
    if str(solver).upper() != "DG":
        raise WignerError(_lib.WG_ERR_ARG, "RTD:UnsupportedSolver: the self-consistency loop uses the Full-2D DG solver")
    o = _options(options)
    prm = mat["dg"]["params"]
    if str(prm.get("full2D_solver", "gmres")).lower() != "gmres":
        raise WignerError(_lib.WG_ERR_ARG, "RTD:SelfConsistencyNeedsGmres")
    if str(mat.get("poisson", {}).get("xBoundary", "dirichlet")).lower() == "neumann":
        raise WignerError(_lib.WG_ERR_ARG, "Neumann RTD contacts (prepare_RTD_neumann_contacts) are not built")
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    Vc = np.asarray(mat["Vc"], dtype=float).reshape(nx, ny)
    bias = np.atleast_1d(np.asarray(mat["Vdd"], dtype=float))
    x = np.asarray(mat["x"], dtype=float)
    ramp_len = x[-1] - float(mat["Lc1"]) - float(mat["Lc2"])
    if ramp_len <= 0:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:ContactGeometry")
    ramp = np.repeat(np.clip((x - float(mat["Lc1"])) / ramp_len, 0.0, 1.0)[:, None], ny, axis=1)
    periodic = str(prm.get("full2D_Y_boundary", "")).lower() == "periodic"
    method = o["poissonMethod"] or mat.get("poisson", {}).get("opt", {}).get("solve", "direct")
    step, setup = make_RTD_poisson_step(mat, method)
    tol = float(prm.get("full2D_solverTol", 1e-6))
    restart = int(prm.get("full2D_gmresRestart", 40))
    maxit = int(prm.get("full2D_solverMaxIt", 150))
    op = Full2DOperator(mat, Vc)
    op.set_preconditioner()
    p_axes = {"X": op.factors["axes"][0], "Y": op.factors["axes"][1], "coordinateScale": op.factors["scale"]}
    nb = bias.size
    sweep = dict(bias=np.full(nb, np.nan), current=None, density=None, potential=np.zeros((nx, ny, nb)),
                 phi=np.zeros((nx, ny, nb)), flag=np.full(nb, -1), relres=np.full(nb, np.nan),
                 converged=np.zeros(nb, dtype=bool), iterations=np.zeros(nb, dtype=int), status=[])
    histories = []
    timing = dict(potential_s=0.0, reservoir_s=0.0, transport_s=0.0, observables_s=0.0, poisson_s=0.0)
    clock = time.perf_counter
    rho = o["initialRho"]            # host warm start of the first solve; afterwards the state stays on the device
    resident = False
    rhs_key = None                   # the reservoir right-hand side depends on the contact-edge potentials only
    prev_phi = None
    try:
        for ib in range(nb):
            if ib == 0:
                phi = bias[0] * ramp if o["initialPhi"] is None else np.asarray(o["initialPhi"], dtype=float)
            else:
                phi = prev_phi + (bias[ib] - bias[ib - 1]) * ramp
            _check_phi(phi, mat, bias[ib], periodic)
            prev_n = None
            history = []
            status, converged = "iteration-limit", False
            for it in range(1, int(o["maxIterations"]) + 1):
                V = Vc - phi
                efl = float(mat["EfL"]) if "EfL" in mat else Vc[0, 0] + 0.05
                efr = (float(mat["EfR"]) if "EfR" in mat else Vc[-1, 0] + 0.05) - bias[ib]
                t0 = clock()
                op.set_potential(V)
                t1 = clock()
                key = (efl, efr, V[0].tobytes(), V[-1].tobytes())
                rhs = None
                if key != rhs_key:
                    rhs, _ = op.reservoir_rhs(efl, efr, V)
                    rhs_key = key
                t2 = clock()
                mixed = bool(o["mixed"])
                m_in = int(o["innerRestart"] or restart) if mixed else restart
                st, info, _ = op.solve(rhs, x0=None if resident else rho, warm=resident, resident=True, tol=tol,
                                       maxit=maxit if not mixed else maxit * max(1, restart * 4 // m_in),
                                       restart=m_in, mixed=mixed)
                resident = True
                t3 = clock()
                timing["potential_s"] += t1 - t0
                timing["reservoir_s"] += t2 - t1
                timing["transport_s"] += t3 - t2
                h = dict(iteration=it, transportFlag=int(st), transportRelres=info["relres"],
                         gmresIterations=info["iterations"], densityChange=np.inf, potentialDefect=np.inf,
                         poissonConverged=False, poissonPhysicalRelres=np.nan)
                if st != 0 or not np.isfinite(info["relres"]) or info["relres"] > tol:
                    history.append(h)
                    status = "transport-not-converged"
                    break
                t0 = clock()
                n, j, nDG, _ = op.observables()          # on the device, from the resident state
                timing["observables_s"] += clock() - t0
                if prev_n is not None:
                    h["densityChange"] = float(np.linalg.norm(n - prev_n) /
                                               max(np.linalg.norm(n), np.linalg.norm(prev_n), np.finfo(float).tiny))
                t0 = clock()
                cand, pinfo = step({"transport": {"nDG": nDG, "p": p_axes}, "phi": phi, "bias": bias[ib]})
                timing["poisson_s"] += clock() - t0
                _check_phi(cand, mat, bias[ib], periodic)
                h["poissonConverged"] = bool(pinfo["converged"])
                h["potentialDefect"] = float(np.abs(cand - phi).max())
                h["poissonPhysicalRelres"] = float(pinfo["physical_relres_before"])
                history.append(h)
                if callback is not None:
                    callback(ib, it, h)
                if not pinfo["converged"]:
                    status = "poisson-not-converged"
                    break
                if h["potentialDefect"] <= o["potentialTolerance"] and h["densityChange"] <= o["densityTolerance"] \
                        and h["poissonPhysicalRelres"] <= o["poissonResidualTolerance"]:
                    status, converged = "fixed-point-converged", True
                    break
                if it == int(o["maxIterations"]):
                    break
                prev_n = n
                phi = phi + o["mixing"] * (cand - phi)
            histories.append(history)
            if sweep["current"] is None:
                sweep["current"] = np.zeros((j.size, nb))
                sweep["density"] = np.zeros(n.shape + (nb,))
            sweep["bias"][ib] = bias[ib]
            sweep["current"][:, ib] = j
            sweep["density"][:, :, ib] = n
            sweep["potential"][:, :, ib] = V
            sweep["phi"][:, :, ib] = phi
            sweep["flag"][ib] = st
            sweep["relres"][ib] = info["relres"]
            sweep["converged"][ib] = converged
            sweep["iterations"][ib] = len(history)
            sweep["status"].append(status)
            if not converged:
                break
            prev_phi = phi
    finally:
        op.close()
        setup["operator"].close()
    return {"sweep": sweep, "histories": histories, "phi": phi, "status": "self-consistency-" + status,
            "timing": {k: round(v, 3) for k, v in timing.items()},
            "Id": np.nanmean(sweep["current"], axis=0) if sweep["current"] is not None else None,
            "converged": bool(np.all(sweep["converged"]))}
