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
(candidate - phi).  Dirichlet contacts (phi(source) = 0, phi(drain) = bias) or Neumann contacts
(options.poissonXBoundary / mat.poisson.xBoundary = 'neumann', periodic Y and contact-mode
reservoirs): the contact modes are calibrated once to charge neutrality at the flat bands
(prepare_RTD_neumann_contacts.m), mu_S is held at the source's neutral level and mu_D = mu_S - bias,
phi starts from (bias + built-in voltage) x ramp, the Poisson step is the approximate Newton one
and convergence also asks the global charge balance (chargeNeutralityTolerance).
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
                poissonXBoundary="", initialPhi=None, initialRho=None, mixed=True, innerRestart=None,
                innerBasisFP16=False)


def _options(options):
    o = dict(DEFAULTS)
    for k, v in (options or {}).items():
        if k not in o:
            raise WignerError(_lib.WG_ERR_ARG, "RTD:UnknownSelfConsistencyOption: %s" % k)
        o[k] = v
    if not (0 < o["mixing"] <= 1):
        raise WignerError(_lib.WG_ERR_ARG, "mixing must be in (0, 1]")
    return o


def _check_phi(phi, mat, bias, periodic, neumann=False):
    tol = 1e-10 * max(1.0, abs(bias))
    if not np.all(np.isfinite(phi)) or phi.shape != (int(mat["Nx"]), int(mat["Ny"])):
        raise WignerError(_lib.WG_ERR_ARG, "RTD:InvalidPoissonPotential")
    if not neumann and (np.abs(phi[0]).max() > tol or np.abs(phi[-1] - bias).max() > tol):
        raise WignerError(_lib.WG_ERR_ARG, "RTD:PoissonContactPotential: phi(source) = 0, phi(drain) = bias")
    if periodic and np.abs(phi[:, 0] - phi[:, -1]).max() > tol:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:NonperiodicPoissonPotential")


def rtd_doping_si(mat):
    """(Nd, Na) [Nx x Ny] in m^-3 (RTD/get_RTD_doping_SI.m): mat.Nd / mat.Na in SI, or the legacy
    N_d / N_a in cm^-3; both given must agree."""
    nx, ny = int(mat["Nx"]), int(mat["Ny"])

    def field(si, legacy, required):
        if si not in mat and legacy not in mat:
            if required:
                raise WignerError(_lib.WG_ERR_ARG, "Provide mat.Nd [m^-3] or mat.N_d [cm^-3].", "RTD:MissingDoping")
            return np.zeros((nx, ny))
        v = np.asarray(mat[si] if si in mat else np.asarray(mat[legacy], dtype=float) * 1e6, dtype=float)
        if v.shape != (nx, ny) or not np.all(np.isfinite(v)) or (v < 0).any():
            raise WignerError(_lib.WG_ERR_ARG, "mat.%s must be a finite nonnegative Nx x Ny array" % si,
                              "RTD:MissingDoping")
        if si in mat and legacy in mat and \
                np.abs(v - np.asarray(mat[legacy], dtype=float) * 1e6).max() > 1e-12 * max(1.0, v.max()):
            raise WignerError(_lib.WG_ERR_ARG, "mat.%s and mat.%s disagree after cm^-3 to m^-3 conversion."
                              % (si, legacy), "RTD:InconsistentDopingUnits")
        return v
    return field("Nd", "N_d", True), field("Na", "N_a", False)


def prepare_RTD_neumann_contacts(mat):
    """(mat, reference) (RTD/prepare_RTD_neumann_contacts.m): calibrate the contact modes of both
    contacts once to charge neutrality (sheet densities from the contact columns' net doping,
    flat bands V = Vc as the energy reference), then fix the Fermi levels ('external' model).
    reference: sourceMuEV, neutralDrainMuEV, builtInVoltage = mu_D - mu_S."""
    from . import full2d, reservoir
    prm = mat["dg"]["params"]
    model = str(prm.get("full2D_reservoirModel", "material-default")).strip().lower().replace("_", "-")
    if full2d._ytype(prm) != "periodic" or model not in ("contact-modes", "contact-mode", "modes"):
        raise WignerError(_lib.WG_ERR_ARG, "Neumann RTD requires periodic Y and contact-modes reservoirs.",
                          "RTD:NeumannContactModel")
    Nd, Na = rtd_doping_si(mat)
    dy = np.diff(np.asarray(mat["y"], dtype=float) * 1e-9)

    def sheet(v):                            # trapz(y, v) over the contact column
        return float(0.5 * np.sum((v[1:] + v[:-1]) * dy))
    cal = dict(prm, full2D_contactModeFermiModel="contact-neutrality", full2D_contactModeIntegrateKz=True,
               full2D_sourceContactSheetDensity=sheet(Nd[0] - Na[0]),
               full2D_drainContactSheetDensity=sheet(Nd[-1] - Na[-1]))
    mcal = dict(mat, dg=dict(mat["dg"], params=cal))
    f = full2d.build_factors(mcal)
    Vc = np.asarray(mat["Vc"], dtype=float).reshape(int(mat["Nx"]), int(mat["Ny"]))
    _, src = reservoir.contact_mode_reservoir(mcal, f, "source", None, Vc)
    _, drn = reservoir.contact_mode_reservoir(mcal, f, "drain", None, Vc)
    mu_s, mu_d = float(src["fermiLevelUsed"]), float(drn["fermiLevelUsed"])
    if not (np.isfinite(mu_s) and np.isfinite(mu_d)):
        raise WignerError(_lib.WG_ERR_ARG, "Both contact-mode neutrality calibrations must converge.",
                          "RTD:ReservoirCalibration")
    reference = dict(sourceMuEV=mu_s, neutralDrainMuEV=mu_d, builtInVoltage=mu_d - mu_s,
                     sourceSheetDensity=cal["full2D_sourceContactSheetDensity"],
                     drainSheetDensity=cal["full2D_drainContactSheetDensity"])
    out = dict(mcal, dg=dict(mcal["dg"], params=dict(cal, full2D_contactModeFermiModel="external")),
               reservoirReference=reference)
    return out, reference


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
    if o["poissonXBoundary"]:
        mat = dict(mat, poisson=dict(mat.get("poisson", {}), xBoundary=o["poissonXBoundary"]))
    xbc = str(mat.get("poisson", {}).get("xBoundary", "dirichlet")).strip().lower()
    if xbc not in ("dirichlet", "neumann"):
        raise WignerError(_lib.WG_ERR_ARG, "poisson.xBoundary must be 'dirichlet' or 'neumann'",
                          "RTD:PoissonXBoundary")
    neumann = xbc == "neumann"
    reference, builtin = None, 0.0
    if neumann:
        if str(prm.get("full2D_Y_boundary", "")).lower() != "periodic":
            raise WignerError(_lib.WG_ERR_ARG, "Neumann RTD contacts require periodic Y.",
                              "RTD:PoissonBoundaryMismatch")
        if str(mat.get("poisson", {}).get("yBoundary", "periodic")).lower() != "periodic":
            raise WignerError(_lib.WG_ERR_ARG, "Neumann RTD contacts require periodic Poisson Y.",
                              "RTD:PoissonBoundaryMismatch")
        mat = dict(mat, poisson=dict(mat.get("poisson", {}), yBoundary="periodic"))
        mat, reference = prepare_RTD_neumann_contacts(mat)
        builtin = reference["builtInVoltage"]
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    Vc = np.asarray(mat["Vc"], dtype=float).reshape(nx, ny)
    bias = np.atleast_1d(np.asarray(mat["Vdd"], dtype=float))
    x = np.asarray(mat["x"], dtype=float)
    ramp_len = x[-1] - float(mat["Lc1"]) - float(mat["Lc2"])
    if ramp_len <= 0:
        raise WignerError(_lib.WG_ERR_ARG, "RTD:ContactGeometry")
    ramp = np.repeat(np.clip((x - float(mat["Lc1"])) / ramp_len, 0.0, 1.0)[:, None], ny, axis=1)
    periodic = str(prm.get("full2D_Y_boundary", "")).lower() == "periodic"
    method = o["poissonMethod"] or mat.get("poisson", {}).get("opt", {}).get(
        "solve", "newton-raphson" if neumann else "direct")
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
                phi = (bias[0] + builtin) * ramp if o["initialPhi"] is None else \
                    np.asarray(o["initialPhi"], dtype=float)
            else:
                phi = prev_phi + (bias[ib] - bias[ib - 1]) * ramp
            _check_phi(phi, mat, bias[ib], periodic, neumann)
            prev_n = None
            history = []
            status, converged = "iteration-limit", False
            for it in range(1, int(o["maxIterations"]) + 1):
                V = Vc - phi
                efl = float(mat["EfL"]) if "EfL" in mat else Vc[0, 0] + 0.05
                efr = (float(mat["EfR"]) if "EfR" in mat else Vc[-1, 0] + 0.05) - bias[ib]
                if neumann:                   # the calibrated source level, mu_S - mu_D = bias
                    efl = reference["sourceMuEV"]
                    efr = efl - bias[ib]
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
                                       restart=m_in, mixed=mixed, inner_basis_fp16=bool(o["innerBasisFP16"]))
                resident = True
                t3 = clock()
                timing["potential_s"] += t1 - t0
                timing["reservoir_s"] += t2 - t1
                timing["transport_s"] += t3 - t2
                h = dict(iteration=it, transportFlag=int(st), transportRelres=info["relres"],
                         gmresIterations=info["iterations"], densityChange=np.inf, potentialDefect=np.inf,
                         poissonConverged=False, poissonPhysicalRelres=np.nan, relativeChargeImbalance=np.nan)
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
                _check_phi(cand, mat, bias[ib], periodic, neumann)
                h["poissonConverged"] = bool(pinfo["converged"])
                h["potentialDefect"] = float(np.abs(cand - phi).max())
                h["poissonPhysicalRelres"] = float(pinfo["physical_relres_before"])
                balance_ok = True
                if neumann:
                    h["relativeChargeImbalance"] = float(pinfo["relative_charge_imbalance"])
                    balance_ok = bool(np.isfinite(h["relativeChargeImbalance"])
                                      and h["relativeChargeImbalance"] <= o["chargeNeutralityTolerance"])
                history.append(h)
                if callback is not None:
                    callback(ib, it, h)
                if not pinfo["converged"]:
                    status = "poisson-not-converged"
                    break
                if h["potentialDefect"] <= o["potentialTolerance"] and h["densityChange"] <= o["densityTolerance"] \
                        and h["poissonPhysicalRelres"] <= o["poissonResidualTolerance"] and balance_ok:
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
    if neumann:
        sweep["reservoirMuEV"] = np.vstack([np.full(nb, reference["sourceMuEV"]),
                                            reference["sourceMuEV"] - bias])
    return {"sweep": sweep, "histories": histories, "phi": phi, "status": "self-consistency-" + status,
            "poissonXBoundary": xbc, "reservoirReference": reference,
            "timing": {k: round(v, 3) for k, v in timing.items()},
            "Id": np.nanmean(sweep["current"], axis=0) if sweep["current"] is not None else None,
            "converged": bool(np.all(sweep["converged"]))}
