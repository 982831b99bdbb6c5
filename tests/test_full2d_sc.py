"""Full-2D self-consistent loop (RTD/solve2D_rtd_self_consistent.m): option and contact checks on the
host, and on the GPU the first bias point of the reference's recorded run reproduced iteration by
iteration (potential defect, density change, Poisson residual) with its converged potential and
density."""
import numpy as np
import pytest

from test_reservoir import recorded


def recorded_sc_mat():
    g, mat = recorded()
    mat.update(Vc=g["Vc"], eps=g["eps"], Nd=g["Nd"], Lc1=float(g["Lc1"]), Lc2=float(g["Lc2"]), dx=float(g["dx"]),
               dy=float(g["dy"]), Vdd=np.array([0.0]), poisson=dict(opt=dict(solve="newton-raphson")))
    mat["dg"]["params"].update(full2D_solverTol=5e-6, full2D_gmresRestart=40, full2D_solverMaxIt=150)
    return g, mat


def test_options_and_contact_checks():
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.full2d_sc import _check_phi, _options, solve2D_rtd_self_consistent
    assert _options({"mixing": 0.3})["mixing"] == 0.3
    with pytest.raises(WignerError):
        _options({"mixingg": 0.3})
    with pytest.raises(WignerError):
        _options({"mixing": 0.0})
    _, mat = recorded_sc_mat()
    phi = np.zeros((mat["Nx"], mat["Ny"]))
    phi[-1] = 0.2
    _check_phi(phi, mat, 0.2, True)
    bad = phi.copy()
    bad[-1, 3] = 0.1
    with pytest.raises(WignerError):
        _check_phi(bad, mat, 0.2, True)                  # phi(drain) must equal the bias
    bad = phi.copy()
    bad[5, -1] = 0.01
    with pytest.raises(WignerError):
        _check_phi(bad, mat, 0.2, True)                  # periodic Y endpoints must agree
    with pytest.raises(WignerError):
        solve2D_rtd_self_consistent("QTBM", mat)
    flat = dict(mat, dg=dict(mat["dg"], params=dict(mat["dg"]["params"], full2D_Y_boundary="zero-inflow")))
    with pytest.raises(WignerError) as e:                # Neumann contacts need a periodic Y cell
        solve2D_rtd_self_consistent("DG", flat, {"poissonXBoundary": "neumann"})
    assert e.value.identifier == "RTD:PoissonBoundaryMismatch"
    _neumann = dict(mat, poisson=dict(mat["poisson"], xBoundary="neumann", yBoundary="neumann"))
    with pytest.raises(WignerError) as e:
        solve2D_rtd_self_consistent("DG", _neumann)
    assert e.value.identifier == "RTD:PoissonBoundaryMismatch"


def test_neumann_calibration_reproduces_the_recorded_contact_levels():
    """prepare_RTD_neumann_contacts.m on the recorded device: the sheet densities are the contact
    columns' net doping integrated over y, and the flat-band neutrality levels are the contact
    levels the recorded run used (its source level; its drain level plus the 0.6 V bias it was
    recorded at), so the built-in voltage of the symmetric device is zero; the returned mat fixes
    the levels ('external').  The doping helper's unit checks (get_RTD_doping_SI.m)."""
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.full2d_sc import prepare_RTD_neumann_contacts, rtd_doping_si
    g, mat = recorded_sc_mat()
    out, ref = prepare_RTD_neumann_contacts(mat)
    y = np.asarray(mat["y"], dtype=float) * 1e-9
    Nd = np.asarray(g["Nd"], dtype=float)
    want = float(np.sum(0.5 * (Nd[0, 1:] + Nd[0, :-1]) * np.diff(y)))
    assert ref["sourceSheetDensity"] == pytest.approx(want, rel=1e-14)
    assert abs(ref["sourceMuEV"] - float(g["ef_used_source"])) < 1e-12
    assert abs(ref["neutralDrainMuEV"] - (float(g["ef_used_drain"]) + 0.6)) < 1e-9
    assert abs(ref["builtInVoltage"]) < 1e-9
    assert out["dg"]["params"]["full2D_contactModeFermiModel"] == "external"
    assert out["reservoirReference"] is ref
    legacy = dict(mat, N_d=Nd / 1e6)
    legacy.pop("Nd")
    assert np.array_equal(rtd_doping_si(legacy)[0], Nd)
    with pytest.raises(WignerError) as e:
        rtd_doping_si(dict(mat, N_d=Nd / 1e6 * 1.01))
    assert e.value.identifier == "RTD:InconsistentDopingUnits"
    with pytest.raises(WignerError) as e:
        prepare_RTD_neumann_contacts(dict(mat, dg=dict(mat["dg"], params=dict(
            mat["dg"]["params"], full2D_reservoirModel="material-default"))))
    assert e.value.identifier == "RTD:NeumannContactModel"


@pytest.mark.gpu
def test_gpu_recorded_bias_point_reproduced(built_lib):
    from real_space_dg_gb300.full2d_sc import solve2D_rtd_self_consistent
    g, mat = recorded_sc_mat()
    hist = []
    res = solve2D_rtd_self_consistent("DG", mat, {"mixing": 0.3}, callback=lambda ib, it, h: hist.append(h))
    sw = res["sweep"]
    rec = g["history0"]
    assert res["converged"] and sw["iterations"][0] == int(g["iterations0"])
    assert abs(hist[0]["potentialDefect"] - rec[0, 1]) <= 1e-4 * rec[0, 1]
    for h, r in zip(hist, rec):
        assert abs(h["potentialDefect"] - r[1]) <= 1e-2 * r[1]
        assert abs(h["poissonPhysicalRelres"] - r[3]) <= 1e-2 * r[3]
    assert np.abs(sw["potential"][:, :, 0] - g["potential0"]).max() <= 1e-5
    assert np.abs(sw["density"][:, :, 0] - g["density0"]).max() <= 1e-3 * np.abs(g["density0"]).max()


@pytest.mark.gpu
def test_gpu_recorded_sweep_continuation(built_lib):
    """The first two bias points of the recorded sweep (0 and 0.02 V): the second starts from the
    first's potential shifted by the bias step and its state (solve2D_rtd_self_consistent.m:91-96,
    196-198) and needs the recorded 9 Gummel iterations; the mean currents follow the recorded I-V
    curve."""
    from real_space_dg_gb300.full2d_sc import solve2D_rtd_self_consistent
    g, mat = recorded_sc_mat()
    mat["Vdd"] = np.asarray(g["sweep_bias"])[:2]
    res = solve2D_rtd_self_consistent("DG", mat, {"mixing": 0.3})
    sw = res["sweep"]
    assert res["converged"]
    assert list(sw["iterations"]) == [int(v) for v in np.asarray(g["sweep_iterations"])[:2]]
    ids = np.mean(sw["current"], axis=0)
    scale = np.abs(np.asarray(g["sweep_id"])).max()
    assert np.abs(ids - np.asarray(g["sweep_id"])[:2]).max() <= 1e-3 * scale


@pytest.mark.gpu
def test_gpu_neumann_contacts_bias_point(built_lib):
    """The Neumann-contact loop at 0.1 V on the recorded device: mu_S at the calibrated neutral level
    and mu_D = mu_S - bias, the approximate-Newton Poisson step with floating contact potentials,
    converged with the global charge balance inside chargeNeutralityTolerance; the converged state
    satisfies the loop's own tests (potential defect, density change, Poisson residual)."""
    from real_space_dg_gb300.full2d_sc import solve2D_rtd_self_consistent
    g, mat = recorded_sc_mat()
    mat["Vdd"] = np.array([0.1])
    opts = {"mixing": 0.3, "poissonXBoundary": "neumann", "maxIterations": 60}
    res = solve2D_rtd_self_consistent("DG", mat, opts)
    sw, ref = res["sweep"], res["reservoirReference"]
    assert res["poissonXBoundary"] == "neumann" and abs(ref["sourceMuEV"] - float(g["ef_used_source"])) < 1e-12
    assert np.allclose(sw["reservoirMuEV"][:, 0], [ref["sourceMuEV"], ref["sourceMuEV"] - 0.1], rtol=0, atol=1e-15)
    h = res["histories"][0][-1]
    assert res["converged"] and sw["status"][0] == "fixed-point-converged", res["histories"][0][-3:]
    assert h["relativeChargeImbalance"] <= 1e-3 and h["potentialDefect"] <= 5e-4
    assert h["poissonPhysicalRelres"] <= 8e-2 and h["densityChange"] <= 5e-4
