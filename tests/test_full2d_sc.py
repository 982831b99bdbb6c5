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
    with pytest.raises(WignerError):
        solve2D_rtd_self_consistent("DG", dict(mat, poisson=dict(xBoundary="neumann")))


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
