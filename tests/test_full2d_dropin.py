"""The Full-2D drop-in solve_transport_DG_full2D(mat, Vxy, EfL, EfR, rho0).

CPU: the argument and option checks of solveStationarySystem that come before any device work
(validateInitialRho, the GPU direct-solver error, rho0 with BiCGSTAB, the GMRES basis-memory
guard, unknown and host-only preconditioners, full2D_solve = off).

GPU: the solve of a reservoir-driven system through the drop-in (GMRES and BiCGSTAB, with the
line-transverse preconditioner) against the oracle's sparse LU of the same assembled system:
rho to 1e-8 relative, density and currents (oracle get_Observables_full2D on the LU solution)
to 1e-8; the solve info fields (flag, status, trueRelres <= tol, resvec from |b - A x0| down to
the tolerance); the warm start rho0 = DG.rho converges at the start with no iteration.
"""
import numpy as np
import pytest

from oracle import full2d as F2
from test_reservoir import small_mat

TOL = 1e-10


def _mat(**extra):
    mat = small_mat("contact-modes", "periodic")
    XX, YY = np.meshgrid(mat["x"], mat["y"], indexing="ij")
    mat["V"] = 1.424 + 0.15 * np.exp(-((XX - 10) / 3) ** 2) - 0.05 * XX / 20
    mat["dg"]["params"].update(full2D_solverTol=TOL, full2D_solverMaxIt=300, full2D_gmresRestart=20, **extra)
    return mat


def _raises(identifier, **extra):
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.full2d import solve_transport_DG_full2D
    mat = _mat(**extra)
    rho0 = extra.pop("_rho0", None)
    with pytest.raises(WignerError) as e:
        solve_transport_DG_full2D(mat, None, 1.45, 1.40, rho0)
    assert e.value.identifier == identifier, str(e.value)


def test_dropin_rejects_bad_initial_rho():
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.full2d import solve_transport_DG_full2D
    mat = _mat()
    for bad in (np.zeros(7), np.full(F2.init_params_full2d(mat)["nTotal"], np.nan)):
        with pytest.raises(WignerError) as e:
            solve_transport_DG_full2D(mat, None, 1.45, 1.40, bad)
        assert e.value.identifier == "DG:Full2D:InvalidInitialRho"


def test_dropin_option_errors_before_device_work():
    n = F2.init_params_full2d(_mat())["nTotal"]
    _raises("DG:Full2D:GPUDirectSolverUnsupported", full2D_solver="direct")
    _raises("DG:Full2D:UnknownSolver", full2D_solver="cgs")
    _raises("DG:Full2D:GmresMemoryLimit", full2D_gmresMaxBasisBytes=1000.0)
    _raises("DG:Full2D:UnsupportedPreconditioner", full2D_preconditioner="blockjacobi")
    _raises("DG:Full2D:UnknownPreconditioner", full2D_preconditioner="ilu0")
    _raises("DG:Full2D:UnknownSolveMode", full2D_solve="sometimes")
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.full2d import solve_transport_DG_full2D
    mat = _mat(full2D_solver="bicgstab")
    with pytest.raises(WignerError) as e:
        solve_transport_DG_full2D(mat, None, 1.45, 1.40, np.zeros(n, dtype=complex))
    assert e.value.identifier == "DG:Full2D:InitialRhoSolver"


@pytest.mark.gpu
def test_dropin_solve_disabled_returns_the_operator_status(built_lib):
    from real_space_dg_gb300.full2d import solve_transport_DG_full2D
    DG = solve_transport_DG_full2D(_mat(full2D_solve="off"), None, 1.45, 1.40)
    assert DG["status"] == "operator-ready-solve-disabled" and DG["rho"] is None and DG["n"] is None


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["gmres", "bicgstab"])
def test_dropin_matches_sparse_lu(built_lib, solver):
    import scipy.sparse.linalg as spla
    from real_space_dg_gb300.full2d import Full2DOperator, solve_transport_DG_full2D
    mat = _mat(full2D_solver=solver)
    V = mat["V"]
    p, parts, dd = F2.system(mat, V)
    A = (F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"]) + F2.assemble_drift(p, dd)).tocsc()
    with Full2DOperator(mat, V) as op:
        rhs, _ = op.reservoir_rhs(1.45, 1.40)
    want = spla.spsolve(A, rhs)
    DG = solve_transport_DG_full2D(mat, V, 1.45, 1.40)
    s = DG["info"]["solve"]
    assert DG["status"] == "solved-" + solver and s["flag"] == 0, s
    assert s["trueRelres"] <= TOL and s["relres"] == s["trueRelres"]
    rv = s["resvec"]
    assert rv.size >= 3 and abs(rv[0] - np.linalg.norm(rhs)) <= 1e-12 * rv[0] and rv[-1] <= TOL * rv[0]
    assert np.linalg.norm(DG["rho"] - want) <= 1e-8 * np.linalg.norm(want)
    n_ref, j_ref, nDG_ref, jx_ref = F2.observables(p, mat, want)
    jy_ref, _ = F2.observables_y(p, mat, want)
    assert np.linalg.norm(DG["n"] - n_ref) <= 1e-8 * np.linalg.norm(n_ref)
    assert np.linalg.norm(DG["j"] - j_ref) <= 1e-8 * np.linalg.norm(j_ref)
    # the periodic RTD carries no net y current: jy is round-off of the x-current scale on both sides
    assert np.linalg.norm(DG["jy"] - jy_ref) <= 1e-8 * np.linalg.norm(jx_ref)
    assert DG["RHO"].shape == DG["arraySize"]
    assert np.array_equal(DG["RHO"].reshape(-1, order="F"), DG["rho"])
    if solver == "gmres":
        warm = solve_transport_DG_full2D(mat, V, 1.45, 1.40, DG["rho"])
        w = warm["info"]["solve"]
        assert w["initialGuess"]["provided"] and w["initialGuess"]["convergedAtStart"]
        assert w["iterations"] == [0, 0] and w["flag"] == 0
        assert np.array_equal(warm["rho"], DG["rho"])


@pytest.mark.gpu
def test_dropin_hard_wall_matches_sparse_lu(built_lib):
    """full2D_Y_boundary = 'hard-wall' through the drop-in (material-default reservoirs): the face data
    only on the active samples, the constrained system T A P + scale (I - P) with rhs T b
    (constrain_HardWall_full2D.m), solved by GMRES with the constrained line-transverse
    preconditioner; against the sparse LU of the oracle's constrained matrix, 1e-8; the solution
    vanishes on the constrained samples."""
    import scipy.sparse.linalg as spla
    from real_space_dg_gb300.full2d import Full2DOperator, solve_transport_DG_full2D
    mat = small_mat("material-default", "hard-wall", nry=8)
    XX, YY = np.meshgrid(mat["x"], mat["y"], indexing="ij")
    mat["V"] = 1.424 + 0.15 * np.exp(-((XX - 10) / 3) ** 2) - 0.05 * XX / 20
    mat["dg"]["params"].update(L_rho_y=8e-9, full2D_solverTol=TOL, full2D_solverMaxIt=300, full2D_gmresRestart=20)
    V = mat["V"]
    p, parts, dd = F2.system(mat, V)
    wall = F2.hard_wall_geometry(p, F2.transport_scales(mat))
    A = F2.constrain_hard_wall(p, wall, (F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"])
                                         + F2.assemble_drift(p, dd)).tocsr()).tocsc()
    with Full2DOperator(mat, V) as op:
        rhs, inflow = op.reservoir_rhs(1.45, 1.40)
    act = F2.wall_active_mask(p, wall)
    assert np.abs(rhs[act == 0]).max() == 0 and inflow["source"][1]["hardWallSupportApplied"]
    want = spla.spsolve(A, rhs)
    DG = solve_transport_DG_full2D(mat, V, 1.45, 1.40)
    s = DG["info"]["solve"]
    assert DG["status"] == "solved-gmres" and s["flag"] == 0 and s["trueRelres"] <= TOL, s
    assert np.linalg.norm(DG["rho"] - want) <= 1e-8 * np.linalg.norm(want)
    assert np.abs(DG["rho"][act == 0]).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
def test_dropin_contact_masks_match_sparse_lu(built_lib):
    """Source and drain contacts on part of the outer X faces (full2D_<side>ContactMask): the reservoir
    data only on the contact pieces, the closed pieces reflecting rho_x (get_Diff_full2D.m:393-423,
    get_InflowBoundary_full2D.m:23-24); the drop-in's GMRES solve against the sparse LU of the
    oracle's operator with those parts, 1e-8."""
    import scipy.sparse.linalg as spla
    from real_space_dg_gb300.full2d import Full2DOperator, solve_transport_DG_full2D
    mat = small_mat("material-default", "zero-inflow")
    y = np.asarray(mat["y"], dtype=float)
    XX, YY = np.meshgrid(mat["x"], y, indexing="ij")
    mat["V"] = 1.424 + 0.15 * np.exp(-((XX - 10) / 3) ** 2) - 0.05 * XX / 20
    mat["dg"]["params"].update(full2D_solverTol=TOL, full2D_solverMaxIt=300, full2D_gmresRestart=20,
                               full2D_sourceContactMask=(y > 0.5) & (y < 3.5), full2D_drainContactMask=y < 2.5)
    V = mat["V"]
    p, parts, dd = F2.system(mat, V)
    assert sum("closed-face" in q[0] for q in parts) == 2
    A = (F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"]) + F2.assemble_drift(p, dd)).tocsc()
    with Full2DOperator(mat, V) as op:
        rhs, inflow = op.reservoir_rhs(1.45, 1.40)
        u = np.sin(np.arange(p["nTotal"])) + 1j * np.cos(0.3 * np.arange(p["nTotal"]))
        assert np.linalg.norm(op.apply(u) - A @ u) <= 1e-12 * np.linalg.norm(A @ u)
    for side in ("source", "drain"):
        rho_b, info = inflow[side]
        closed = ~F2.contact_mask(mat, p, side)
        assert np.abs(rho_b[:, closed]).max() == 0 and np.abs(rho_b[:, ~closed]).max() > 0
    want = spla.spsolve(A, rhs)
    DG = solve_transport_DG_full2D(mat, V, 1.45, 1.40)
    s = DG["info"]["solve"]
    assert DG["status"] == "solved-gmres" and s["flag"] == 0 and s["trueRelres"] <= TOL, s
    assert np.linalg.norm(DG["rho"] - want) <= 1e-8 * np.linalg.norm(want)


@pytest.mark.gpu
def test_dropin_box_contact_modes_match_sparse_lu(built_lib):
    """Contact-mode reservoirs on a non-periodic Y face (the box contact problem) through the drop-in:
    the reservoir right-hand side from the host's box modes, GMRES on the device, against the sparse
    LU of the oracle's operator; the face data are those of the oracle's restatement."""
    import scipy.sparse.linalg as spla
    from oracle import reservoir as R
    from real_space_dg_gb300.full2d import Full2DOperator, solve_transport_DG_full2D
    mat = small_mat("contact-modes", "zero-inflow", nry=8)
    XX, YY = np.meshgrid(mat["x"], mat["y"], indexing="ij")
    mat["V"] = 1.424 + 0.15 * np.exp(-((XX - 10) / 3) ** 2) - 0.05 * XX / 20
    mat["dg"]["params"].update(L_rho_y=6e-9, full2D_contactModeCount=3, full2D_solverTol=TOL,
                               full2D_solverMaxIt=300, full2D_gmresRestart=20)
    V = mat["V"]
    p, parts, dd = F2.system(mat, V)
    A = (F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"]) + F2.assemble_drift(p, dd)).tocsc()
    with Full2DOperator(mat, V) as op:
        rhs, inflow = op.reservoir_rhs(1.45, 1.40)
    for side, ef in (("source", 1.45), ("drain", 1.40)):
        want_b, _ = R.contact_mode_reservoir(mat, p, side, ef, V)
        assert np.abs(inflow[side][0] - want_b).max() <= 1e-12 * np.abs(want_b).max()
    want = spla.spsolve(A, rhs)
    DG = solve_transport_DG_full2D(mat, V, 1.45, 1.40)
    s = DG["info"]["solve"]
    assert DG["status"] == "solved-gmres" and s["flag"] == 0 and s["trueRelres"] <= TOL, s
    assert np.linalg.norm(DG["rho"] - want) <= 1e-8 * np.linalg.norm(want)
