"""Full-2D contact reservoirs (get_ContactModeReservoirRho_full2D.m, get_DefaultReservoirRho_full2D.m)
and the inflow right-hand side (get_Diff_full2D.m:405-430): the oracle and the host module pinned
to the reservoir data of the reference's recorded run, and the device solve of the resulting
system against the oracle's sparse LU."""
import os

import numpy as np
import pytest

from oracle import full2d as F2
from oracle import reservoir as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "full2d_reservoir_golden.npz")


def recorded():
    g = np.load(GOLDEN)
    prm = {k[4:]: float(g[k]) for k in g.files if k.startswith("prm_")}
    for k in ("N_K_X", "N_K_Y", "N_el_X", "N_el_Y", "N_rho_x", "N_rho_y", "full2D_contactMode_Nkx",
              "full2D_contactMode_Nkz"):
        prm[k] = int(prm[k])
    prm.update(full2D_Y_boundary="periodic", full2D_reservoirModel="contact-modes", full2D_X_flux="upwind",
               full2D_Y_flux="upwind", full2D_contactModeFermiModel="contact-neutrality",
               full2D_potentialQuadratureOrder=5)
    mat = dict(x=g["x"], y=g["y"], Nx=int(g["Nx"]), Ny=int(g["Ny"]), me_x_ch=float(g["me_x_ch"]),
               me_y_ch=float(g["me_y_ch"]), me_z_ch=float(g["me_z_ch"]), deg_factor=float(g["deg_factor"]),
               Temp=float(g["Temp"]), dg=dict(params=prm))
    return g, mat


@pytest.mark.parametrize("side", ["source", "drain"])
def test_oracle_matches_the_recorded_contact_mode_reservoir(side):
    g, mat = recorded()
    p = F2.init_params_full2d(mat)
    rho, info = R.contact_mode_reservoir(mat, p, side, float(g["ef_input_" + side]), g["potential"])
    assert np.array_equal(info["modeEnergy"], g["modes_" + side])
    assert abs(info["fermiLevelUsed"] - float(g["ef_used_" + side])) < 1e-14
    gold = g["rho_" + side]
    assert np.abs(rho.imag).max() == 0.0
    assert np.abs(rho.real - gold).max() <= 1e-14 * np.abs(gold).max()


@pytest.mark.parametrize("side", ["source", "drain"])
def test_host_reservoir_matches_the_recorded_run(side):
    from real_space_dg_gb300 import full2d as H, reservoir as PR
    g, mat = recorded()
    f = H.build_factors(mat)
    inflow = PR.get_InflowBoundary_full2D(mat, f, float(g["ef_input_source"]), float(g["ef_input_drain"]),
                                          g["potential"])
    rho, info = inflow[side]
    gold = g["rho_" + side]
    assert abs(info["fermiLevelUsed"] - float(g["ef_used_" + side])) < 1e-14
    assert np.abs(rho - gold).max() <= 1e-14 * np.abs(gold).max()


def test_host_inflow_rhs_matches_oracle():
    from real_space_dg_gb300 import full2d as H, reservoir as PR
    g, mat = recorded()
    p = F2.init_params_full2d(mat)
    ox = F2.one_dimensional_dg_operators(p["X"])
    Apx, Amx, _ = F2.split_characteristic(p["Ax1D"])
    sx, _ = F2.transport_scales(mat)
    want = R.inflow_rhs(p, g["rho_source"], g["rho_drain"], sx, Apx, Amx, ox["leftLift"], ox["rightLift"])
    f = H.build_factors(mat)
    got = PR.inflow_rhs(f, {"source": (g["rho_source"], {}), "drain": (g["rho_drain"], {})})
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    # only the first and last X element of every Y node row carries inflow
    nrel = p["rhoX"]["nCells"] * p["rhoY"]["nCells"]
    touched = np.flatnonzero(np.abs(want).reshape(-1, nrel).max(axis=1)) % p["X"]["nDof"]
    assert set(touched) <= set(range(3)) | set(range(p["X"]["nDof"] - 3, p["X"]["nDof"]))


def small_mat(model, ybc, nrx=9, nry=4):
    prm = dict(N_K_X=3, N_K_Y=3, N_el_X=5, N_el_Y=2, N_rho_x=nrx, N_rho_y=nry, L_rho_x=8e-9,
               full2D_X_flux="upwind", full2D_Y_flux="upwind", full2D_Y_boundary=ybc,
               full2D_potentialQuadratureOrder=5, full2D_reservoirModel=model,
               full2D_sourceContactSheetDensity=6e15, full2D_drainContactSheetDensity=6e15,
               full2D_contactMode_Nkx=20, full2D_contactMode_Nkz=31, full2D_contactModeIntegrateKz=1)
    x, y = np.linspace(0, 20.0, 11), np.linspace(0, 4.0, 5)
    return dict(x=x, y=y, Nx=11, Ny=5, me_x_ch=0.063, me_y_ch=0.063, me_z_ch=0.063, Temp=300.0, deg_factor=1,
                dg=dict(params=prm))


def test_host_default_reservoir_matches_oracle():
    from real_space_dg_gb300 import full2d as H, reservoir as PR
    mat = small_mat("material-default", "zero-inflow")
    V = 1.424 + 0.1 * np.outer(np.linspace(0, 1, 11), np.ones(5)) + 0.02 * np.random.default_rng(0).normal(size=(11, 5))
    p = F2.init_params_full2d(mat)
    f = H.build_factors(mat)
    for side, ef in (("source", 1.45), ("drain", 1.40)):
        want = R.default_reservoir(mat, p, side, ef, V)
        got, _ = PR.default_reservoir(mat, f, side, ef, V)
        assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_host_reservoir_errors():
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300 import full2d as H, reservoir as PR
    mat = small_mat("contact-modes", "periodic")
    f = H.build_factors(mat)
    V = np.full((11, 5), 1.424)
    V[0, 2] = 1.5                              # a Y-dependent contact potential: modes by diagonalisation
    rho, info = PR.contact_mode_reservoir(mat, f, "source", 1.45, V)
    p = F2.init_params_full2d(mat)
    want, winfo = R.contact_mode_reservoir(mat, p, "source", 1.45, V)
    assert abs(info["fermiLevelUsed"] - winfo["fermiLevelUsed"]) < 1e-12
    assert np.abs(rho - want).max() <= 1e-12 * np.abs(want).max()
    V[0, -1] = 1.3                             # endpoints disagree
    with pytest.raises(WignerError):
        PR.contact_mode_reservoir(mat, f, "source", 1.45, V)
    mat = small_mat("material-default", "zero-inflow")
    mat["dg"]["params"]["full2D_sourceContactMask"] = [1, 1, 0, 1, 1, 1]     # per face dof: one closed
    out = PR.get_InflowBoundary_full2D(mat, H.build_factors(mat), 1.45, 1.4, np.full((11, 5), 1.424))
    src = out["source"][0]
    assert np.abs(src[:, 2]).max() == 0 and np.abs(src[:, [0, 1, 3, 4, 5]]).min(axis=0).max() >= 0
    assert np.abs(out["drain"][0]).max() > 0
    mat["dg"]["params"]["full2D_sourceContactMask"] = [1, 0, 1, 1]           # neither face dofs nor Ny
    with pytest.raises(WignerError) as e:
        H.build_factors(mat)
    assert e.value.identifier == "DG:Full2D:InvalidContactMask"


@pytest.mark.gpu
def test_gpu_solve_of_the_reservoir_driven_system(built_lib):
    """The Full-2D device solve (mixed and FP64) of A rho = rhs with the contact-mode reservoir
    right-hand side, against the oracle's sparse LU of the same system."""
    import scipy.sparse.linalg as spla
    from real_space_dg_gb300.full2d import Full2DOperator
    mat = small_mat("contact-modes", "periodic")
    XX, YY = np.meshgrid(mat["x"], mat["y"], indexing="ij")
    V = 1.424 + 0.15 * np.exp(-((XX - 10) / 3) ** 2) - 0.05 * XX / 20
    p, parts, dd = F2.system(mat, V)
    A = F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"]) + F2.assemble_drift(p, dd)
    with Full2DOperator(mat, V) as op:
        rhs, inflow = op.reservoir_rhs(1.45, 1.40)
        want = spla.spsolve(A.tocsc(), rhs)
        op.set_preconditioner(fp32=True)
        for mixed in (False, True):
            st, info, x = op.solve(rhs, tol=1e-11, maxit=200, restart=20, mixed=mixed)
            assert st == 0
            assert np.linalg.norm(x - want) <= 1e-8 * np.linalg.norm(want)


@pytest.mark.gpu
def test_gpu_observables_match_oracle(built_lib):
    """get_Observables_full2D on the device: density at zero separation, the x and y currents,
    projected onto the material Y grid (odd and even rho_y counts: the exact cell and the linear
    bracket), from a host state and from the resident solution of a solve."""
    from real_space_dg_gb300.full2d import Full2DOperator
    rng = np.random.default_rng(3)
    for ybc, nry in (("periodic", 4), ("zero-inflow", 5)):
        mat = small_mat("material-default", ybc, nry=nry)
        p = F2.init_params_full2d(mat)
        rho = rng.normal(size=p["nTotal"]) + 1j * rng.normal(size=p["nTotal"])
        want = F2.observables(p, mat, rho)
        jy, jyDG = F2.observables_y(p, mat, rho)
        with Full2DOperator(mat) as op:
            got = op.observables(rho)
            for a, b in zip(got, want):
                assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
            allo = op.observables_all(rho)
            assert np.abs(allo["jy"] - jy).max() <= 1e-13 * np.abs(jy).max()
            assert np.abs(allo["jyDG"] - jyDG).max() <= 1e-13 * np.abs(jyDG).max()
        # the resident solution of a solve gives the observables of the returned state
        XX, YY = np.meshgrid(mat["x"], mat["y"], indexing="ij")
        V = 1.424 + 0.1 * np.exp(-((XX - 10) / 3) ** 2)
        with Full2DOperator(mat, V) as op:
            op.set_preconditioner(fp32=True)
            b = rng.normal(size=op.n) + 1j * rng.normal(size=op.n)
            st, info, x = op.solve(b, tol=1e-10, maxit=100, restart=20)
            assert st == 0
            for a, c in zip(op.observables(), F2.observables(p, mat, x)):
                assert np.abs(a - c).max() <= 1e-13 * np.abs(c).max()


@pytest.mark.gpu
def test_gpu_recorded_bias_point_reproduces_the_recorded_density_and_current(built_lib):
    """The recorded run's system at 0.6 V (its stored potential and contact-mode reservoirs) solved
    on the device with the run's settings (GMRES(40), line-transverse preconditioner, 5e-6)
    reproduces the density and current the reference stored for it; both solves stop at a ~5e-6
    relative residual, which bounds the agreement (measured 1.0e-4 / 3.6e-4, mean current 3.6e-5)."""
    from real_space_dg_gb300.full2d import Full2DOperator
    g, mat = recorded()
    with Full2DOperator(mat, g["potential"]) as op:
        rhs, inflow = op.reservoir_rhs(float(g["ef_input_source"]), float(g["ef_input_drain"]))
        op.set_preconditioner()
        st, info, x = op.solve(rhs, tol=5e-6, maxit=600, restart=40, mixed=True)
        assert st == 0
        n, j, _, _ = op.observables(x)
    assert np.abs(n - g["density"]).max() <= 1e-3 * np.abs(g["density"]).max()
    assert np.abs(j - g["current"]).max() <= 3e-3 * np.abs(g["current"]).max()
    assert abs(np.mean(j) - np.mean(g["current"])) <= 3e-4 * abs(np.mean(g["current"]))


@pytest.mark.parametrize("ybc", ["zero-inflow", "hard-wall", "specular"])
def test_host_box_contact_modes_match_oracle(ybc):
    """The non-periodic contact problem (get_ContactModeReservoirRho_full2D.m:153-367): the transverse
    Hamiltonian of the contact column (ghost-node closure, or the hard-wall interior), the modes of
    smallest |E|, their density matrix by linear interpolation, the contact-neutrality level; host
    against the oracle's literal restatement, with a Y-dependent contact potential."""
    from real_space_dg_gb300 import full2d as H, reservoir as PR
    mat = small_mat("contact-modes", ybc, nry=8)
    mat["dg"]["params"].update(L_rho_y=6e-9, full2D_contactModeCount=3)
    V = np.full((11, 5), 1.424)
    V[0] += 0.02 * np.sin(np.linspace(0, np.pi, 5))
    V[-1] -= 0.01 * np.linspace(0, 1, 5)
    f = H.build_factors(mat)
    p = F2.init_params_full2d(mat)
    for side, ef in (("source", 1.45), ("drain", 1.40)):
        rho, info = PR.contact_mode_reservoir(mat, f, side, ef, V)
        want, winfo = R.contact_mode_reservoir(mat, p, side, ef, V)
        assert np.allclose(info["modeEnergy"], winfo["modeEnergy"], rtol=1e-13, atol=0)
        assert abs(info["fermiLevelUsed"] - winfo["fermiLevelUsed"]) < 1e-12
        assert np.abs(rho - want).max() <= 1e-12 * np.abs(want).max() and np.abs(want).max() > 0
    # box modes vanish beyond the grid: no density where both particle coordinates leave the face
    Eb, modes, grid, hard = PR._box_modes(mat, f, "source", V)
    assert modes.shape == (5, 3) and np.all(np.diff(Eb) > 0)
    if ybc == "hard-wall":
        assert hard and np.all(modes[[0, -1]] == 0)
