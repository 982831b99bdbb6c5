"""2D Poisson step (RTD/eval_Poisson2D_rtd.m, solve_Poisson2D_rtd.m, project_DG_density_RTD.m):
the oracle pinned to closed forms, and the CUDA step (libwigner_gb300.so, wg_poisson2d_*) against
the oracle."""
import numpy as np
import pytest

from oracle import full2d as F2
from oracle import poisson2d as P2

Q = 1.602176634e-19


def grid(nx=21, ny=7, dx=1.0, dy=0.5, periodic=False, eps=11.7, seed=None, nd=0.0, **kw):
    mat = dict(Nx=nx, Ny=ny, dx=dx, dy=dy, x=np.arange(nx) * dx, y=np.arange(ny) * dy, Temp=300.0,
               eps=np.full((nx, ny), eps), Nd=np.full((nx, ny), nd))
    if seed is not None:
        rng = np.random.default_rng(seed)
        mat["eps"] = rng.uniform(3.9, 12.0, (nx, ny))
        mat["Nd"] = rng.uniform(0.0, 1e24, (nx, ny))
        if periodic:
            mat["eps"][:, -1] = mat["eps"][:, 0]
            mat["Nd"][:, -1] = mat["Nd"][:, 0]
    if periodic:
        mat["dg"] = dict(params=dict(full2D_Y_boundary="periodic"))
    mat.update(kw)
    return mat


def density(mat, seed=1, scale=1e24):
    rng = np.random.default_rng(seed)
    n = rng.uniform(0.2, 1.0, (mat["Nx"], mat["Ny"])) * scale
    if mat.get("dg", {}).get("params", {}).get("full2D_Y_boundary") == "periodic":
        n[:, -1] = n[:, 0]
    return n


# ------------------------------------------------------------------------------------------ oracle

@pytest.mark.parametrize("periodic", [False, True])
def test_oracle_zero_charge_gives_the_linear_profile(periodic):
    mat = grid(periodic=periodic)
    M, num, typ, _ = P2.eval_poisson2d(mat)
    phi, _, info = P2.solve_poisson2d(M, typ, num, np.zeros((21, 7)), mat, np.zeros((21, 7)), 0.5)
    assert np.abs(phi - np.linspace(0, 0.5, 21)[:, None]).max() < 1e-13
    assert info["converged"] and info["linearRelres"] < 1e-12


def test_oracle_uniform_charge_gives_the_parabola():
    """div(eps0 eps_r grad phi) = q (n - Nd) with a uniform net charge: the 3-point stencil is exact
    on the parabola phi = rho x (x - L) / (2 eps) between grounded contacts."""
    mat = grid(nd=1e24)
    M, num, typ, _ = P2.eval_poisson2d(mat)
    phi, _, _ = P2.solve_poisson2d(M, typ, num, np.zeros((21, 7)), mat, np.zeros((21, 7)), 0.0)
    x = np.arange(21) * 1e-9
    rho = -Q * 1e24
    want = rho * x * (x - x[-1]) / (2 * P2.EPS0 * 11.7)
    assert np.abs(phi - want[:, None]).max() < 1e-12 * np.abs(want).max()


def test_oracle_flux_continuity_across_a_permittivity_step():
    mat = grid(nx=16, ny=3)
    mat["eps"][8:] = 3.9
    M, num, typ, _ = P2.eval_poisson2d(mat)
    phi, _, _ = P2.solve_poisson2d(M, typ, num, np.zeros((16, 3)), mat, np.zeros((16, 3)), 1.0)
    e = mat["eps"][:, 0]
    face = 2 * e[:-1] * e[1:] / (e[:-1] + e[1:])
    flux = face * np.diff(phi[:, 1])
    assert np.abs(flux - flux[0]).max() < 1e-12 * abs(flux[0])


def test_oracle_newton_equals_direct_without_screening_and_converges():
    mat = grid(seed=2)
    M, num, typ, _ = P2.eval_poisson2d(mat)
    n0 = np.zeros((21, 7))
    a, _, _ = P2.solve_poisson2d(M, typ, num, n0, mat, np.zeros((21, 7)), 0.3)
    mat_n = dict(mat, poisson=dict(opt=dict(solve="newton-raphson")))
    b, _, _ = P2.solve_poisson2d(M, typ, num, n0, mat_n, np.zeros((21, 7)), 0.3)
    assert np.abs(a - b).max() < 1e-13
    with pytest.raises(ValueError):
        P2.solve_poisson2d(M, typ, num, n0, dict(mat, poisson=dict(xBoundary="neumann")), np.zeros((21, 7)), 0.3)


def dg_problem(periodic, nex=6, ney=2, nk=3, nx=13, ny=5):
    prm = dict(N_K_X=nk, N_K_Y=nk, N_el_X=nex, N_el_Y=ney, N_rho_x=4, N_rho_y=4, L_rho_x=8e-9,
               full2D_Y_boundary="periodic" if periodic else "zero-inflow")
    mat = grid(nx=nx, ny=ny, dx=1.0, dy=1.0, periodic=periodic, seed=4)
    mat["dg"] = dict(params=prm)
    p = F2.init_params_full2d(mat)
    rng = np.random.default_rng(5)
    nDG = rng.uniform(0.2, 1.0, (p["X"]["nDof"], p["Y"]["nDof"])) * 1e24
    return mat, p, nDG


@pytest.mark.parametrize("periodic", [False, True])
def test_oracle_projection_conserves_and_reproduces_constants(periodic):
    mat, p, nDG = dg_problem(periodic)
    d, info = P2.project_dg_density(nDG, p, mat, periodic)
    assert info["relativeConservationError"] < 1e-13
    dc, _ = P2.project_dg_density(np.full_like(nDG, 3e23), p, mat, periodic)
    assert np.abs(dc / 3e23 - 1).max() < 1e-13
    if periodic:
        assert np.array_equal(d[:, -1], d[:, 0])


# ------------------------------------------------------------------------------------------ GPU

CASES = [dict(periodic=False), dict(periodic=True), dict(periodic=True, seed=3),
         dict(periodic=False, seed=6, nx=40, ny=11)]


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", CASES)
def test_gpu_apply_matches_oracle(built_lib, cfg):
    from real_space_dg_gb300.poisson2d import eval_Poisson2D_rtd
    mat = grid(**cfg)
    M, _, typ, _ = P2.eval_poisson2d(mat)
    op, num, typ2, info = eval_Poisson2D_rtd(mat)
    assert np.array_equal(typ, typ2)
    rng = np.random.default_rng(0)
    phi = rng.normal(size=(mat["Nx"], mat["Ny"]))
    want = (M @ phi.reshape(-1, order="F")).reshape(mat["Nx"], mat["Ny"], order="F")
    got = op.apply(phi)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    op.close()


def _solve_both(mat, n, phi0, bias, method):
    from real_space_dg_gb300.poisson2d import eval_Poisson2D_rtd, solve_Poisson2D_rtd
    mat = dict(mat, poisson=dict(mat.get("poisson", {}), opt=dict(solve=method)))
    M, num, typ, _ = P2.eval_poisson2d(mat)
    want, err_o, info_o = P2.solve_poisson2d(M, typ, num, n, mat, phi0, bias)
    op, num2, typ2, _ = eval_Poisson2D_rtd(mat)
    got, err_g, info_g = solve_Poisson2D_rtd(op, typ2, num2, n, mat, phi0, bias)
    op.close()
    return want, err_o, info_o, got, err_g, info_g


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["direct", "newton-raphson"])
@pytest.mark.parametrize("cfg", CASES)
def test_gpu_update_matches_oracle(built_lib, cfg, method):
    mat = grid(**cfg)
    n = density(mat)
    rng = np.random.default_rng(7)
    phi0 = 0.05 * rng.normal(size=(mat["Nx"], mat["Ny"]))
    if cfg["periodic"]:
        phi0[:, -1] = phi0[:, 0]
    want, err_o, io, got, err_g, ig = _solve_both(mat, n, phi0, 0.25, method)
    assert np.abs(got - want).max() <= 1e-11 * max(1.0, np.abs(want).max())
    assert abs(err_g - err_o) <= 1e-10 * max(1.0, err_o)
    assert ig["converged"] and ig["linear_relres"] < 1e-10
    for a, b in [("physical_relres_before", "physicalRelresBefore"), ("residual_scale", "residualScale"),
                 ("net_charge_per_length", "netChargePerLength"), ("unmixed_step", "unmixedStep"),
                 ("relative_charge_imbalance", "relativeChargeImbalance")]:
        assert abs(ig[a] - io[b]) <= 1e-9 * max(abs(io[b]), 1e-30), (a, ig[a], io[b])
    # the direct update zeroes the physical residual; the Newton step leaves the screening term's part
    assert abs(ig["physical_relres_after"] - io["physicalRelresAfter"]) <= 1e-8 * io["physicalRelresAfter"] + 1e-12
    if method == "direct":
        assert ig["physical_relres_after"] < 1e-9


@pytest.mark.gpu
def test_gpu_neumann_x_newton_and_custom_contacts(built_lib):
    """Neumann X (no Dirichlet node, Newton screening only), and a mat.boundary mask with an
    interior gate node set through mat.Vbc."""
    mat = grid(seed=8, poisson=dict(xBoundary="neumann"))
    n = density(mat)
    want, _, _, got, _, ig = _solve_both(mat, n, np.zeros((21, 7)), 0.0, "newton-raphson")
    assert np.abs(got - want).max() <= 1e-11 * max(1.0, np.abs(want).max())
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.poisson2d import Poisson2D
    with Poisson2D(mat) as op, pytest.raises(WignerError):
        op.solve(n, np.zeros((21, 7)), 0.0, method="direct")
    mat2 = grid(seed=9)
    b = np.zeros((21, 7), dtype=int)
    b[[0, -1], :] = 1
    b[10, 3] = 1
    vbc = np.zeros((21, 7))
    vbc[-1, :] = 0.2
    vbc[10, 3] = -0.1
    mat2.update(boundary=b, Vbc=vbc)
    want, _, _, got, _, _ = _solve_both(mat2, density(mat2), np.zeros((21, 7)), 0.0, "direct")
    assert abs(got[10, 3] + 0.1) < 1e-15 and np.abs(got - want).max() <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("periodic", [False, True])
def test_gpu_dg_step_matches_oracle(built_lib, periodic):
    """make_RTD_poisson_step: projection of nDG onto the dual volumes and the update in one device
    call, against the oracle's project_dg_density + solve_poisson2d."""
    from real_space_dg_gb300.poisson2d import make_RTD_poisson_step, project_DG_density_RTD
    mat, p, nDG = dg_problem(periodic)
    d_o, pinfo = P2.project_dg_density(nDG, p, mat, periodic)
    d_h, _ = project_DG_density_RTD(nDG, p, mat, periodic)
    assert np.abs(d_h - d_o).max() <= 1e-13 * np.abs(d_o).max()
    M, num, typ, _ = P2.eval_poisson2d(mat)
    phi0 = np.zeros((mat["Nx"], mat["Ny"]))
    want, _, io = P2.solve_poisson2d(M, typ, num, d_o, mat, phi0, 0.1)
    step, setup = make_RTD_poisson_step(mat, "direct")
    got, info = step({"transport": {"nDG": nDG, "p": p}, "phi": phi0, "bias": 0.1})
    assert np.abs(info["electronDensity"] - d_o).max() <= 1e-12 * np.abs(d_o).max()
    assert np.abs(got - want).max() <= 1e-11 * max(1.0, np.abs(want).max())
    assert abs(info["source_integral"] - pinfo["sourceIntegral"]) <= 1e-12 * abs(pinfo["sourceIntegral"])
    assert abs(info["target_integral"] - info["source_integral"]) <= 1e-12 * abs(info["source_integral"])
    setup["operator"].close()


@pytest.mark.gpu
def test_gpu_batch_of_bias_points(built_lib):
    from real_space_dg_gb300.poisson2d import Poisson2D
    mat = grid(periodic=True, seed=3, nx=30)
    n = np.stack([density(mat, seed=s) for s in range(3)])
    phi0 = np.zeros((3, 30, 7))
    bias = np.array([0.0, 0.2, 0.4])
    with Poisson2D(mat, batch=3) as op:
        phis, dens, infos = op.solve(n, phi0, bias, method="newton-raphson")
    with Poisson2D(mat) as op1:
        for b in range(3):
            phi1, d1, i1 = op1.solve(n[b], phi0[b], bias[b], method="newton-raphson")
            assert np.array_equal(phi1, phis[b]) and np.array_equal(d1, dens[b])
            assert i1["iter_err"] == infos[b]["iter_err"]


@pytest.mark.gpu
def test_gpu_recorded_run_grid(built_lib):
    """The material grid of the reference's recorded Full-2D run (361 x 13, periodic Y: 12 unique
    rows) against the oracle."""
    mat = grid(nx=361, ny=13, dx=0.25, dy=0.25, periodic=True, seed=11)
    n = density(mat)
    want, _, _, got, _, ig = _solve_both(mat, n, np.zeros((361, 13)), 0.2, "newton-raphson")
    assert np.abs(got - want).max() <= 1e-11 * max(1.0, np.abs(want).max())


@pytest.mark.gpu
def test_gpu_argument_errors(built_lib):
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.poisson2d import Poisson2D
    with pytest.raises(WignerError):
        Poisson2D(grid(ny=40))                              # more than 32 unique Y rows
    bad = grid(periodic=True)
    bad["eps"][:, -1] = 5.0
    with pytest.raises(WignerError):
        Poisson2D(bad)                                      # RTD:PoissonPeriodicMaterial
    with pytest.raises(WignerError):
        Poisson2D(grid(poisson=dict(xBoundary="neumann"), boundary=np.ones((21, 7))))
    mat = grid(periodic=True)
    with Poisson2D(mat) as op:
        n = density(mat)
        n[:, -1] *= 2
        with pytest.raises(WignerError):
            op.solve(n, np.zeros((21, 7)), 0.1)             # RTD:NonperiodicPoissonData
        phi, _, info = op.solve(density(mat), np.zeros((21, 7)), 0.1)   # usable afterwards
        assert info["converged"]
