"""Full-2D (X, Y, rho_x, rho_y) operator: the oracle's invariants, the host-built
factors against the oracle's literal assembly, and the GPU apply against both.

Tolerances: matrix-free == assembled 1e-13 relative (the reference's own
full2DDiffOperatorTest bar is 1e-10); the host factors reassemble the oracle's
transport operator to 1e-13; the GPU apply (FP64) matches the oracle to 1e-12
relative L2; with a constant potential the drift term reduces to the CAP term up
to the rounding of the interpolated potential differences (relative 1e-12).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import full2d as F2

CONFIGS = [
    dict(yb="periodic", fx="upwind", fy="upwind"),          # the shape of the reference's Sim_Res run
    dict(yb="zero-inflow", fx="rusanov", fy="central"),
    dict(yb="specular", fx="upwind", fy="rusanov"),
    dict(yb="hard-wall", fx="upwind", fy="upwind"),         # constrain_HardWall_full2D.m
    dict(yb="zero-inflow", fx="upwind", fy="upwind", masks=True),   # closed X-face pieces (contact masks)
]


def make_mat(yb="periodic", fx="upwind", fy="upwind", nex=5, ney=2, nkx=3, nky=3, nrx=9, nry=4, nq=5, masks=False):
    lx, w = 20.0, 4.0
    nx, ny = nex * (nkx - 1) + 1, ney * (nky - 1) + 1
    x, y = np.linspace(0, lx, nx), np.linspace(0, w, ny)
    prm = dict(N_K_X=nkx, N_K_Y=nky, N_el_X=nex, N_el_Y=ney, N_rho_x=nrx, N_rho_y=nry, L_rho_x=8e-9,
               full2D_X_flux=fx, full2D_Y_flux=fy, full2D_Y_boundary=yb, full2D_potentialQuadratureOrder=nq)
    if masks:     # contacts on part of each outer X face (per material y point); the rest is closed
        prm["full2D_sourceContactMask"] = (y > 0.5) & (y < 3.5)
        prm["full2D_drainContactMask"] = y < 2.5
    if yb != "periodic":
        prm["L_rho_y"] = 3e-9
    mat = dict(x=x, y=y, Nx=nx, Ny=ny, dg=dict(params=prm))
    X, Y = np.meshgrid(x, y, indexing="ij")
    V = 0.1 * np.exp(-((X - 10) / 3) ** 2) + 0.02 * np.cos(2 * np.pi * Y / w)
    return mat, V


def oracle_apply(mat, p, parts, dd, u):
    """The oracle's A u; with hard walls the constrained apply T A (mask u) + scale (u - mask u)."""
    if p["ytype"] != "hard-wall":
        return F2.apply_system(p, parts, dd, u)
    wall = F2.hard_wall_geometry(p, F2.transport_scales(mat))
    return F2.apply_hard_wall(p, wall, lambda v: F2.apply_system(p, parts, dd, v), u)


def oracle_matrix(mat, p, parts, dd):
    A = (F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"]) + F2.assemble_drift(p, dd)).tocsr()
    if p["ytype"] == "hard-wall":
        A = F2.constrain_hard_wall(p, F2.hard_wall_geometry(p, F2.transport_scales(mat)), A)
    return A


def det_vec(n):
    i = np.arange(n, dtype=float)
    return np.sin(1.3 * i) + 1j * np.cos(0.7 * i)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.mark.parametrize("cfg", CONFIGS)
def test_oracle_matrix_free_equals_assembled(cfg):
    mat, V = make_mat(**cfg)
    p, parts, dd = F2.system(mat, V)
    u = det_vec(p["nTotal"])
    A = F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"]) + F2.assemble_drift(p, dd)
    assert rel(F2.apply_system(p, parts, dd, u), A @ u) < 1e-13


def test_oracle_constant_potential_leaves_only_the_cap():
    mat, V = make_mat()
    p, parts, dd = F2.system(mat, np.full_like(V, 0.3))
    u = det_vec(p["nTotal"])
    cap = np.tile(dd["capc"] * dd["cap"], p["nCenterDof"]) * u
    assert rel(F2.apply_drift(p, dd, u), cap) < 1e-12


def test_oracle_periodic_y_derivative_and_seam():
    """Periodic Y: the rho_y derivative is circulant and the closed DG chain conserves
    the discrete mass (columns of H1 sum to zero against the mass-weighted constants)."""
    mat, V = make_mat()
    p = F2.init_params_full2d(mat)
    D = p["rhoY"]["D"].toarray()
    assert np.allclose(D, -np.roll(np.roll(D, 1, 0), 1, 1)[::-1, ::-1].T) or np.allclose(D + D.T, 0)
    assert np.allclose(D.sum(axis=1), 0)
    oy = F2.close_periodic_dg_axis(F2.one_dimensional_dg_operators(p["Y"]))
    Mg = sp.kron(sp.identity(p["Y"]["nElements"]), p["Y"]["M"] * p["Y"]["jacobian"][0]).toarray()
    ones = np.ones(p["Y"]["nDof"])
    assert abs(ones @ Mg @ oy["H1"].toarray() @ ones) < 1e-12 * np.abs(oy["H1"]).sum()


@pytest.mark.parametrize("cfg", CONFIGS)
def test_host_factors_reassemble_the_oracle_operator(cfg):
    from real_space_dg_gb300 import full2d
    mat, V = make_mat(**cfg)
    p, parts, dd = F2.system(mat, V)
    f = full2d.build_factors(mat)
    nX, nY = p["X"]["nDof"], p["Y"]["nDof"]
    nrx, nry = p["rhoX"]["nCells"], p["rhoY"]["nCells"]
    A = sp.csr_matrix((p["nTotal"], p["nTotal"]), dtype=complex)
    for c, Cm, R in f["terms"][0]:
        A = A + c * sp.kron(sp.kron(sp.identity(nY), sp.csr_matrix(Cm)), sp.kron(sp.identity(nry), sp.csr_matrix(R)))
    for c, Cm, R, m in f["closed_terms"]:      # closed X-face pieces: only their Y dofs
        A = A + c * sp.kron(sp.kron(sp.diags(m.astype(float)), sp.csr_matrix(Cm)),
                            sp.kron(sp.identity(nry), sp.csr_matrix(R)))
    for c, Cm, R in f["terms"][1]:
        A = A + c * sp.kron(sp.kron(sp.csr_matrix(Cm), sp.identity(nX)), sp.kron(sp.csr_matrix(R), sp.identity(nrx)))
    ref = F2.assemble_kron(parts, p["nCenterDof"], p["nRelative"])
    assert sp.linalg.norm(A - ref) <= 1e-13 * sp.linalg.norm(ref)
    d, cpd = f["drift"], dd["cpd"]
    assert np.allclose(d["interp"], cpd["interp"], rtol=0, atol=1e-14)
    assert np.allclose(d["proj"], cpd["proj"], rtol=1e-13, atol=1e-14)
    assert np.allclose(d["xq"].T, cpd["XQ"], rtol=1e-15, atol=0) and np.allclose(d["yq"].T, cpd["YQ"], rtol=1e-15, atol=0)
    _, vx, vy = F2.relative_projection(p)
    assert np.array_equal(d["vx"], vx) and np.array_equal(d["vy"], vy)
    assert np.allclose(d["cap"], dd["cap"], rtol=1e-15, atol=0)
    assert d["capc"] == dd["capc"] and d["pot"] == dd["pot"]


@pytest.mark.gpu
@pytest.mark.parametrize("tensor_cores", [False, True])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_gpu_apply_matches_oracle(built_lib, cfg, tensor_cores):
    """FP64 CUDA-core path and the dense |A_x| factor emulated on the tensor cores."""
    from real_space_dg_gb300.full2d import Full2DOperator
    mat, V = make_mat(**cfg)
    p, parts, dd = F2.system(mat, V)
    u = det_vec(p["nTotal"])
    with Full2DOperator(mat, V, tensor_cores=tensor_cores) as op:
        y = op.apply(u)
        # a new potential is rebuilt on the device
        V2 = V * 1.7 + 0.05
        op.set_potential(V2)
        y2 = op.apply(u)
    assert rel(y, oracle_apply(mat, p, parts, dd, u)) < 1e-12
    dd2 = F2.drift_data(mat, p, V2)
    assert rel(y2, oracle_apply(mat, p, parts, dd2, u)) < 1e-12


@pytest.mark.gpu
def test_gpu_apply_larger_orders(built_lib):
    from real_space_dg_gb300.full2d import Full2DOperator
    mat, V = make_mat(nex=4, ney=2, nkx=4, nky=2, nrx=37, nry=6, nq=4)
    p, parts, dd = F2.system(mat, V)
    u = det_vec(p["nTotal"])
    for tc in (False, True):
        with Full2DOperator(mat, V, tensor_cores=tc) as op:
            assert rel(op.apply(u), F2.apply_system(p, parts, dd, u)) < 1e-12


@pytest.mark.gpu
def test_gpu_argument_errors(built_lib):
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.full2d import Full2DOperator
    mat, V = make_mat()
    with Full2DOperator(mat) as op:
        with pytest.raises(WignerError):
            op.apply(det_vec(op.n))                 # no potential yet
        with pytest.raises(WignerError):
            op.set_potential(V[:, :1])
        op.set_potential(V)
        with pytest.raises(WignerError):
            op.apply(det_vec(op.n - 1))


@pytest.mark.parametrize("cfg", CONFIGS)
def test_host_preconditioner_factors_match_oracle(cfg):
    """The product's host set-up of the line-transverse preconditioner against the oracle's
    restatement: shift, transverse reference blocks, X-line factors, transverse inverses."""
    from real_space_dg_gb300 import full2d
    mat, V = make_mat(**cfg)
    p, parts, dd = F2.system(mat, V)
    ref = F2.line_transverse(mat, p, V, dd)
    f = full2d.build_factors(mat)
    pre = full2d.build_preconditioner(mat, V, f)
    K, Vt = full2d._transverse_reference(mat, V, 0)
    assert np.allclose(K, ref["K"], rtol=1e-13, atol=1e-13 * np.abs(ref["K"]).max())
    assert np.allclose(Vt, ref["Vt"], rtol=1e-12, atol=1e-12 * np.abs(ref["Vt"]).max())
    assert abs(pre["sigma"] - ref["sigma"]) <= 1e-13 * ref["sigma"]
    assert np.allclose(pre["lam"], ref["lam"], rtol=0, atol=1e-12 * np.abs(ref["lam"]).max())
    assert np.allclose(np.transpose(pre["xinv"], (2, 3, 0, 1)), ref["xinv"], rtol=1e-12, atol=1e-14)
    assert np.allclose(np.transpose(pre["xcpl"], (2, 3, 0, 1)), ref["xcpl"], rtol=1e-12,
                       atol=1e-14 * np.abs(ref["xcpl"]).max())
    assert np.allclose(pre["tinv"], ref["Binv"], rtol=1e-10, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("tensor_cores,fp32,tol", [(False, False, 1e-12), (True, False, 1e-12), (True, True, 2e-5)])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_gpu_preconditioner_matches_oracle(built_lib, cfg, tensor_cores, fp32, tol):
    """FP64 (CUDA cores, or the mode transforms on the tensor cores): 1e-12; the FP32 form:
    the single-precision rounding of an approximate inverse (2e-5)."""
    from real_space_dg_gb300.full2d import Full2DOperator
    mat, V = make_mat(**cfg)
    p, parts, dd = F2.system(mat, V)
    ref = F2.line_transverse(mat, p, V, dd)
    r = det_vec(p["nTotal"])
    with Full2DOperator(mat, V, tensor_cores=tensor_cores) as op:
        op.set_preconditioner(fp32=fp32)
        z = op.precondition(r)
    assert rel(z, F2.line_transverse_apply(p, ref, r)) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("fp32,mixed,basis16", [(True, False, False), (False, False, False), (True, True, False),
                                                 (True, True, True)])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_gpu_solve_matches_direct_solve(built_lib, cfg, fp32, mixed, basis16):
    """Flexible GMRES(20) on the device, preconditioned in FP32 or FP64, and the mixed form (FP64
    refinement around FP32 inner solves, inner basis in FP32 or FP16), against the oracle's sparse LU
    (the same FP64 accuracy every way); a warm start from the solution needs no iteration."""
    import scipy.sparse.linalg as spla
    from real_space_dg_gb300.full2d import Full2DOperator
    mat, V = make_mat(**cfg)
    p, parts, dd = F2.system(mat, V)
    A = oracle_matrix(mat, p, parts, dd).tocsc()
    b = det_vec(p["nTotal"])
    ref = spla.spsolve(A, b)
    with Full2DOperator(mat, V) as op:
        op.set_preconditioner(fp32=fp32)
        st, info, x = op.solve(b, tol=1e-11, maxit=200, restart=20, mixed=mixed, inner_basis_fp16=basis16)
        assert st == 0 and info["flag"] == 0, info
        assert info["relres"] <= 1e-11 and info["iterations"] > 0
        assert rel(x, ref) < 1e-8
        st2, info2, x2 = op.solve(b, x0=x, tol=1e-10, maxit=5, restart=20)
        assert st2 == 0 and info2["iterations"] == 0 and info2["cycles"] == 0
        assert np.array_equal(x2, x)


def test_oracle_hard_wall_geometry_and_constraint():
    """get_HardWallGeometry_full2D.m: the active samples form the diamond |rho_y|/2 < distance to
    the nearer wall; T is a projection (T T = T) that keeps every function supported on the
    element's active nodes; the matrix-free constrained apply equals the constrained matrix, and
    its constraint rows are scale * u."""
    mat, V = make_mat(yb="hard-wall")
    p, parts, dd = F2.system(mat, V)
    wall = F2.hard_wall_geometry(p, F2.transport_scales(mat))
    Y, rho = p["Y"]["nodes"], p["rhoY"]["cells"]
    dist = np.minimum(Y - p["y"][0], p["y"][-1] - Y)
    assert np.array_equal(wall["active"], np.abs(rho)[:, None] / 2 < dist[None, :] - 1e-20)
    assert wall["active"].any() and not wall["active"].all()
    T = wall["T"].toarray()
    assert np.abs(T @ T - T).max() < 1e-13
    act = wall["active"].T.reshape(-1).astype(float)
    v = np.cos(np.arange(act.size)) * act
    assert np.abs(T @ v - v).max() < 1e-13
    u = det_vec(p["nTotal"])
    A = oracle_matrix(mat, p, parts, dd)
    y = oracle_apply(mat, p, parts, dd, u)
    assert rel(y, A @ u) < 1e-13
    m = F2.wall_active_mask(p, wall)
    assert np.array_equal(y[m == 0], wall["scale"] * u[m == 0])


def test_host_hard_wall_matches_oracle():
    """The product's host wall data (geometry, projection blocks, scale, the rhs projection)
    against the oracle's restatement; an empty diamond is the reference's error."""
    from real_space_dg_gb300 import WignerError, full2d
    mat, V = make_mat(yb="hard-wall")
    p = F2.init_params_full2d(mat)
    wall = F2.hard_wall_geometry(p, F2.transport_scales(mat))
    f = full2d.build_factors(mat)
    assert np.array_equal(f["wall"]["active"], wall["active"])
    assert f["wall"]["scale"] == pytest.approx(wall["scale"], rel=1e-14)
    u = det_vec(p["nTotal"])
    assert rel(full2d.wall_project(f, u), F2.wall_project(p, wall, u)) < 1e-14
    thin, _ = make_mat(yb="hard-wall", ney=1, nky=2)
    thin["dg"]["params"]["L_rho_y"] = 40e-9
    with pytest.raises(WignerError) as e:
        full2d.build_factors(thin)
    assert e.value.identifier == "DG:Full2D:HardWallEmptyDomain"
    bad, _ = make_mat(yb="sticky")
    with pytest.raises(WignerError) as e:
        full2d.build_factors(bad)
    assert e.value.identifier == "DG:Full2D:UnknownYBoundaryType"


def test_contact_masks_match_oracle_and_close_the_face():
    """get_ContactMask_full2D.m: the explicit per-y masks taken to the face dofs by nearest
    neighbour, the doping-edge rule with its threshold, and the whole face without data; the host's
    masks equal the oracle's; the closed pieces add the reflected-characteristic parts (the assembled
    operators differ exactly there)."""
    from real_space_dg_gb300 import full2d
    mat, V = make_mat(yb="zero-inflow", masks=True)
    p = F2.init_params_full2d(mat)
    f = full2d.build_factors(mat)
    for side in ("source", "drain"):
        want = F2.contact_mask(mat, p, side)
        assert np.array_equal(f["contact_masks"][side], want)
        assert want.any() and not want.all()
    assert len(f["closed_terms"]) == 2
    nd_mat, _ = make_mat(yb="zero-inflow")
    Nd = np.full((nd_mat["Nx"], nd_mat["Ny"]), 1e24)
    Nd[:, 0] = 0.0
    nd_mat["Nd"] = Nd
    pn = F2.init_params_full2d(nd_mat)
    m = F2.contact_mask(nd_mat, pn, "drain")
    assert not m[0] and m[1:].all()
    assert np.array_equal(full2d.build_factors(nd_mat)["contact_masks"]["drain"], m)
    nd_mat["dg"]["params"]["full2D_contactNdThreshold"] = 2e24          # nothing above: whole face
    assert F2.contact_mask(nd_mat, pn, "source").all()
    open_mat, _ = make_mat(yb="zero-inflow")
    p0, parts0, dd0 = F2.system(open_mat, V)
    p1, parts1, dd1 = F2.system(mat, V)
    extra = [q for q in parts1 if "closed-face" in q[0]]
    assert len(extra) == 2 and len(parts1) == len(parts0) + 2


def test_periodic_contacts_need_full_masks():
    from real_space_dg_gb300 import WignerError, full2d, reservoir
    mat, V = make_mat(yb="periodic", masks=True)
    f = full2d.build_factors(mat)
    with pytest.raises(WignerError) as e:
        reservoir.get_InflowBoundary_full2D(mat, f, 1.45, 1.40, V)
    assert e.value.identifier == "DG:Full2D:PeriodicContactMask"
