"""GPU parity at the sizes of the headline configurations.

C1 (the stationary flat-band RTD: 60 nm GaAs, 15 nm contacts at 1e18 cm^-3, a
0.27 eV x 3 nm double barrier around a 5 nm well, 0.1 V linear drop, DG p=2,
N_el=120, Nk=128, L_xi=30 nm; 46,080 complex unknowns) against the oracle's
solve_transport_DG_2D, i.e. the sparse LU of the assembled system (the
reference's A\\rhs, DG_code/solve_transport_DG_2D.m:101):
  - plain FP64 (native FP64 transforms and FP64 emulated on the tensor cores),
    GMRES(50) + k-line preconditioner to the config's 1e-10 residual:
    density <= 1e-9, current <= 1e-8 relative L2;
  - the mixed form (BF16 transforms, FP32 flux/preconditioner, FP64 refinement)
    to the same residual: density <= 1e-8, current <= 1e-7.

The chosen form inside the self-consistent loop: a fixed number of Gummel
iterations (mixing 0.3, every transport solve at 1e-10) in the mixed and in the
plain FP64 form land on the same iterate, so the bars are those of the transport
itself: terminal current <= 1e-7 relative, density <= 1e-8, potential <= 1e-9 V.
"""
import numpy as np
import pytest

from oracle import dg1d

pytestmark = pytest.mark.gpu

C1 = dict(length_nm=60.0, contact_nm=15.0, barrier_ev=0.27, barrier_nm=3.0, well_nm=5.0, doping_m3=1e24,
          m_rel=0.067, temp_k=300.0, order=2, n_el=120, nk=128, l_xi_m=30e-9)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.fixture(scope="module")
def c1_reference():
    from real_space_dg_gb300 import devices
    spec = devices.RTDSpec(**C1)
    mat = devices.make_mat(spec)
    E = devices.flatband_potential(mat, 0.1)
    efl, efr = devices.contact_fermi_levels(mat, 0.1)
    m = np.full(mat["Nx"], spec.m_rel * 9.109e-31)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    import scipy.sparse.linalg as spla
    rho = spla.spsolve(A.tocsc(), rhs)
    n_ref, j_ref, _ = dg1d.observables(p, rho, dg1d.node_map(p, m))
    return spec, mat, E, efl, efr, m, rho, n_ref, j_ref


@pytest.mark.parametrize("precision,fp64_tc,basis16,tol_n,tol_j", [("fp64", False, False, 1e-9, 1e-8),
                                                                   ("fp64", True, False, 1e-9, 1e-8),
                                                                   ("mixed", False, False, 1e-8, 1e-7),
                                                                   ("mixed", False, True, 1e-8, 1e-7)])
def test_c1_solve_matches_sparse_lu(built_lib, c1_reference, precision, fp64_tc, basis16, tol_n, tol_j):
    """basis16: the mixed form's inner Krylov basis stored in FP16 (the default) or in FP32; the
    FP64 refinement holds the same bars either way."""
    from real_space_dg_gb300.transport import Problem1D, shape_from_mat
    spec, mat, E, efl, efr, m, rho, n_ref, j_ref = c1_reference
    assert spec.n_el * spec.n_local * spec.nk == 46080
    with Problem1D(batch=1, precision=precision, restart=50, fp64_tc=fp64_tc, inner_basis_fp32=not basis16,
                   **shape_from_mat(mat)) as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        st, info = P.solve(tol=1e-10, maxit=200)
        assert st == 0 and info[0]["flag"] == 0 and info[0]["relres"] <= 1e-10, info
        n, j = P.observables(0)
        assert rel(n, n_ref) < tol_n
        assert rel(j, j_ref) < tol_j
        if precision == "fp64":
            assert rel(P.rho(0), rho) < 1e-8


def test_mixed_gummel_iterates_match_fp64_at_fixed_count(built_lib):
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.rtd import RTDSweep
    spec = devices.RTDSpec(**dict(C1, length_nm=40.0, contact_nm=10.0, n_el=60, nk=64, order=3))
    mat = devices.make_mat(spec)
    mat["dy_norm_nm"] = devices.density_normalisation_nm(mat)
    biases = [0.05, 0.15]
    base = dict(mixing=0.3, potentialTolerance=1e-30, densityTolerance=1e-30, maxIterations=4,
                transportTolerance=1e-10, transportMaxCycles=80)
    out = {}
    for form, o in (("fp64", dict(precision="fp64")), ("mixed", dict(precision="mixed"))):
        S = RTDSweep(mat, len(biases), dict(base, **o))
        try:
            for b, v in enumerate(biases):
                S.set(b, v)
            st, info = S.run()
            assert all(i["iterations"] == 4 for i in info), info
            assert max(i["transport_relres"] for i in info) <= 1e-10
            out[form] = [S.get(b) for b in range(len(biases))]
        finally:
            S.close()
    for (phi64, n64, j64), (phim, nm, jm) in zip(out["fp64"], out["mixed"]):
        assert np.abs(phim - phi64).max() < 1e-9
        assert rel(nm, n64) < 1e-8
        assert abs(np.mean(jm) - np.mean(j64)) <= 1e-7 * abs(np.mean(j64))
        assert rel(jm, j64) < 1e-7
