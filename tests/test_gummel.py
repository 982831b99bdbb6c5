"""Gummel / Poisson self-consistency: CPU pins of the oracle and GPU parity.

GPU tolerances: a fixed number of Gummel iterations reproduces the oracle's
potential to 1e-9 V and the density to 1e-8 relative (the transport solves
differ only by the 1e-12 GMRES tolerance); a converged loop reproduces the
oracle's fixed point to the potential tolerance.
"""
import numpy as np
import pytest

from conftest import small_rtd
from oracle import dg1d, gummel1d


def test_poisson_matrix_is_second_difference():
    x = np.linspace(0, 10, 41)
    eps = np.full(41, 12.9)
    lo, di, up = gummel1d.poisson_matrix(x, eps)
    phi = 0.3 * x ** 2
    lap = lo[1:-1] * phi[:-2] + di[1:-1] * phi[1:-1] + up[1:-1] * phi[2:]
    assert np.allclose(lap, gummel1d.EPS0 * 12.9 * 0.6 * 1e18, rtol=1e-10)


def test_poisson_step_keeps_neutral_linear_potential():
    x = np.linspace(0, 20, 81)
    tri = gummel1d.poisson_matrix(x, np.full(81, 12.9))
    nd = np.full(81, 1e24)
    phi = 0.2 * x / 20
    cand, info = gummel1d.poisson_step(tri, nd.copy(), nd, phi, 0.2, 300.0)
    assert info["converged"] and np.abs(cand - phi).max() < 1e-14


def test_projection_conserves_the_dg_integral():
    spec, mat, E, efl, efr, m = small_rtd(n_el=7, nk=16, order=3)
    p = dg1d.init_params(mat, efl, efr, E, m)
    T = gummel1d.projection(mat["x"], p)
    x = mat["x"]
    widths = np.diff(np.concatenate(([x[0]], (x[:-1] + x[1:]) / 2, [x[-1]])))
    n = np.cos(np.arange(T.shape[1]))
    # integral over the control volumes == integral of the DG polynomial (mass row sums)
    w = np.tile(dg1d.jacobi.jacobi_gl(0, 0, 3)[1], 7) * (x[3] - x[0]) / 2
    assert abs(widths @ (T @ n) - w @ n) < 1e-12 * abs(w @ n)


def _rtd(n_el=12, nk=32, order=2, bias=0.1):
    from real_space_dg_gb300 import devices
    spec, mat, E, efl, efr, m = small_rtd(n_el=n_el, nk=nk, order=order, bias=bias)
    dy = devices.density_normalisation_nm(mat)
    return spec, mat, dy


@pytest.mark.gpu
def test_gummel_iterates_match_oracle(built_lib):
    from real_space_dg_gb300.rtd import RTDSweep
    spec, mat, dy = _rtd()
    bias = 0.1
    ref = gummel1d.gummel(mat, bias, bias * mat["ramp"], dy_nm=dy, mixing=0.3, potential_tol=1e-30,
                          density_tol=1e-30, max_iterations=4)
    S = RTDSweep(mat, 1, dict(mixing=0.3, potentialTolerance=1e-30, densityTolerance=1e-30, maxIterations=4,
                              transportTolerance=1e-12, transportMaxCycles=60))
    S.dy = dy
    try:
        S.set(0, bias)
        st, info = S.run()
        phi, n, j = S.get(0)
    finally:
        S.close()
    assert info[0]["iterations"] == 4 and info[0]["status"] == 1
    assert np.abs(phi - ref["phi"]).max() < 1e-9
    assert np.linalg.norm(n - ref["n"]) < 1e-8 * np.linalg.norm(ref["n"])
    assert np.linalg.norm(j - ref["j"]) < 1e-7 * np.linalg.norm(ref["j"])
    assert abs(info[0]["potential_defect"] - ref["history"][-1]["defect"]) < 1e-9


@pytest.mark.gpu
def test_gummel_fixed_point_and_batch_independence(built_lib):
    from real_space_dg_gb300.rtd import RTDSweep, solve_rtd_self_consistent
    spec, mat, dy = _rtd(n_el=10, nk=24)
    opts = dict(mixing=0.5, potentialTolerance=1e-6, densityTolerance=1e-5, maxIterations=120,
                transportTolerance=1e-11, transportMaxCycles=60)
    mat = dict(mat, dy_norm_nm=dy)
    biases = [0.0, 0.1, 0.2]
    res = solve_rtd_self_consistent(mat, biases, opts, mode="batched")
    assert res["selfConsistency"]["converged"], res["sweep"]["status"]
    for ib, bias in enumerate(biases):
        ref = gummel1d.gummel(mat, bias, bias * mat["ramp"], dy_nm=dy, mixing=0.5, potential_tol=1e-6,
                              density_tol=1e-5, max_iterations=120)
        assert ref["status"] == "fixed-point-converged"
        assert np.abs(res["sweep"]["phi"][:, ib] - ref["phi"]).max() < 2e-5
        assert np.linalg.norm(res["sweep"]["current"][:, ib] - ref["j"]) <= 1e-3 * np.linalg.norm(ref["j"]) + 1e-30
    # one bias alone gives the same as inside the batch
    alone = solve_rtd_self_consistent(mat, [0.1], opts, mode="batched")
    assert np.abs(alone["sweep"]["phi"][:, 0] - res["sweep"]["phi"][:, 1]).max() < 1e-12
    # sequential continuation reaches the same fixed points
    seq = solve_rtd_self_consistent(mat, biases, opts, mode="sequential")
    assert seq["selfConsistency"]["converged"]
    assert np.abs(seq["sweep"]["phi"] - res["sweep"]["phi"]).max() < 2e-5


@pytest.mark.gpu
@pytest.mark.parametrize("precision,factor,cap", [("fp64", 1e-2, 1e-4), ("mixed", 1e-2, 1e-4), ("mixed", 0.3, 1e-3)])
def test_inexact_gummel_reaches_the_same_fixed_point(built_lib, precision, factor, cap):
    """Transport tolerance tied to the potential defect (opt-in) converges to the
    fixed point of the exact loop; the accepted state is solved at 1e-8."""
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.rtd import solve_rtd_self_consistent
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=32, order=2)
    mat = dict(mat, dy_norm_nm=devices.density_normalisation_nm(mat))
    opts = dict(mixing=0.5, potentialTolerance=1e-6, densityTolerance=1e-5, maxIterations=150,
                transportTolerance=1e-8, transportMaxCycles=60, precision=precision)
    exact = solve_rtd_self_consistent(mat, [0.05, 0.15], opts)
    inexact = solve_rtd_self_consistent(mat, [0.05, 0.15], dict(opts, inexactFactor=factor, inexactCap=cap))
    assert exact["selfConsistency"]["converged"] and inexact["selfConsistency"]["converged"]
    assert max(inexact["sweep"]["transport_relres"]) <= 1e-8
    assert np.abs(inexact["sweep"]["phi"] - exact["sweep"]["phi"]).max() < 1e-5
    assert sum(inexact["sweep"]["gmres_iterations"]) < sum(exact["sweep"]["gmres_iterations"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_deferred_final_resolves_keep_every_problems_iterates(built_lib, precision):
    """Batching the final-tolerance re-solves (a loosely converged problem waits, frozen, until the
    others leave their loose phase) changes when a problem's iterations run, not what they compute:
    the same Gummel and GMRES iteration counts per problem and the same fixed point (bit-identical
    in FP64; the mixed form's emulated residual GEMM shares column tiles between problems, 1e-10 V)."""
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.rtd import solve_rtd_self_consistent
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=32, order=2)
    mat = dict(mat, dy_norm_nm=devices.density_normalisation_nm(mat))
    opts = dict(mixing=0.5, potentialTolerance=1e-6, densityTolerance=1e-5, maxIterations=150,
                transportTolerance=1e-8, transportMaxCycles=60, precision=precision, inexactFactor=0.3,
                inexactCap=1e-3)
    biases = [0.02, 0.1, 0.18, 0.25]
    now = solve_rtd_self_consistent(mat, biases, dict(opts, deferFinal=-1))
    deferred = solve_rtd_self_consistent(mat, biases, dict(opts, deferFinal=0))
    assert now["selfConsistency"]["converged"] and deferred["selfConsistency"]["converged"]
    if precision == "fp64":
        assert now["sweep"]["iterations"] == deferred["sweep"]["iterations"]
        assert now["sweep"]["gmres_iterations"] == deferred["sweep"]["gmres_iterations"]
        assert np.array_equal(now["sweep"]["phi"], deferred["sweep"]["phi"])
    else:
        assert np.abs(now["sweep"]["phi"] - deferred["sweep"]["phi"]).max() < 1e-10


@pytest.mark.gpu
def test_kept_handles_give_the_results_of_fresh_handles(built_lib):
    """solve_rtd_self_consistent keeps its handles for the next call with the same shape, layout and
    options; a kept set rebound to another device of the same node count, and back, reproduces the
    fresh handles' sweep bit for bit (FP64: the same launches on the same inputs)."""
    from real_space_dg_gb300 import devices, rtd
    mats = []
    for barrier in (0.3, 0.2):
        spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=32, order=2, barrier_ev=barrier)
        mats.append(dict(mat, dy_norm_nm=devices.density_normalisation_nm(mat)))
    opts = dict(mixing=0.5, potentialTolerance=1e-6, densityTolerance=1e-5, maxIterations=150,
                transportTolerance=1e-8, transportMaxCycles=60, precision="fp64")
    biases = [0.05, 0.1, 0.2]
    try:
        fresh = [rtd.solve_rtd_self_consistent(M, biases, dict(opts, keepHandles=False), handles=2) for M in mats]
        assert rtd._KEPT["sweeps"] == []
        first = rtd.solve_rtd_self_consistent(mats[0], biases, opts, handles=2)
        kept = list(rtd._KEPT["sweeps"])
        assert len(kept) == 2
        other = rtd.solve_rtd_self_consistent(mats[1], biases, opts, handles=2)
        again = rtd.solve_rtd_self_consistent(mats[0], biases, opts, handles=2)
        assert rtd._KEPT["sweeps"] == kept            # the same handles served all three calls
        for got, want in ((first, fresh[0]), (other, fresh[1]), (again, fresh[0])):
            assert got["selfConsistency"]["converged"]
            assert got["sweep"]["iterations"] == want["sweep"]["iterations"]
            assert got["sweep"]["gmres_iterations"] == want["sweep"]["gmres_iterations"]
            for k in ("phi", "density", "current"):
                assert np.array_equal(got["sweep"][k], want["sweep"][k]), k
        assert np.abs(fresh[0]["sweep"]["phi"] - fresh[1]["sweep"]["phi"]).max() > 1e-3   # two devices
        rtd.solve_rtd_self_consistent(mats[0], biases[:2], opts, handles=2)           # another layout
        assert rtd._KEPT["sweeps"] and all(a is not b for a in rtd._KEPT["sweeps"] for b in kept)
        assert all(sw.P.h is None for sw in kept)     # the replaced set was closed
    finally:
        rtd.release_handles()
    assert rtd._KEPT["sweeps"] == []
