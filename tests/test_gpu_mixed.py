"""GPU tests of the mixed-precision form (tcgen05 BF16 transforms in FP64 refinement).

Tolerances: the tensor-core GEMM against a float64 product of the same
bf16-rounded operands, 1e-5 relative (FP32 accumulation); the emulated FP64
GEMM against numpy FP64, 2e-13 of |A| |B| elementwise, and the mixed handle's
FP64 operator built on it against the oracle's sparse matrix, 1e-12; the low-precision
operator against the FP64 operator, 2e-2 relative (BF16 operands); the refined
solution against the oracle's sparse LU at a 1e-10 residual target: density
1e-8 and current 1e-7 relative (the mixed form's bar against FP64).
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from conftest import small_rtd
from oracle import dg1d

pytestmark = pytest.mark.gpu


def bf16_round(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def test_bounded_barrier_wait_gives_up_and_leaves_the_context_usable(built_lib):
    """The failure path of the tensor-core kernels without a GPU fault: an mbarrier wait that nothing
    completes gives up after its poll limit, raises the error flag the host reads (WG_ERR_TIMEOUT,
    the GEMMs' "bounded barrier wait timed out"), and the same context then runs the tcgen05 GEMM
    correctly."""
    from real_space_dg_gb300 import _lib
    lib = _lib.load()
    assert lib.wg_debug_wait_timeout(1 << 14) == _lib.WG_ERR_TIMEOUT
    assert b"bounded barrier wait timed out" in lib.wg_global_error()
    test_tcgen05_bf16_gemm(built_lib, 128, 64, 64)


@pytest.mark.parametrize("M,N,K", [(256, 300, 128), (128, 64, 64), (512, 1000, 512), (40, 37, 64)])
def test_tcgen05_bf16_gemm(built_lib, M, N, K):
    from real_space_dg_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)            # row-major M x K
    B = rng.standard_normal((N, K)).astype(np.float32)            # column-major K x N == row-major N x K
    Cout = np.zeros((N, M), dtype=np.float32)                     # column-major M x N
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    st = lib.wg_debug_gemm_bf16(fp(A), fp(B), fp(Cout), M, N, K)
    assert st == 0, lib.wg_global_error()
    ref = bf16_round(B) @ bf16_round(A).T                          # (N x M) = column-major M x N
    assert rel(Cout, ref) < 1e-5


@pytest.mark.parametrize("M,N,K", [(256, 300, 512), (200, 150, 512), (128, 64, 64), (40, 37, 72), (1024, 130, 1024)])
def test_fp64_emulated_gemm(built_lib, M, N, K):
    """Digit-sliced FP64 GEMM on the tensor cores against numpy FP64: rows and
    columns spanning many binades, a zero column and a ragged tile edge; the
    error is bounded by 2e-13 of |A| |B| elementwise."""
    from real_space_dg_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(M * N + K)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-20, 20, (M, 1)))      # row-major M x K
    Bt = rng.standard_normal((N, K)) * np.exp(rng.uniform(-20, 20, (N, 1)))     # column-major K x N
    Bt[N // 2] = 0.0
    Bt[1, ::3] *= 1e-30                                                          # wide range inside a column
    Cout = np.zeros((N, M))                                                      # column-major M x N
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    st = lib.wg_debug_gemm_f64_tc(dp(A), dp(Bt), dp(Cout), M, N, K)
    assert st == 0, lib.wg_global_error()
    ref = Bt @ A.T
    bound = np.abs(Bt) @ np.abs(A).T
    assert np.all(np.abs(Cout - ref) <= 2e-13 * bound)
    assert np.all(Cout[N // 2] == 0.0)


@pytest.mark.parametrize("nd", [3, 4, 5, 6, 7, 8])
def test_fp64_emulated_gemm_fewer_digits(built_lib, nd):
    """The emulated GEMM with only nd leading digits per operand (the mixed form's residual at
    loose tolerances): error within 64 * 2^(-6 nd) of |A| |B| elementwise, and below it the
    full split is more accurate."""
    from real_space_dg_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(nd)
    M, N, K = 256, 150, 512
    A = rng.standard_normal((M, K)) * np.exp2(rng.integers(-20, 20, (M, 1)))
    Bt = rng.standard_normal((N, K)) * np.exp2(rng.integers(-20, 20, (N, 1)))
    Cout = np.zeros((N, M))
    dp = lambda a: np.ascontiguousarray(a).ctypes.data_as(_lib._D)
    st = lib.wg_debug_gemm_f64_tc_digits(dp(A), dp(Bt), dp(Cout), M, N, K, nd)
    assert st == 0, lib.wg_global_error()
    bound = np.abs(Bt) @ np.abs(A).T
    err = np.abs(Cout - Bt @ A.T)
    assert np.all(err <= 64 * 2.0 ** (-6 * nd) * bound)
    if nd < 8:
        assert err.max() / bound.max() > 2.0 ** (-6 * (nd + 1)) * 1e-3   # the digits really were dropped


def make(spec, precision, batch=1, **kw):
    from real_space_dg_gb300 import Problem1D
    return Problem1D(n_el=spec.n_el, n_local=spec.n_local, nk=spec.nk, n_xi=spec.n_xi or spec.nk,
                     l_xi=spec.l_xi_m, batch=batch, precision=precision, **kw)


@pytest.mark.parametrize("order,nk,nxi", [(2, 32, 0), (3, 64, 0), (1, 32, 40)])
def test_lowprec_operator_close_to_fp64(built_lib, order, nk, nxi):
    spec, mat, E, efl, efr, m = small_rtd(n_el=12, nk=nk, order=order, n_xi=nxi)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    with make(spec, "mixed") as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        rng = np.random.default_rng(0)
        x = rng.standard_normal(P.N) + 1j * rng.standard_normal(P.N)
        y64 = P.apply(x)
        ylo = P.apply_lowprec(x)
        assert rel(y64, A @ x) < 1e-12
        assert rel(ylo, y64) < 2e-2


@pytest.mark.parametrize("order,nk", [(2, 32), (3, 64)])
def test_mixed_solve_matches_direct_solve(built_lib, order, nk):
    spec, mat, E, efl, efr, m = small_rtd(n_el=12, nk=nk, order=order)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    ref = spla.spsolve(A.tocsc(), rhs)
    n_ref, j_ref, _ = dg1d.observables(p, ref, dg1d.node_map(p, m))
    with make(spec, "mixed") as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        st, info = P.solve(tol=1e-10, maxit=40)
        assert st == 0 and info[0]["flag"] == 0 and info[0]["relres"] <= 1e-10
        assert info[0]["refinements"] >= 2
        n, j = P.observables(0)
        assert rel(n, n_ref) < 1e-8
        assert rel(j, j_ref) < 1e-7


def test_mixed_batch_and_warm_start(built_lib):
    specs = [small_rtd(n_el=10, nk=32, order=2, bias=b) for b in (0.05, 0.15, 0.25)]
    spec0 = specs[0][0]
    with make(spec0, "mixed", batch=3) as P:
        for b, (spec, mat, E, efl, efr, m) in enumerate(specs):
            P.set_potential(b, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        st, info = P.solve(tol=1e-10, maxit=40)
        assert st == 0
        for b, (spec, mat, E, efl, efr, m) in enumerate(specs):
            p = dg1d.init_params(mat, efl, efr, E, m)
            A, rhs = dg1d.get_sysm(mat, p, E)
            assert rel(P.rho(b), spla.spsolve(A.tocsc(), rhs)) < 1e-8
        st, info = P.solve(tol=1e-10, maxit=40, warm=True)
        assert all(i["iterations"] == 0 for i in info)


def test_mixed_gummel_matches_fp64_gummel(built_lib):
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.rtd import solve_rtd_self_consistent
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=32, order=2)
    mat = dict(mat, dy_norm_nm=devices.density_normalisation_nm(mat))
    opts = dict(mixing=0.5, potentialTolerance=1e-6, densityTolerance=1e-5, maxIterations=150,
                transportTolerance=1e-10, transportMaxCycles=40)
    r64 = solve_rtd_self_consistent(mat, [0.1, 0.2], dict(opts, precision="fp64"))
    rmx = solve_rtd_self_consistent(mat, [0.1, 0.2], dict(opts, precision="mixed"))
    assert r64["selfConsistency"]["converged"] and rmx["selfConsistency"]["converged"]
    assert np.abs(rmx["sweep"]["phi"] - r64["sweep"]["phi"]).max() < 1e-5
    assert rel(rmx["Id"], r64["Id"]) < 1e-3


def test_mixed_rejects_unsupported_shapes(built_lib):
    from real_space_dg_gb300 import WignerError
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=16, order=2)
    with pytest.raises(WignerError):
        make(spec, "mixed")


@pytest.mark.parametrize("order", [1, 2, 3])
def test_fused_apply_matches_the_four_launch_apply(built_lib, order, monkeypatch):
    """The opt-in two-launch apply (GEMM 1 with the xi stencil in its TMEM epilogue, GEMM 2 with
    the flux in its epilogue, WG_FUSED_APPLY=1) computes the same low-precision operator as the
    four-launch apply (the same BF16 operands and FP32 arithmetic in another order: 1e-3 relative),
    and the mixed solve built on it reaches the sparse-LU bars (density 1e-8, current 1e-7)."""
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=128, order=order)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    rng = np.random.default_rng(order)
    out = {}
    for fused in ("0", "1"):
        monkeypatch.setenv("WG_FUSED_APPLY", fused)
        with make(spec, "mixed") as P:
            P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
            x = rng.standard_normal(P.N) + 1j * rng.standard_normal(P.N) if fused == "0" else out["x"]
            out["x"] = x
            out[fused] = P.apply_lowprec(x)
            if fused == "1":
                st, info = P.solve(tol=1e-10, maxit=40)
                assert st == 0 and info[0]["relres"] <= 1e-10
                n, j = P.observables(0)
    assert rel(out["1"], out["0"]) < 1e-3
    ref = spla.spsolve(A.tocsc(), rhs)
    n_ref, j_ref, _ = dg1d.observables(p, ref, dg1d.node_map(p, m))
    assert rel(n, n_ref) < 1e-8 and rel(j, j_ref) < 1e-7
