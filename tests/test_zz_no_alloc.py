"""The allocation-free operator apply (wg_apply_noalloc).

wg_apply_noalloc serves callers that may not allocate device memory while they
call in: a MATLAB MEX gateway working on gpuArray storage, or an application
whose own pool already holds the device, where a library cudaMalloc would fail
or break the owner's accounting.  They pass their own device buffers; the
library's only scratch is a fixed static device array.  The parity test fills
such buffers (torch provides the device memory here), applies the operator
twice in a row with different inputs, and compares every problem of the batch
with the oracle's assembled matrix (A @ x) and with the handle-based wg_apply,
at the FP64 operator tolerance of the other parity tests (1e-12 relative), for
N_K = 2, 3, 4 and for N_xi != Nk.  The size check runs without a GPU.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import small_rtd

TOL = 1e-12
CASES = [(10, 24, 1, 0), (10, 24, 2, 0), (8, 16, 3, 0), (9, 20, 2, 26)]   # n_el, nk, order, n_xi


def _view(lib_mod, arrays, n_el, nK, nk, nxi, batch, K):
    v = lib_mod.WgOperatorView()
    v.n_el, v.n_local, v.nk, v.n_xi, v.batch = n_el, nK, nk, nxi, batch
    v.phi, v.kvec, v.qd, v.beta, v.betai = [a.data_ptr() for a in arrays]
    for name in ("K1", "K2", "K3", "K5"):
        arr = getattr(v, name)
        flat = np.asarray(K[name], dtype=float).ravel()
        for i in range(16):
            arr[i] = flat[i] if i < flat.size else 0.0
    return v


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.gpu
@pytest.mark.parametrize("n_el,nk,order,nxi", CASES)
def test_noalloc_apply_matches_oracle_and_handle_apply(built_lib, n_el, nk, order, nxi):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import dg1d, krylov
    from real_space_dg_gb300 import Problem1D, _lib
    lib = _lib.load()
    cases = [small_rtd(n_el=n_el, nk=nk, order=order, n_xi=nxi, bias=b) for b in (0.05, 0.2)]
    spec = cases[0][0]
    nK, nxi_ = spec.n_local, spec.n_xi or spec.nk
    batch = len(cases)
    betas, qds, mats = [], [], []
    with Problem1D(n_el=n_el, n_local=nK, nk=nk, n_xi=nxi_, l_xi=spec.l_xi_m, batch=batch) as P:
        for b, (sp, mat, E, efl, efr, m) in enumerate(cases):
            P.set_potential(b, mat["x"], E, m, sp.m_rel, sp.temp_k, efl, efr)
            p = dg1d.init_params(mat, efl, efr, E, m)
            op = krylov.Operator1D(mat, p, E)
            betas.append(np.real(op.beta))
            qds.append(p["Q_diff"] / (p["delta_chi"] / 2))
            mats.append(dg1d.get_sysm(mat, p, E)[0])
        Kb = dg1d.k_blocks(p)
        K = {"K1": Kb["K1"], "K2": Kb["K2L"] + Kb["K2R"], "K3": Kb["K3"], "K5": Kb["K5"]}
        dev = torch.device("cuda:0")
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).ravel()).to(dev)
        arrays = [f64(p["phi"].view(np.float64)), f64(p["k"]), f64(qds), f64(np.stack(betas)),
                  f64(np.imag(op.beta[0]))]
        view = _view(_lib, arrays, n_el, nK, nk, nxi_, batch, K)
        rng = np.random.default_rng(7)
        N = P.N
        for call in range(2):
            x = rng.standard_normal(N * batch) + 1j * rng.standard_normal(N * batch)
            xd = f64(x.view(np.float64))
            yd = torch.full_like(xd, float("nan"))
            st = lib.wg_apply_noalloc(C.byref(view), C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), None)
            assert st == 0, lib.wg_global_error()
            torch.cuda.synchronize()
            y = yd.cpu().numpy().view(np.complex128)
            for b in range(batch):
                seg = slice(b * N, (b + 1) * N)
                assert _rel(y[seg], mats[b] @ x[seg]) <= TOL, (call, b)
            y_ref = P.apply(x)
            assert _rel(y, y_ref) <= TOL, call


def test_noalloc_rejects_sizes_beyond_the_static_scratch(built_lib):
    """The size check comes before any CUDA call, so it runs on a machine without a GPU."""
    from real_space_dg_gb300 import _lib
    lib = _lib.load()
    v = _lib.WgOperatorView()
    v.n_el, v.n_local, v.nk, v.n_xi, v.batch = 4096, 4, 256, 256, 1        # 4096*4*256 > 2^19
    v.phi = v.kvec = v.qd = v.beta = v.betai = 1                          # never dereferenced
    st = lib.wg_apply_noalloc(C.byref(v), C.c_void_p(1), C.c_void_p(1), None)
    assert st == _lib.WG_ERR_ARG
    assert b"exceeds the fixed scratch" in lib.wg_global_error()
