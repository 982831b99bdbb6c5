"""The allocation-free operator apply (wg_apply_noalloc) against wg_apply.

wg_apply_noalloc serves callers that may not allocate device memory while they
call in (applications that own all device memory through their own allocator,
or code recording a CUDA graph).  They pass their own device buffers; the
library's only scratch is a fixed static device array.  This test fills such
buffers (torch provides the device memory here), applies the operator twice in
a row with different inputs, and compares with the handle-based wg_apply at
the FP64 operator tolerance of the other parity tests (1e-12 relative).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import small_rtd

pytestmark = pytest.mark.gpu


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


def test_noalloc_apply_matches_handle_apply(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import dg1d, krylov
    from real_space_dg_gb300 import Problem1D, _lib
    lib = _lib.load()
    cases = [small_rtd(n_el=10, nk=24, order=2, bias=b) for b in (0.05, 0.2)]
    spec = cases[0][0]
    nK, n_el, nk = spec.n_local, spec.n_el, spec.nk
    nxi = spec.n_xi or nk
    batch = len(cases)
    betas, qds = [], []
    with Problem1D(n_el=n_el, n_local=nK, nk=nk, n_xi=nxi, l_xi=spec.l_xi_m, batch=batch) as P:
        for b, (sp, mat, E, efl, efr, m) in enumerate(cases):
            P.set_potential(b, mat["x"], E, m, sp.m_rel, sp.temp_k, efl, efr)
            p = dg1d.init_params(mat, efl, efr, E, m)
            op = krylov.Operator1D(mat, p, E)
            betas.append(np.real(op.beta))
            qds.append(p["Q_diff"] / (p["delta_chi"] / 2))
        Kb = dg1d.k_blocks(p)
        K = {"K1": Kb["K1"], "K2": Kb["K2L"] + Kb["K2R"], "K3": Kb["K3"], "K5": Kb["K5"]}
        dev = torch.device("cuda:0")
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).ravel()).to(dev)
        arrays = [f64(p["phi"].view(np.float64)), f64(p["k"]), f64(qds), f64(np.stack(betas)),
                  f64(np.imag(op.beta[0]))]
        view = _view(_lib, arrays, n_el, nK, nk, nxi, batch, K)
        rng = np.random.default_rng(7)
        for call in range(2):
            x = rng.standard_normal(P.N * batch) + 1j * rng.standard_normal(P.N * batch)
            xd = f64(x.view(np.float64))
            yd = torch.full_like(xd, float("nan"))
            st = lib.wg_apply_noalloc(C.byref(view), C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), None)
            assert st == 0, lib.wg_global_error()
            torch.cuda.synchronize()
            y = yd.cpu().numpy().view(np.complex128)
            y_ref = P.apply(x)
            assert np.linalg.norm(y - y_ref) <= 1e-12 * np.linalg.norm(y_ref), call


def test_noalloc_rejects_sizes_beyond_the_static_scratch(built_lib):
    from real_space_dg_gb300 import _lib
    lib = _lib.load()
    v = _lib.WgOperatorView()
    v.n_el, v.n_local, v.nk, v.n_xi, v.batch = 4096, 4, 256, 256, 1        # 4096*4*256 > 2^19
    v.phi = v.kvec = v.qd = v.beta = v.betai = 1                          # never dereferenced
    st = lib.wg_apply_noalloc(C.byref(v), C.c_void_p(1), C.c_void_p(1), None)
    assert st == _lib.WG_ERR_ARG
    assert b"exceeds the fixed scratch" in lib.wg_global_error()
