"""CPU checks of the C ABI: the library loads, exports every declared symbol,
and its struct layouts agree with the header (no GPU call is made)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "wigner_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wg(?:2d)?_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("wg_problem_create", "wg_set_potential", "wg_solve", "wg_get_observables",
                     "wg_problem_destroy", "wg_last_error", "wg_apply", "wg_precondition"):
        assert required in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_symbol(built_lib):
    from real_space_dg_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)
    _lib.load()


def test_struct_layouts_match_header(tmp_path):
    """Compile a C probe against the header and compare sizeof/offsetof with ctypes."""
    from real_space_dg_gb300 import _lib
    src = tmp_path / "probe.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "wigner_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(wg_params), sizeof(wg_device), sizeof(wg_solve_opts), sizeof(wg_solve_info));
  printf("%zu %zu %zu\n", offsetof(wg_params, l_xi), offsetof(wg_params, precision), offsetof(wg_params, mem_budget_bytes));
  printf("%zu %zu\n", offsetof(wg_solve_info, relres), offsetof(wg_solve_info, rhs_norm));
  printf("%zu %zu %zu %zu %zu\n", sizeof(wg_rtd_1d), sizeof(wg_gummel_opts), sizeof(wg_gummel_info),
         sizeof(wg_transient_opts), sizeof(wg_transient_info));
  printf("%zu %zu %zu %zu %zu\n", sizeof(wg_server_opts), sizeof(wg_request), sizeof(wg_request_status),
         sizeof(wg_server_stats), sizeof(wg_operator_view));
  printf("%zu %zu %zu\n", offsetof(wg_server_opts, gummel), offsetof(wg_request, rtd),
         offsetof(wg_request_status, t_submit));
  printf("%zu %zu\n", sizeof(wg_runtime_stats), offsetof(wg_runtime_stats, stencil_cells));
  printf("%zu %zu %zu %zu\n", sizeof(wg2d_shape), sizeof(wg2d_solve_opts), offsetof(wg2d_solve_opts, inner_tol),
         sizeof(wg2d_solve_info));
  printf("%zu %zu %zu %zu\n", sizeof(wg_poisson2d_desc), offsetof(wg_poisson2d_desc, temp),
         sizeof(wg_poisson2d_info), offsetof(wg_poisson2d_info, target_integral));
  printf("%zu %zu %zu\n", sizeof(wg2d_observables_desc), offsetof(wg2d_observables_desc, dx_val),
         offsetof(wg2d_observables_desc, n_target_y));
  return 0;
}''')
    exe = tmp_path / "probe"
    r = subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode:
        pytest.skip("no C compiler: " + r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()
    got = list(map(int, out))
    want = [C.sizeof(_lib.WgParams), C.sizeof(_lib.WgDevice), C.sizeof(_lib.WgSolveOpts),
            C.sizeof(_lib.WgSolveInfo), _lib.WgParams.l_xi.offset, _lib.WgParams.precision.offset,
            _lib.WgParams.mem_budget_bytes.offset, _lib.WgSolveInfo.relres.offset, _lib.WgSolveInfo.rhs_norm.offset,
            C.sizeof(_lib.WgRtd1D), C.sizeof(_lib.WgGummelOpts), C.sizeof(_lib.WgGummelInfo),
            C.sizeof(_lib.WgTransientOpts), C.sizeof(_lib.WgTransientInfo),
            C.sizeof(_lib.WgServerOpts), C.sizeof(_lib.WgRequest), C.sizeof(_lib.WgRequestStatus),
            C.sizeof(_lib.WgServerStats), C.sizeof(_lib.WgOperatorView),
            _lib.WgServerOpts.gummel.offset, _lib.WgRequest.rtd.offset, _lib.WgRequestStatus.t_submit.offset,
            C.sizeof(_lib.WgRuntimeStats), _lib.WgRuntimeStats.stencil_cells.offset,
            C.sizeof(_lib.Wg2dShape), C.sizeof(_lib.Wg2dSolveOpts), _lib.Wg2dSolveOpts.inner_tol.offset,
            C.sizeof(_lib.Wg2dSolveInfo),
            C.sizeof(_lib.WgPoisson2dDesc), _lib.WgPoisson2dDesc.temp.offset, C.sizeof(_lib.WgPoisson2dInfo),
            _lib.WgPoisson2dInfo.target_integral.offset,
            C.sizeof(_lib.Wg2dObservablesDesc), _lib.Wg2dObservablesDesc.dx_val.offset,
            _lib.Wg2dObservablesDesc.n_target_y.offset]
    assert got == want


def test_errors_without_handle_are_statuses(built_lib):
    """Argument errors return a status and a message; the library never aborts."""
    from real_space_dg_gb300 import _lib
    lib = _lib.load()
    assert lib.wg_problem_create(None, 1, None) == _lib.WG_ERR_ARG
    assert b"null" in lib.wg_global_error()
    prm = _lib.WgParams(1, 3, 16, 16, 30e-9, 0.0, 1.0, 0, 0, 0.0)    # n_el = 1 is invalid
    h = C.c_void_p()
    assert lib.wg_problem_create(C.byref(prm), 1, C.byref(h)) == _lib.WG_ERR_ARG
    assert b"n_el" in lib.wg_global_error()
    prm = _lib.WgParams(8, 3, 16, 12, 30e-9, 0.0, 1.0, 0, 0, 0.0)    # n_xi < nk
    assert lib.wg_problem_create(C.byref(prm), 1, C.byref(h)) == _lib.WG_ERR_ARG
    prm = _lib.WgParams(8, 3, 16, 16, 30e-9, 0.0, 1.0, 0, 0, 1.0)    # 1-byte budget -> OOM status
    assert lib.wg_problem_create(C.byref(prm), 1, C.byref(h)) == _lib.WG_ERR_OOM
    assert b"budget" in lib.wg_global_error()
    # the bounded-wait diagnostic checks its limit before any CUDA call
    assert lib.wg_debug_wait_timeout(0) == _lib.WG_ERR_ARG
    assert b"spin_limit" in lib.wg_global_error()
