"""ctypes binding of libwigner_gb300.so (the C ABI of include/wigner_gb300.h).

The library is built in-tree by real_space_dg_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback for the product path.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwigner_gb300.so")

WG_OK, WG_NOT_CONVERGED, WG_ERR_ARG, WG_ERR_OOM, WG_ERR_TIMEOUT, WG_ERR_CUDA, WG_ERR_NUMERIC = range(7)
WG_PREC_FP64, WG_PREC_MIXED = 0, 1
STATUS_NAMES = {0: "WG_OK", 1: "WG_NOT_CONVERGED", 2: "WG_ERR_ARG", 3: "WG_ERR_OOM", 4: "WG_ERR_TIMEOUT",
                5: "WG_ERR_CUDA", 6: "WG_ERR_NUMERIC"}
# Error identifiers of the reference (DG:Full2D:*), by status.
ERROR_IDS = {WG_ERR_ARG: "DG:Full2D:InvalidArgument", WG_ERR_OOM: "DG:Full2D:GmresMemoryLimit",
             WG_ERR_TIMEOUT: "DG:Full2D:Timeout", WG_ERR_CUDA: "DG:Full2D:CUDA",
             WG_ERR_NUMERIC: "DG:Full2D:NonFinite"}


class WgParams(C.Structure):
    _fields_ = [("n_el", C.c_int), ("n_local", C.c_int), ("nk", C.c_int), ("n_xi", C.c_int),
                ("l_xi", C.c_double), ("m_diff", C.c_double), ("mpc", C.c_double), ("precision", C.c_int),
                ("restart", C.c_int), ("mem_budget_bytes", C.c_double), ("inner_restart", C.c_int),
                ("inner_tol", C.c_double), ("reorth", C.c_double), ("inner_reorth", C.c_double),
                ("fp64_tc", C.c_int), ("inner_basis_fp32", C.c_int)]


class WgDevice(C.Structure):
    _fields_ = [("nx", C.c_int), ("x_nm", C.POINTER(C.c_double)), ("m_kg", C.POINTER(C.c_double)),
                ("me_z", C.c_double), ("temp", C.c_double)]


class WgOperatorView(C.Structure):
    _fields_ = [("n_el", C.c_int), ("n_local", C.c_int), ("nk", C.c_int), ("n_xi", C.c_int), ("batch", C.c_int),
                ("phi", C.c_void_p), ("kvec", C.c_void_p), ("qd", C.c_void_p), ("beta", C.c_void_p),
                ("betai", C.c_void_p), ("K1", C.c_double * 16), ("K2", C.c_double * 16), ("K3", C.c_double * 16),
                ("K5", C.c_double * 16)]


class WgSolveOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("maxit", C.c_int), ("use_rho0", C.c_int)]


class WgRtd1D(C.Structure):
    _fields_ = [("vc_ev", C.POINTER(C.c_double)), ("nd_m3", C.POINTER(C.c_double)), ("eps_r", C.POINTER(C.c_double)),
                ("phi0", C.POINTER(C.c_double)), ("bias", C.c_double), ("ef_offset", C.c_double),
                ("dy_nm", C.c_double)]


class WgGummelOpts(C.Structure):
    _fields_ = [("max_iterations", C.c_int), ("mixing", C.c_double), ("potential_tol", C.c_double),
                ("density_tol", C.c_double), ("poisson_residual_tol", C.c_double), ("transport_tol", C.c_double),
                ("transport_maxit", C.c_int), ("warm_start", C.c_int), ("restart_from_phi0", C.c_int),
                ("inexact_factor", C.c_double), ("inexact_cap", C.c_double), ("defer_final", C.c_int)]


class WgGummelInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("gmres_iterations", C.c_int),
                ("potential_defect", C.c_double), ("density_change", C.c_double), ("poisson_relres", C.c_double),
                ("transport_relres", C.c_double), ("seconds", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


GUMMEL_STATUS = {0: "fixed-point-converged", 1: "iteration-limit", 2: "transport-not-converged",
                 3: "poisson-not-converged"}


class WgTransientOpts(C.Structure):
    _fields_ = [("dt", C.c_double), ("nsteps", C.c_int), ("method", C.c_int), ("scale_a", C.c_double),
                ("scale_rhs", C.c_double), ("refresh_every", C.c_int), ("refresh_first", C.c_int),
                ("tol", C.c_double), ("maxit", C.c_int), ("record_every", C.c_int), ("fixed_rhs", C.c_int)]


class WgTransientInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("steps", C.c_int), ("gmres_iterations", C.c_longlong),
                ("max_relres", C.c_double), ("refreshes", C.c_int), ("poisson_solves", C.c_int),
                ("seconds", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


TRANSIENT_METHODS = {"cn": 0, "rk4": 1}


class WgServerOpts(C.Structure):
    _fields_ = [("mem_budget_bytes", C.c_double), ("max_slots", C.c_int), ("precision", C.c_int),
                ("restart", C.c_int), ("inner_restart", C.c_int), ("inner_tol", C.c_double),
                ("reorth", C.c_double), ("inner_reorth", C.c_double), ("gummel", WgGummelOpts), ("warm_start", C.c_int), ("idle_release_s", C.c_double)]


class WgRequest(C.Structure):
    _fields_ = [("n_el", C.c_int), ("n_local", C.c_int), ("nk", C.c_int), ("n_xi", C.c_int), ("l_xi", C.c_double),
                ("m_diff", C.c_double), ("mpc", C.c_double), ("dev", WgDevice), ("rtd", WgRtd1D),
                ("device_key", C.c_longlong)]


class WgRequestStatus(C.Structure):
    _fields_ = [("state", C.c_int), ("info", WgGummelInfo), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("handle", C.c_int), ("slot", C.c_int), ("warm", C.c_int),
                ("error", C.c_char * 192)]


class WgServerStats(C.Structure):
    _fields_ = [("handles", C.c_int), ("queued", C.c_int), ("running", C.c_int), ("done", C.c_longlong),
                ("failed", C.c_longlong), ("device_bytes", C.c_double), ("device_bytes_peak", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class WgRuntimeStats(C.Structure):
    _fields_ = [("graph_replays", C.c_longlong), ("graphs_captured", C.c_int), ("graphs_disabled", C.c_int),
                ("tuned", C.c_int), ("kline_chunk", C.c_int), ("stencil_cells", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Wg2dShape(C.Structure):
    _fields_ = [("n_el_x", C.c_int), ("nk_x", C.c_int), ("n_el_y", C.c_int), ("nk_y", C.c_int),
                ("n_rho_x", C.c_int), ("n_rho_y", C.c_int), ("periodic_y", C.c_int), ("n_quad", C.c_int),
                ("tensor_cores", C.c_int)]


class Wg2dSolveOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("maxit", C.c_int), ("restart", C.c_int), ("use_x0", C.c_int),
                ("mixed", C.c_int), ("inner_tol", C.c_double), ("inner_basis_fp16", C.c_int)]


class Wg2dObservablesDesc(C.Structure):
    _fields_ = [("n_zero_x", C.c_int), ("n_zero_y", C.c_int), ("zero_x", C.c_int * 2), ("zero_y", C.c_int * 2),
                ("w_zero_x", C.c_double * 2), ("w_zero_y", C.c_double * 2), ("n_dx", C.c_int), ("n_dy", C.c_int),
                ("dx_idx", C.c_int * 8), ("dy_idx", C.c_int * 8), ("dx_val", C.c_double * 8),
                ("dy_val", C.c_double * 8), ("scale_x", C.c_double), ("scale_y", C.c_double),
                ("n_target_y", C.c_int)]


class Wg2dSolveInfo(C.Structure):
    _fields_ = [("flag", C.c_int), ("iterations", C.c_int), ("cycles", C.c_int), ("relres", C.c_double),
                ("initial_relres", C.c_double), ("rhs_norm", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


REQUEST_STATES = {0: "queued", 1: "running", 2: "done", 3: "failed"}


class WgSolveInfo(C.Structure):
    _fields_ = [("flag", C.c_int), ("iterations", C.c_int), ("cycles", C.c_int), ("refinements", C.c_int),
                ("relres", C.c_double), ("initial_relres", C.c_double), ("rhs_norm", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# Every symbol the header declares, with its ctypes signature.
class WgPoisson2dDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dx_nm", C.c_double), ("dy_nm", C.c_double),
                ("periodic_y", C.c_int), ("neumann_x", C.c_int), ("temp", C.c_double), ("batch", C.c_int)]


class WgPoisson2dInfo(C.Structure):
    _fields_ = [("converged", C.c_int), ("linear_relres", C.c_double), ("physical_relres_before", C.c_double),
                ("physical_relres_after", C.c_double), ("physical_residual_before", C.c_double),
                ("residual_scale", C.c_double), ("unmixed_step", C.c_double), ("iter_err", C.c_double),
                ("net_charge_per_length", C.c_double), ("relative_charge_imbalance", C.c_double),
                ("source_integral", C.c_double), ("target_integral", C.c_double)]


_H = C.c_void_p
_D = C.POINTER(C.c_double)
SIGNATURES = {
    "wg_debug_wait_timeout": ([C.c_longlong], C.c_int),
    "wg_problem_create": ([C.POINTER(WgParams), C.c_int, C.POINTER(_H)], C.c_int),
    "wg_problem_destroy": ([_H], C.c_int),
    "wg_problem_bytes": ([C.POINTER(WgParams), C.c_int, _D], C.c_int),
    "wg_last_error": ([_H], C.c_char_p),
    "wg_global_error": ([], C.c_char_p),
    "wg_problem_sizes": ([_H, C.POINTER(C.c_longlong), C.POINTER(C.c_int), _D], C.c_int),
    "wg_runtime_stats_get": ([_H, C.POINTER(WgRuntimeStats)], C.c_int),
    "wg_set_launch_shapes": ([_H, C.c_int, C.c_int], C.c_int),
    "wg2d_create": ([C.POINTER(Wg2dShape), C.POINTER(_H)], C.c_int),
    "wg2d_destroy": ([_H], C.c_int),
    "wg2d_last_error": ([_H], C.c_char_p),
    "wg2d_set_transport": ([_H, C.c_int, C.c_int, _D, _D, C.POINTER(C.c_int), C.POINTER(C.c_int), _D], C.c_int),
    "wg2d_set_drift": ([_H, _D, _D, _D, _D, _D, _D, _D, C.c_double, _D], C.c_int),
    "wg2d_set_potential": ([_H, C.c_int, C.c_int, _D, _D, _D], C.c_int),
    "wg2d_set_hard_wall": ([_H, C.c_void_p, _D, C.c_double], C.c_int),
    "wg2d_set_transport_masks": ([_H, C.c_int, C.c_int, C.c_void_p], C.c_int),
    "wg2d_apply": ([_H, _D, _D], C.c_int),
    "wg2d_apply_repeat": ([_H, C.c_int, _D, _D], C.c_int),
    "wg2d_set_preconditioner": ([_H, _D, C.c_double, _D, _D, C.POINTER(C.c_int), _D, C.c_int], C.c_int),
    "wg2d_precondition": ([_H, _D, _D], C.c_int),
    "wg2d_solve": ([_H, _D, _D, C.POINTER(Wg2dSolveOpts), C.POINTER(Wg2dSolveInfo)], C.c_int),
    "wg2d_get_state": ([_H, _D], C.c_int),
    "wg2d_solve_bicgstab": ([_H, _D, _D, C.POINTER(Wg2dSolveOpts), C.POINTER(Wg2dSolveInfo)], C.c_int),
    "wg2d_solve_resvec": ([_H, _D, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "wg2d_set_observables": ([_H, C.POINTER(Wg2dObservablesDesc), _D, _D], C.c_int),
    "wg2d_observables": ([_H, _D, _D, _D, _D, _D, _D, _D, _D], C.c_int),
    "wg_poisson2d_create": ([C.POINTER(WgPoisson2dDesc), _D, C.POINTER(C.c_ubyte), _D, _D, C.POINTER(_H)], C.c_int),
    "wg_poisson2d_destroy": ([_H], C.c_int),
    "wg_poisson2d_last_error": ([_H], C.c_char_p),
    "wg_poisson2d_set_projection": ([_H, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), _D, C.c_int,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), _D, _D, _D, _D, _D], C.c_int),
    "wg_poisson2d_apply": ([_H, _D, _D], C.c_int),
    "wg_poisson2d_solve": ([_H, _D, C.c_int, _D, _D, _D, C.c_int, C.c_double, _D, _D,
                            C.POINTER(WgPoisson2dInfo)], C.c_int),
    "wg_poisson2d_contacts": ([_H, _D, _D, _D], C.c_int),
    "wg_poisson2d_solve_device": ([_H, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                   C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "wg_poisson2d_info_get": ([_H, C.c_void_p, C.POINTER(WgPoisson2dInfo)], C.c_int),
    "wg_poisson2d_buffers": ([_H] + [C.POINTER(C.c_void_p)] * 5, C.c_int),
    "wg_subbands_create": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(_H)], C.c_int),
    "wg_subbands_destroy": ([_H], C.c_int),
    "wg_subbands_last_error": ([_H], C.c_char_p),
    "wg_subbands_solve": ([_H, C.c_double, _D, _D, _D, _D], C.c_int),
    "wg_subbands_solve_device": ([_H, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
                                 C.c_int),
    "wg_subbands_status": ([_H, C.c_void_p], C.c_int),
    "wg_subbands_buffers": ([_H, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                             C.POINTER(C.c_void_p)], C.c_int),
    "wg_set_potential": ([_H, C.c_int, C.POINTER(WgDevice), _D, C.c_double, C.c_double], C.c_int),
    "wg_solve": ([_H, C.POINTER(WgSolveOpts), _D, C.POINTER(WgSolveInfo)], C.c_int),
    "wg_get_rho": ([_H, C.c_int, _D], C.c_int),
    "wg_set_rho": ([_H, C.c_int, _D], C.c_int),
    "wg_set_rhs": ([_H, C.c_int, _D], C.c_int),
    "wg_get_observables": ([_H, C.c_int, _D, _D], C.c_int),
    "wg_get_rho_xi": ([_H, C.c_int, _D], C.c_int),
    "wg_apply": ([_H, _D, _D], C.c_int),
    "wg_apply_lowprec": ([_H, _D, _D], C.c_int),
    "wg_precondition": ([_H, _D, _D], C.c_int),
    "wg_get_rhs": ([_H, _D], C.c_int),
    "wg_gummel_set": ([_H, C.c_int, C.POINTER(WgDevice), C.POINTER(WgRtd1D)], C.c_int),
    "wg_gummel_run": ([_H, C.POINTER(WgGummelOpts), C.POINTER(WgGummelInfo)], C.c_int),
    "wg_gummel_get": ([_H, C.c_int, _D, _D, _D], C.c_int),
    "wg_transient_set_bias": ([_H, C.c_int, C.c_double], C.c_int),
    "wg_transient_run": ([_H, C.POINTER(WgTransientOpts), _D, _D, C.POINTER(WgTransientInfo)], C.c_int),
    "wg_server_create": ([C.POINTER(WgServerOpts), C.POINTER(_H)], C.c_int),
    "wg_server_submit": ([_H, C.POINTER(WgRequest), C.POINTER(C.c_longlong)], C.c_int),
    "wg_server_wait": ([_H, C.c_longlong, C.c_double, C.POINTER(WgRequestStatus)], C.c_int),
    "wg_server_result": ([_H, C.c_longlong, _D, _D, _D], C.c_int),
    "wg_server_release": ([_H, C.c_longlong], C.c_int),
    "wg_server_stats_get": ([_H, C.POINTER(WgServerStats)], C.c_int),
    "wg_server_destroy": ([_H], C.c_int),
    "wg_apply_noalloc": ([C.POINTER(WgOperatorView), C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "wg_debug_gemm_bf16": ([C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int,
                            C.c_int], C.c_int),
    "wg_debug_gemm_f64_tc": ([_D, _D, _D, C.c_int, C.c_int, C.c_int], C.c_int),
    "wg_debug_gemm_f64_tc_digits": ([_D, _D, _D, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
    "wg_apply_repeat": ([_H, C.c_int, C.c_int, _D], C.c_int),
    "wg_event_record": ([_H, C.c_int], C.c_int),
    "wg_event_elapsed": ([_H, C.c_int, C.c_int, _D], C.c_int),
    "wg_event_wait": ([_H, _H, C.c_int], C.c_int),
    "wg_profile_enable": ([_H, C.c_int], C.c_int),
    "wg_profile_read": ([_H, _D, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), _D, _D, C.c_int], C.c_int),
}
PROF_CLASSES = ["flux", "gemm_f64", "gemm_bf16", "stencil", "precond", "multidot", "gs_update", "krylov_small", "other",
                "gemm_f64_tc", "flux_f64", "stencil_f64", "gemm_stencil", "gemm_flux"]

_lib = None


class WignerError(RuntimeError):
    """Raised for every non-OK status except WG_NOT_CONVERGED (which is a status)."""

    def __init__(self, status, message, identifier=None):
        self.status = status
        self.identifier = identifier or ERROR_IDS.get(status, "DG:Full2D:Error")
        super().__init__("%s (%s): %s" % (self.identifier, STATUS_NAMES.get(status, status), message))


def load(path=LIB_PATH):
    """Load the library and bind every declared symbol (no GPU call is made)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libwigner_gb300.so is not built (%s); run real_space_dg_gb300.build.build() "
                          "or __graft_entry__.build(). There is no CPU fallback." % path)
    lib = C.CDLL(path)
    for name, (argtypes, restype) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = restype
    _lib = lib
    return lib


def dptr(a):
    return a.ctypes.data_as(_D)


def as_c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)
