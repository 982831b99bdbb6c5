"""Host-side mirror of the reference's 1D Wigner transport interface.

``solve_transport_DG_2D(mat, Esub, Vsub, EfL, EfR)`` keeps the signature, the
argument meaning and the output fields of the MATLAB function
DG_code/solve_transport_DG_2D.m:1-226 (Xi_solver = 'FV', permute_shell = true).
All numerical work runs in libwigner_gb300.so on the GPU: the host only maps
``mat`` fields to the C ABI, loops over nothing (valleys x modes are one
batch), and weights the density by |Vsub|^2/dy (solve_transport_DG_2D.m:203-212).
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import WignerError

M0 = 9.109e-31  # solve_transport_DG_2D.m:7

PRECISIONS = {"fp64": _lib.WG_PREC_FP64, "plain": _lib.WG_PREC_FP64, "mixed": _lib.WG_PREC_MIXED}


class Problem1D:
    """One handle of `batch` 1D Wigner problems sharing the discretisation shape.

    Mirrors the function-handle seams of the reference: ``apply`` is
    sysInfo.apply (get_SysM_full2D.m:80), ``precondition`` is
    preconditioner.apply (get_LineTransversePreconditioner_full2D.m:113).
    """

    def __init__(self, n_el, n_local, nk, n_xi=None, l_xi=30e-9, batch=1, precision="fp64", restart=50,
                 m_diff=0.0, mpc=1.0, mem_budget_bytes=0.0, inner_restart=0, inner_tol=0.0, reorth=0.0,
                 inner_reorth=0.0, fp64_tc=False, inner_basis_fp32=False):
        self.lib = _lib.load()
        prm = _lib.WgParams(int(n_el), int(n_local), int(nk), int(n_xi or nk), float(l_xi), float(m_diff),
                            float(mpc), PRECISIONS[precision] if isinstance(precision, str) else int(precision),
                            int(restart), float(mem_budget_bytes), int(inner_restart), float(inner_tol),
                            float(reorth), float(inner_reorth), 1 if fp64_tc else 0, 1 if inner_basis_fp32 else 0)
        h = C.c_void_p()
        st = self.lib.wg_problem_create(C.byref(prm), int(batch), C.byref(h))
        if st != _lib.WG_OK:
            raise WignerError(st, self.lib.wg_global_error().decode())
        self.h = h
        self.n_el, self.n_local, self.nk, self.n_xi = int(n_el), int(n_local), int(nk), int(n_xi or nk)
        self.batch = int(batch)
        self.N = self.n_el * self.n_local * self.nk
        self.nx = self.n_el * (self.n_local - 1) + 1
        self.ncol = self.n_el * self.n_local

    # -- lifecycle -------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.wg_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, allow_not_converged=False):
        if st == _lib.WG_OK or (allow_not_converged and st == _lib.WG_NOT_CONVERGED):
            return st
        raise WignerError(st, self.lib.wg_last_error(self.h).decode())

    @property
    def device_bytes(self):
        n = C.c_longlong(); b = C.c_int(); d = C.c_double()
        self._check(self.lib.wg_problem_sizes(self.h, C.byref(n), C.byref(b), C.byref(d)))
        return d.value

    @property
    def runtime_stats(self):
        """CUDA-graph replays and the autotuner's launch shapes (wg_runtime_stats_get)."""
        st = _lib.WgRuntimeStats()
        self._check(self.lib.wg_runtime_stats_get(self.h, C.byref(st)))
        return st.as_dict()

    def set_launch_shapes(self, kline_chunk=0, stencil_cells=0):
        """Pin the k-line chunk length and the FP32 stencil's cells per thread (0 keeps)."""
        self._check(self.lib.wg_set_launch_shapes(self.h, int(kline_chunk), int(stencil_cells)))

    # -- data ------------------------------------------------------------
    def set_potential(self, b, x_nm, esub_ev, m_kg, me_z, temp, ef_l, ef_r):
        x = np.ascontiguousarray(x_nm, dtype=np.float64)
        m = np.ascontiguousarray(np.broadcast_to(np.asarray(m_kg, dtype=np.float64), x.shape))
        e = np.ascontiguousarray(esub_ev, dtype=np.float64)
        if x.size != self.nx or e.size != self.nx:
            raise WignerError(_lib.WG_ERR_ARG, "x_nm and esub_ev need %d entries" % self.nx)
        dev = _lib.WgDevice(int(x.size), _lib.dptr(x), _lib.dptr(m), float(me_z), float(temp))
        self._check(self.lib.wg_set_potential(self.h, int(b), C.byref(dev), _lib.dptr(e), float(ef_l), float(ef_r)))

    def solve(self, tol=1e-10, maxit=50, rho0=None, warm=False):
        """Solve every problem; returns (status, [info dict per problem])."""
        info = (_lib.WgSolveInfo * self.batch)()
        opts = _lib.WgSolveOpts(float(tol), int(maxit), 1 if (warm or rho0 is not None) else 0)
        r0 = None
        if rho0 is not None:
            r0 = _lib.as_c128(rho0).reshape(-1)
            if r0.size != self.N * self.batch:
                raise WignerError(_lib.WG_ERR_ARG, "rho0 needs batch*N entries")
        st = self.lib.wg_solve(self.h, C.byref(opts), r0.view(np.float64).ctypes.data_as(_lib._D) if r0 is not None
                               else None, info)
        self._check(st, allow_not_converged=True)
        return st, [i.as_dict() for i in info]

    def rho(self, b=0):
        out = np.empty(self.N, dtype=np.complex128)
        self._check(self.lib.wg_get_rho(self.h, int(b), out.view(np.float64).ctypes.data_as(_lib._D)))
        return out

    def set_rho(self, b, rho):
        """Overwrite problem b's resident Wigner function (the warm start of the next solve)."""
        r = np.ascontiguousarray(np.asarray(rho, dtype=np.complex128).reshape(-1))
        if r.size != self.N:
            raise WignerError(_lib.WG_ERR_ARG, "rho needs %d entries" % self.N)
        self._check(self.lib.wg_set_rho(self.h, int(b), r.view(np.float64).ctypes.data_as(_lib._D)))

    def set_rhs(self, b, rhs):
        """Overwrite problem b's right-hand side (kept until the next potential update)."""
        r = np.ascontiguousarray(np.asarray(rhs, dtype=np.complex128).reshape(-1))
        if r.size != self.N:
            raise WignerError(_lib.WG_ERR_ARG, "rhs needs %d entries" % self.N)
        self._check(self.lib.wg_set_rhs(self.h, int(b), r.view(np.float64).ctypes.data_as(_lib._D)))

    def rho_xi(self, b=0):
        out = np.empty((self.ncol, self.n_xi), dtype=np.complex128)
        self._check(self.lib.wg_get_rho_xi(self.h, int(b), out.view(np.float64).ctypes.data_as(_lib._D)))
        return out

    def observables(self, b=0):
        n = np.empty(self.ncol); j = np.empty(self.ncol)
        self._check(self.lib.wg_get_observables(self.h, int(b), _lib.dptr(n), _lib.dptr(j)))
        return n, j

    def apply(self, x):
        x = _lib.as_c128(x).reshape(-1)
        y = np.empty_like(x)
        self._check(self.lib.wg_apply(self.h, x.view(np.float64).ctypes.data_as(_lib._D),
                                      y.view(np.float64).ctypes.data_as(_lib._D)))
        return y

    def apply_time(self, which="fp64", n=20):
        """Mean device time [ms] of one operator apply on the resident state: ``fp64``,
        ``lowprec`` (mixed inner operator) or ``fp64_tc`` (mixed FP64 operator)."""
        code = {"fp64": 0, "lowprec": 1, "fp64_tc": 2}[which]
        ms = C.c_double()
        self._check(self.lib.wg_apply_repeat(self.h, code, int(n), C.byref(ms)))
        return ms.value

    def apply_lowprec(self, x):
        """The mixed form's inner operator (BF16 tensor-core transforms, FP32 flux)."""
        x = _lib.as_c128(x).reshape(-1)
        y = np.empty_like(x)
        self._check(self.lib.wg_apply_lowprec(self.h, x.view(np.float64).ctypes.data_as(_lib._D),
                                              y.view(np.float64).ctypes.data_as(_lib._D)))
        return y

    def precondition(self, r):
        r = _lib.as_c128(r).reshape(-1)
        z = np.empty_like(r)
        self._check(self.lib.wg_precondition(self.h, r.view(np.float64).ctypes.data_as(_lib._D),
                                             z.view(np.float64).ctypes.data_as(_lib._D)))
        return z

    def profile(self, on=None, reset=False):
        """Enable/disable kernel timing (on=True/False) and/or read the counters:
        {class: (ms, timed launches, launches, algorithmic bytes, algorithmic flops)}."""
        if on is not None:
            self._check(self.lib.wg_profile_enable(self.h, 1 if on else 0))
        n = len(_lib.PROF_CLASSES)
        ms = np.zeros(n); timed = (C.c_longlong * n)(); launches = (C.c_longlong * n)()
        by = np.zeros(n); fl = np.zeros(n)
        self._check(self.lib.wg_profile_read(self.h, _lib.dptr(ms), timed, launches, _lib.dptr(by), _lib.dptr(fl),
                                             1 if reset else 0))
        return {c: (ms[i], timed[i], launches[i], by[i], fl[i]) for i, c in enumerate(_lib.PROF_CLASSES)}

    def event(self, slot):
        """Record CUDA event `slot` on this handle's stream."""
        self._check(self.lib.wg_event_record(self.h, int(slot)))

    def wait_event(self, other, slot):
        """This handle's stream waits on the device for event `slot` of handle `other`."""
        self._check(self.lib.wg_event_wait(self.h, other.h, int(slot)))

    def elapsed_ms(self, a, b):
        ms = C.c_double()
        self._check(self.lib.wg_event_elapsed(self.h, int(a), int(b), C.byref(ms)))
        return ms.value

    def rhs(self):
        out = np.empty(self.N * self.batch, dtype=np.complex128)
        self._check(self.lib.wg_get_rhs(self.h, out.view(np.float64).ctypes.data_as(_lib._D)))
        return out


def shape_from_mat(mat):
    """Discretisation of mat.dg.params (initParams.m:58-63)."""
    prm = mat["dg"]["params"]
    if str(prm.get("Xi_solver", "FV")).upper() != "FV":
        raise WignerError(_lib.WG_ERR_ARG, "only Xi_solver='FV' is on this path")
    if not prm.get("permute_shell", True):
        raise WignerError(_lib.WG_ERR_ARG, "only permute_shell=true ordering is on this path")
    nK = int(prm["N_K_chi"])
    nx = int(mat["Nx"])
    if (nx - 1) % (nK - 1):
        raise WignerError(_lib.WG_ERR_ARG, "(Nx-1) must be divisible by N_K_chi-1")
    return dict(n_el=(nx - 1) // (nK - 1), n_local=nK, nk=int(prm["N"]), n_xi=int(prm["N_xi"]),
                l_xi=float(prm["Ly"]), m_diff=float(prm.get("m_elektron", 0.0)), mpc=float(prm.get("MPC", 1.0)))


def solve_transport_DG_2D(mat, Esub, Vsub, EfL, EfR, *, tol=1e-10, maxit=50, restart=50, precision="fp64",
                          rho0=None, problem=None, return_info=True):
    """DG = solve_transport_DG_2D(mat, Esub, Vsub, EfL, EfR) on the GPU.

    Esub [nv x Nx x nm] eV, Vsub [nv x Nx x nm x Ny], EfL/EfR eV.  Returns a
    dict with the reference's fields n [Nxdof x Ny], j [Nxdof],
    RHO [nv x nm x Nxdof x N_xi], chi, xi and, for st_init, rhs and rho per mode;
    ``info`` carries the solver status per (valley, mode) in the form of
    DG.info.solve (flag, relres, iterations, ...).  The iterative solve replaces
    the reference's direct ``rho = A\\rhs`` (solve_transport_DG_2D.m:101); tol is
    the relative residual target.
    """
    nv, nm = int(mat["n_of_valleys"]), int(mat["n_of_modes"])
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    Esub = np.asarray(Esub, dtype=float).reshape(nv, nx, nm)
    Vsub = np.asarray(Vsub, dtype=float).reshape(nv, nx, nm, ny)
    me_x = np.asarray(mat["me_x"], dtype=float).reshape(nv, nx, ny)
    mid = int(np.ceil(ny / 2)) - 1
    shp = shape_from_mat(mat)
    own = problem is None
    P = problem or Problem1D(batch=nv * nm, precision=precision, restart=restart, **shp)
    x_nm = np.asarray(mat["x"], dtype=float)
    try:
        for iv in range(nv):
            m = me_x[iv, :, mid] * M0
            for im in range(nm):
                P.set_potential(iv * nm + im, x_nm, Esub[iv, :, im], m, float(mat["me_z_ch"]), float(mat["Temp"]),
                                EfL, EfR)
        status, info = P.solve(tol=tol, maxit=maxit, rho0=rho0)
        n_el, nK = shp["n_el"], shp["n_local"]
        node = (np.arange(n_el)[:, None] * (nK - 1) + np.arange(nK)[None, :]).ravel()
        nT = np.zeros((n_el * nK, ny))
        jT = np.zeros(n_el * nK)
        RHO = np.zeros((nv, nm, n_el * nK, shp["n_xi"]), dtype=complex)
        rhos = []
        for iv in range(nv):
            for im in range(nm):
                b = iv * nm + im
                n_dg, j = P.observables(b)
                vs = Vsub[iv, :, im, :][node]
                nT += n_dg[:, None] * np.abs(vs) ** 2 / float(mat["dy"]) / 1e-9
                jT += j
                RHO[iv, im] = P.rho_xi(b)
                if mat["dg"]["params"].get("st_init", False) or rho0 is not None:
                    rhos.append(P.rho(b))
        dx = (float(mat["L_x"]) * 1e-9) / n_el
        chi = np.concatenate([np.linspace(e * dx, (e + 1) * dx, nK) for e in range(n_el)])
        lxi = shp["l_xi"]
        dxi = lxi / (shp["n_xi"] - 1)
        xi = np.linspace(-(lxi - dxi) / 2, (lxi - dxi) / 2, shp["n_xi"])
        DG = {"n": nT, "j": jT, "RHO": RHO, "chi": chi, "xi": xi, "status": status}
        if return_info:
            DG["info"] = info
        if mat["dg"]["params"].get("st_init", False):
            DG["rho"] = rhos
            DG["rhs"] = P.rhs().reshape(nv * nm, -1)
        return DG
    finally:
        if own:
            P.close()
