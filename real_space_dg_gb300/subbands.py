"""Transverse subband eigensolve on the GPU: ``[E, V] = solve_subbands(mat)``.

Drop-in for the reference's mode-space set-up (solve_subbands.m:1-40,
solve_bandstructure.m:1-33, eval_transversal_Hamiltonian.m:1-37): for every valley
and x slice the ``n_of_modes`` eigenpairs of smallest magnitude of the Ny x Ny
transverse Hamiltonian (position-dependent mass ``mat.me_y``, potential ``mat.V``,
grid step ``mat.dy`` in nm), ascending, each vector normalised with a positive last
entry, then valley 1's vectors sign-aligned with its first slice.  The results are
the ``Esub`` [nv x Nx x nm] and ``Vsub`` [nv x Nx x nm x Ny] that
``solve_transport_DG_2D`` takes.

All slices are solved at once by ``wg_subbands_*`` in libwigner_gb300.so (Sturm
bisection and twisted-factorisation eigenvectors, one warp per slice).
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import WignerError


class SubbandSolver:
    """A device handle for repeated solves of one shape (n_valleys, Nx, Ny, n_modes), e.g. once
    per Poisson iteration of a self-consistent loop; ``batch`` independent problems (gate or bias
    points) are solved in one launch."""

    def __init__(self, n_valleys, nx, ny, n_modes, batch=1):
        self.lib = _lib.load()
        self.batch = int(batch)
        self.shape = (int(n_valleys), int(nx), int(ny), int(n_modes))
        h = _lib._H()
        rc = self.lib.wg_subbands_create(self.batch, *self.shape, C.byref(h))
        if rc != _lib.WG_OK:
            raise WignerError(rc, "wg_subbands_create failed for batch %d, (nv, Nx, Ny, nm) = %s"
                              % (self.batch, self.shape))
        self.h = h

    def _check(self, rc):
        if rc != _lib.WG_OK:
            raise WignerError(rc, self.lib.wg_subbands_last_error(self.h).decode())

    def solve(self, me_y, V, dy_nm):
        """(E [nv x Nx x nm], Vsub [nv x Nx x nm x Ny]) from host arrays me_y [nv x Nx x Ny]
        and V [Nx x Ny] (eV), dy in nm; with batch > 1 every array gains a leading problem
        axis (me_y [batch x nv x Nx x Ny], or [nv x Nx x Ny] shared by all problems)."""
        nv, nx, ny, nm = self.shape
        b = self.batch
        me = np.asarray(me_y, dtype=float)
        if me.size == nv * nx * ny and b > 1:
            me = np.broadcast_to(me.reshape(1, nv, nx, ny), (b, nv, nx, ny))
        me = np.ascontiguousarray(me.reshape(b, nv, nx, ny))
        pot = np.ascontiguousarray(np.asarray(V, dtype=float).reshape(b, nx, ny))
        E = np.empty((b, nv, nx, nm))
        Vs = np.empty((b, nv, nx, nm, ny))
        self._check(self.lib.wg_subbands_solve(self.h, float(dy_nm), _lib.dptr(me), _lib.dptr(pot), _lib.dptr(E),
                                               _lib.dptr(Vs)))
        return (E[0], Vs[0]) if b == 1 else (E, Vs)

    def solve_device(self, dy_nm, me_y_ptr, V_ptr, E_ptr, Vsub_ptr, stream=None):
        """Enqueue a solve of the whole batch on device pointers (no allocation, no
        synchronisation)."""
        self._check(self.lib.wg_subbands_solve_device(self.h, float(dy_nm), me_y_ptr, V_ptr, E_ptr, Vsub_ptr, stream))

    def status(self, stream=None):
        """Synchronise and raise on a numeric failure of the last device solve."""
        self._check(self.lib.wg_subbands_status(self.h, stream))

    def buffers(self):
        """Device pointers (me_y, V, E, Vsub) of the handle's own buffers."""
        p = [C.c_void_p() for _ in range(4)]
        self._check(self.lib.wg_subbands_buffers(self.h, *[C.byref(x) for x in p]))
        return tuple(x.value for x in p)

    def close(self):
        if getattr(self, "h", None):
            self.lib.wg_subbands_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_subbands(mat):
    """[E, V] = solve_subbands(mat) on the GPU (solve_subbands.m:1-40).  ``mat`` holds
    n_of_modes, n_of_valleys, Nx, Ny, dy (nm), me_y [nv x Nx x Ny] and V [Nx x Ny] (eV)."""
    nv, nx, ny, nm = int(mat["n_of_valleys"]), int(mat["Nx"]), int(mat["Ny"]), int(mat["n_of_modes"])
    with SubbandSolver(nv, nx, ny, nm) as s:
        return s.solve(mat["me_y"], mat["V"], mat["dy"])
