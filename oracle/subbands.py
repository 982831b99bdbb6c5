"""Transverse subband eigensolve in mode space (oracle; test infrastructure only).

Restates, in NumPy, the reference's per-slice transverse eigenproblem that supplies
the subband energies Esub and mode functions Vsub of the mode-space transport:

  eval_transversal_Hamiltonian.m:1-37   the Ny x Ny finite-difference Hamiltonian of one
                                        x slice and valley (position-dependent mass,
                                        harmonic-mean hopping, copied end rows)
  solve_bandstructure.m:1-33            the n_of_modes eigenpairs of smallest magnitude
                                        (eigs 'sm'), ascending, real parts, each vector
                                        2-norm normalised with the sign of its last entry
  solve_subbands.m:1-40                 the loop over slices and valleys, then the sign
                                        clean-up of valley 1 against its first slice

The eigenpairs come from a dense eigensolve of the literal (non-symmetric) matrix, so
the restatement needs no assumption about its structure.  Parity of the CUDA solver is
pinned against closed-form spectra (uniform mass and potential: the discrete box) and
against this restatement on seeded devices.
"""
import numpy as np

H_PLANCK = 6.626e-34
M0 = 9.109e-31
Q = 1.602e-19


def hopping_scale(dy_nm):
    """t0 = hbar^2 / (2 m0 dy^2 q 1e-18) in eV for dy in nm (eval_transversal_Hamiltonian.m:3-20)."""
    hb = H_PLANCK / 2 / np.pi
    return hb ** 2 / 2 / (M0 * dy_nm ** 2 * Q * 1e-18)


def transversal_hamiltonian(m_eff, V, dy_nm):
    """Dense Ht of one slice (eval_transversal_Hamiltonian.m:20-37): rows 2..Ny-1 carry
    -2 t0 / (m_{i-1} + m_i) and -2 t0 / (m_{i+1} + m_i) off the diagonal and minus their
    sum plus V_i on it; row 1 copies row 2's diagonal and upper entry, row Ny copies row
    Ny-1's diagonal and lower entry (MATLAB 1-based rows)."""
    m = np.asarray(m_eff, dtype=float)
    V = np.asarray(V, dtype=float)
    ny = m.size
    t0 = hopping_scale(dy_nm)
    H = np.zeros((ny, ny))
    for i in range(1, ny - 1):
        H[i, i - 1] = -2 * t0 / (m[i - 1] + m[i])
        H[i, i + 1] = -2 * t0 / (m[i + 1] + m[i])
        H[i, i] = -(H[i, i - 1] + H[i, i + 1]) + V[i]
    H[0, 0] = H[1, 1]
    H[0, 1] = H[1, 2]
    H[ny - 1, ny - 1] = H[ny - 2, ny - 2]
    H[ny - 1, ny - 2] = H[ny - 2, ny - 3]
    return H


def solve_bandstructure(m_eff, V, dy_nm, n_modes):
    """(E [n_modes], V [n_modes x Ny]) of one slice (solve_bandstructure.m:17-33)."""
    H = transversal_hamiltonian(m_eff, V, dy_nm)
    w, vr = np.linalg.eig(H)
    pick = np.argsort(np.abs(w), kind="stable")[:n_modes]       # eigs(Ht, n, 'sm')
    w, vr = w[pick], vr[:, pick]
    order = np.argsort(w.real, kind="stable")
    E = w[order].real
    vecs = np.real(vr[:, order])
    for k in range(n_modes):
        v = vecs[:, k]
        vecs[:, k] = np.sign(v[-1]) * v / np.sqrt(np.sum(v ** 2))
    return E, vecs.T


def solve_subbands(mat):
    """(E [nv x Nx x nm], V [nv x Nx x nm x Ny]) (solve_subbands.m:1-40).  ``mat`` holds
    n_of_modes, n_of_valleys, Nx, Ny, dy (nm), me_y [nv x Nx x Ny] and V [Nx x Ny] (eV)."""
    nm, nv = int(mat["n_of_modes"]), int(mat["n_of_valleys"])
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    me_y = np.asarray(mat["me_y"], dtype=float).reshape(nv, nx, ny)
    pot = np.asarray(mat["V"], dtype=float).reshape(nx, ny)
    E = np.zeros((nv, nx, nm))
    Vs = np.zeros((nv, nx, nm, ny))
    for ix in range(nx):
        for iv in range(nv):
            E[iv, ix], Vs[iv, ix] = solve_bandstructure(me_y[iv, ix], pot[ix], float(mat["dy"]), nm)
    return E, cleanup_signs(Vs)


def cleanup_signs(Vs, cutoff=0.5):
    """Flip valley 1's mode vectors whose overlap with the same mode of slice 1 is below
    -cutoff (solve_subbands.m:22-40); slice 1 itself is never flipped."""
    Vs = Vs.copy()
    for m in range(Vs.shape[2]):
        v0 = Vs[0, 0, m].copy()
        for ix in range(1, Vs.shape[1]):
            if np.sum(v0 * Vs[0, ix, m]) < -cutoff:
                Vs[0, ix, m] = -Vs[0, ix, m]
    return Vs


def box_spectrum(ny, m_eff, dy_nm, V0, n_modes):
    """Closed form for uniform mass m and potential V0: Ht is then the symmetric
    tridiagonal (2 t, -t) with t = t0 / m plus V0 (the copied end rows equal the interior
    ones), so E_k = V0 + 2 t (1 - cos(k pi / (Ny + 1))) and v_k(i) ~ sin(k pi i / (Ny + 1))."""
    t = hopping_scale(dy_nm) / m_eff
    k = np.arange(1, n_modes + 1)
    E = V0 + 2 * t * (1 - np.cos(k * np.pi / (ny + 1)))
    i = np.arange(1, ny + 1)
    vec = np.sin(np.outer(k, i) * np.pi / (ny + 1))
    vec /= np.linalg.norm(vec, axis=1, keepdims=True)
    vec *= np.sign(vec[:, -1:])
    return E, vec
