"""Full-2D contact reservoirs and the Source/Drain inflow right-hand side (host set-up).

Drop-in for the reservoir data of the reference's Full-2D solve, computed once per bias on the
host (a few MFLOP: five contact modes x 160 k_x x 201 k_z) and handed to the device solve as
its right-hand side:

  get_InflowBoundary_full2D(mat, f, EfL, EfR, Vxy)   DG_code/core/get_InflowBoundary_full2D.m:1-56
      'contact-modes' (the recorded run's model): get_ContactModeReservoirRho_full2D.m on a
      periodic Y cell (Fourier-Galerkin contact modes, get_PeriodicContactModes_full2D.m),
      contact-neutrality Fermi level from the k_z-integrated sheet density, the density matrix
      phi_n(Y + rho_y/2) conj(phi_n(Y - rho_y/2)) F_n(rho_x);
      'material-default': get_DefaultReservoirRho_full2D.m (separable (k_x, k_y) Fermi
      distribution of the contact edge, cosine-transformed)
  inflow_rhs(f, inflow)                               get_Diff_full2D.m:405-430, :609-615

``f`` is ``full2d.build_factors(mat)``.  Contact modes: the Fourier-Galerkin modes of a periodic Y
cell, or the box contact problem (get_ContactModeReservoirRho_full2D.m:153-302) for the other Y
boundaries, with constant masses.  Contacts on part of an X face keep their data on the contact
pieces only (the operator closes the rest).
"""
import numpy as np

from . import _lib
from ._lib import WignerError

HBAR = 1.054571817e-34
QE = 1.602176634e-19
KB_RES = 1.38064852e-23      # Boltzmann constant of the reference's reservoir files
M0 = 9.1093837015e-31


def _p(prm, name, default):
    v = prm.get(name)
    if v is None and isinstance(prm.get("full2D"), dict):
        v = prm["full2D"].get(name)
    return default if v is None else v


def _k_grid(nk, length):
    nk = max(2, int(round(nk)))
    k = (2 * np.pi / length) * (0.5 * (nk + 1) - np.arange(1, nk + 1))
    return k, abs(k[1] - k[0])


def _rel_mass(mat, axis):
    m = mat.get("me_%s_ch" % axis, mat.get("me_x_ch", 0.041))
    m = float(m) / M0 if m < 1e-25 else float(m)
    if not (m > 0 and np.isfinite(m)):
        raise WignerError(_lib.WG_ERR_ARG, "DG:Full2D:PeriodicContactMass: masses must be positive scalars")
    return m


def _softplus(eta):
    return np.where(eta > 40, eta, np.where(eta < -40, np.exp(np.minimum(eta, 0.0)),
                                            np.log1p(np.exp(np.clip(eta, -40, 40)))))


def _edge(mat, Vxy, side):
    ix = int(mat["Nx"]) - 1 if side == "drain" else 0
    return np.asarray(Vxy, dtype=float).reshape(int(mat["Nx"]), int(mat["Ny"]))[ix]


def _periodic_modes(mat, f, side, Vxy):
    prm = mat["dg"]["params"]
    y = f["y"]
    gy = np.asarray(mat["y"], dtype=float) * f["scale"]
    width = y[-1] - y[0]
    nu = gy.size - 1
    if nu < 2 or np.abs(np.diff(gy) - width / nu).max() > 1e-10 * width / nu:
        raise WignerError(_lib.WG_ERR_ARG, "DG:Full2D:PeriodicContactGrid: uniform material Y grid required")
    kmax = min((nu - 1) // 2, (f["rel"][1]["n"] - 2) // 4)
    order = _p(prm, "full2D_periodicModeOrder", kmax)
    if order != int(order) or not (0 <= order <= kmax):
        raise WignerError(_lib.WG_ERR_ARG, "DG:Full2D:PeriodicModeOrder: integer in 0..%d" % kmax)
    v = _edge(mat, Vxy, side)
    if abs(v[0] - v[-1]) > 1e-10 * max(1.0, np.abs(v).max()):
        raise WignerError(_lib.WG_ERR_ARG, "DG:Full2D:NonperiodicPotential: contact potential endpoints must agree")
    my = _rel_mass(mat, "y")
    kw = (2 * np.pi / width) * np.arange(-int(order), int(order) + 1)
    kin = HBAR ** 2 * kw ** 2 / (2 * my * M0 * QE)
    if np.abs(v - v[0]).max() < 1e-13 * max(1.0, abs(v[0])):
        ids = np.argsort(v[0] + kin, kind="stable")
        return (v[0] + kin)[ids], np.eye(kw.size)[:, ids], kw, gy, width
    E = np.exp(1j * np.outer(gy[:-1] - gy[0], kw)) / np.sqrt(width)
    H = np.diag(kin) + (width / nu) * (E.conj().T @ (v[:-1, None] * E))
    w, c = np.linalg.eigh(0.5 * (H + H.conj().T))
    ids = np.argsort(w, kind="stable")
    return w[ids], c[:, ids], kw, gy, width


def _sheet(ef, E, mx, mz, temp, deg):
    kbt = KB_RES * temp
    return float(np.sum(deg * np.sqrt(mx * mz) * kbt / (np.pi * HBAR ** 2) * _softplus(QE * (ef - E) / kbt)))


def _neutral_fermi(E, mx, mz, target, temp, deg, prm, guess):
    tol = _p(prm, "full2D_contactModeFermiTolerance", 1e-10)
    maxit = int(_p(prm, "full2D_contactModeFermiMaxIterations", 200))
    ktev = KB_RES * temp / QE
    step = max(0.5, 20 * ktev)
    lo, hi = E.min() - max(2, 80 * ktev), E.min() + max(2, 80 * ktev)
    if np.isfinite(guess):
        lo, hi = min(lo, guess - step), max(hi, guess + step)
    nlo, nhi = _sheet(lo, E, mx, mz, temp, deg), _sheet(hi, E, mx, mz, temp, deg)
    for _ in range(50):
        if nlo <= target <= nhi:
            break
        step *= 2
        if nlo > target:
            lo -= step
            nlo = _sheet(lo, E, mx, mz, temp, deg)
        if nhi < target:
            hi += step
            nhi = _sheet(hi, E, mx, mz, temp, deg)
    if not nlo <= target <= nhi:
        raise WignerError(_lib.WG_ERR_NUMERIC, "DG:Full2D:ContactFermiBracketFailed for %g m^-2" % target)
    for _ in range(maxit):
        mid = 0.5 * (lo + hi)
        nm_ = _sheet(mid, E, mx, mz, temp, deg)
        if abs(nm_ - target) / target <= tol:
            return mid
        if nm_ < target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def _box_modes(mat, f, side, Vxy):
    """The transverse contact problem of a non-periodic Y face (get_ContactModeReservoirRho_full2D.m:
    153-302): H on the sorted material Y grid of the contact column, three-point interior rows with
    the harmonic-mean mass, boundary rows repeating their neighbour's diagonal and outer coupling
    (the mode vanishes one step beyond the grid), or with hard walls the interior unknowns alone (it
    vanishes at the walls); the n modes of smallest |E| in ascending order, unit trapezoid norm over
    y, last grid value nonnegative.  Returns (E, modes [nY x n], grid, hard)."""
    for key in ("me_x", "me_y", "me_z"):
        if mat.get(key) is not None and np.size(mat[key]) > 1:
            raise WignerError(_lib.WG_ERR_ARG, "position-dependent contact masses (the variable-mass model) are "
                              "not built", "DG:Full2D:ContactModeMass")
    prm = mat["dg"]["params"]
    raw = np.asarray(mat["y"], dtype=float) * f["scale"]
    order = np.argsort(raw, kind="stable")
    grid = raw[order]
    n = grid.size
    if n < 3:
        raise WignerError(_lib.WG_ERR_ARG, "Contact-mode reservoir needs at least three Y grid points.",
                          "DG:Full2D:ContactModeGridTooSmall")
    v = _edge(mat, Vxy, side)[order]
    my = _rel_mass(mat, "y")
    t0 = HBAR ** 2 / (2 * M0 * QE * np.mean(np.diff(grid)) ** 2)
    off = -2 * t0 / (2 * my)                       # -2 t0 / (m_i + m_j), constant mass
    diag = np.empty(n)
    diag[1:-1] = -2 * off + v[1:-1]
    diag[0], diag[-1] = diag[1], diag[-2]
    H = np.diag(diag) + np.diag(np.full(n - 1, off), 1) + np.diag(np.full(n - 1, off), -1)
    hard = f.get("ytype") == "hard-wall"
    lo, hi = 0, n
    if hard:
        if max(abs(grid[0] - f["y"][0]), abs(grid[-1] - f["y"][-1])) > 64 * np.spacing(np.abs(grid).max()):
            raise WignerError(_lib.WG_ERR_ARG, "Hard-wall contact modes require the material and DG Y bounds to "
                              "agree.", "DG:Full2D:HardWallContactDomainMismatch")
        lo, hi = 1, n - 1
    Hs = H[lo:hi, lo:hi]
    ng = Hs.shape[0]
    nm = int(mat["n_of_modes"]) if mat.get("n_of_modes") is not None else min(4, ng - 1)
    nm = max(1, min(int(round(_p(prm, "full2D_contactModeCount", nm))), ng))
    w, vec = np.linalg.eigh(Hs)                  # constant mass: H is symmetric
    if nm < ng:
        pick = np.sort(np.argsort(np.abs(w), kind="stable")[:nm])
        w, vec = w[pick], vec[:, pick]
    modes = np.zeros((n, nm))
    modes[lo:hi] = vec[:, :nm]
    wts = np.concatenate([[0.0], 0.5 * np.diff(grid)]) + np.concatenate([0.5 * np.diff(grid), [0.0]])
    modes /= np.sqrt(wts @ modes ** 2)[None, :]
    modes *= np.where(modes[-1] < 0, -1.0, 1.0)[None, :]
    return w[:nm], modes, grid, hard


def _box_density(modes, grid, hard, yn, rho_y):
    """phi_n(Y + rho_y/2) phi_n(Y - rho_y/2) [rho_y, node, mode], linear between the grid values and
    zero beyond (transverseModeDensity, :343-367)."""
    if not hard:
        d = np.mean(np.diff(grid))
        grid = np.concatenate([[grid[0] - d], grid, [grid[-1] + d]])
        modes = np.vstack([np.zeros((1, modes.shape[1])), modes, np.zeros((1, modes.shape[1]))])
    yp = (yn[None, :] + 0.5 * rho_y[:, None]).ravel()
    ym = (yn[None, :] - 0.5 * rho_y[:, None]).ravel()
    out = np.empty((rho_y.size, yn.size, modes.shape[1]))
    for m in range(modes.shape[1]):
        a = np.interp(yp, grid, modes[:, m], left=0.0, right=0.0)
        b = np.interp(ym, grid, modes[:, m], left=0.0, right=0.0)
        out[:, :, m] = (a * b).reshape(rho_y.size, yn.size)
    return out


def contact_mode_reservoir(mat, f, side, Ef, Vxy):
    """(rhoBoundary [N_rho_x N_rho_y x N_Y_nodes], info) (get_ContactModeReservoirRho_full2D.m): the
    Fourier-Galerkin contact modes of a periodic Y cell, or the box contact problem."""
    prm = mat["dg"]["params"]
    temp = float(mat.get("Temp", 300))
    deg = float(np.ravel(mat.get("deg_factor", [1]))[0])
    periodic = f.get("ytype") == "periodic"
    if periodic:
        E, coef, kw, gy, width = _periodic_modes(mat, f, side, Vxy)
    else:
        E, modes, grid, hard = _box_modes(mat, f, side, Vxy)
    mx, mz = _rel_mass(mat, "x") * M0, _rel_mass(mat, "z") * M0
    RX, RY = f["rel"]
    kx, dkx = _k_grid(_p(prm, "full2D_contactMode_Nkx", _p(prm, "full2D_reservoir_Nkx", RX["n"])), RX["length"])
    integrate = bool(_p(prm, "full2D_contactModeIntegrateKz", "me_z" in mat or "me_z_ch" in mat))
    model = str(_p(prm, "full2D_contactModeFermiModel", "contact-neutrality")).strip().lower().replace("_", "-")
    target = float(_p(prm, "full2D_%sContactSheetDensity" % side, np.nan))
    ef = float(Ef) if Ef is not None and np.isfinite(Ef) else np.nan
    if model == "contact-neutrality" and integrate and np.isfinite(target) and target > 0:
        ef = _neutral_fermi(E, mx, mz, target, temp, deg, prm, ef)
    if not np.isfinite(ef):
        return np.zeros((RX["n"] * RY["n"], f["axes"][1]["nd"])), {"fermiLevelUsed": np.nan, "modeEnergy": E}
    ekx = HBAR ** 2 * kx ** 2 / (2 * mx * QE)
    if integrate:
        tail = _p(prm, "full2D_contactModeKzThermalTail", 10) * KB_RES * temp / QE
        window = max(_p(prm, "full2D_contactModeKzEnergyWindow", 0.3), max(ef - E.min(), 0.0) + tail)
        kz = np.linspace(0.0, np.sqrt(max(window, np.finfo(float).eps) * 2 * mz * QE) / HBAR,
                         max(2, int(round(_p(prm, "full2D_contactMode_Nkz", _p(prm, "full2D_reservoir_Nkz", 1001))))))
        ekz = HBAR ** 2 * kz ** 2 / (2 * mz * QE)
        arg = np.clip(QE * (E[:, None, None] + ekx[None, :, None] + ekz[None, None, :] - ef) / (KB_RES * temp),
                      -80, 80)
        occ = 1.0 / (1.0 + np.exp(arg))                         # [mode, kx, kz]
        h = np.diff(kz)
        fk = 2 * deg * (0.5 * (occ[:, :, 1:] + occ[:, :, :-1]) @ h) / np.pi
    else:
        arg = np.clip(QE * (E[:, None] + ekx[None, :] - ef) / (KB_RES * temp), -80, 80)
        fk = 2 * deg / (1.0 + np.exp(arg))
    rx = (np.cos(np.outer(RX["cells"], kx)) @ fk.T) * dkx / (2 * np.pi)          # [rho_x, mode]
    yn = f["axes"][1]["nodes"]
    if periodic:
        yp = (yn[None, :] + 0.5 * RY["cells"][:, None]) - gy[0]                   # [rho_y, node]
        ym = (yn[None, :] - 0.5 * RY["cells"][:, None]) - gy[0]
        php = np.exp(1j * yp[..., None] * kw) @ coef / np.sqrt(width)            # [rho_y, node, mode]
        phm = np.exp(1j * ym[..., None] * kw) @ coef / np.sqrt(width)
        ry = php * np.conj(phm)
    else:
        ry = _box_density(modes, grid, hard, yn, RY["cells"])
    rho = np.einsum("am,bnm->abn", rx, ry)                                         # [rho_x, rho_y, node]
    rho = rho.reshape(RX["n"] * RY["n"], yn.size, order="F")
    return rho.real if np.abs(rho.imag).max() <= 1e-12 * max(np.abs(rho.real).max(), 1e-300) else rho, \
        {"fermiLevelUsed": ef, "modeEnergy": E, "model": "contact-modes"}


def default_reservoir(mat, f, side, Ef, Vxy):
    """(rhoBoundary, info) (get_DefaultReservoirRho_full2D.m:15-96)."""
    prm = mat["dg"]["params"]
    RX, RY = f["rel"]
    if not _p(prm, "full2D_useMaterialReservoir", True) or Ef is None or not np.isfinite(Ef):
        return np.zeros((RX["n"] * RY["n"], f["axes"][1]["nd"])), {"model": "zero-placeholder"}
    temp = float(mat.get("Temp", 300))
    deg = float(np.ravel(mat.get("deg_factor", [1]))[0])
    kx, dkx = _k_grid(_p(prm, "full2D_reservoir_Nkx", RX["n"]), RX["length"])
    ky, dky = _k_grid(_p(prm, "full2D_reservoir_Nky", RY["n"]), RY["length"])
    yn = f["axes"][1]["nodes"]
    gy = np.asarray(mat["y"], dtype=float) * f["scale"]

    def at_edge(a):
        a = np.asarray(a, dtype=float)
        a = a.reshape(int(mat["Nx"]), int(mat["Ny"])) if a.size == int(mat["Nx"]) * int(mat["Ny"]) else \
            np.full((int(mat["Nx"]), int(mat["Ny"])), float(np.ravel(a)[0]))
        row = a[-1] if side == "drain" else a[0]
        return np.interp(yn, gy, row) if gy.size > 1 else np.full(yn.shape, row[0])

    def kg(m):
        m = np.where(np.abs(m) > 1e-25, m * M0, m)
        return np.where(m <= 0, 0.041 * M0, m)
    V = at_edge(Vxy)
    mX = kg(at_edge(mat.get("me_x", mat.get("me_x_ch", 0.041))))
    mY = kg(at_edge(mat.get("me_y", mat.get("me_y_ch", 0.041))))
    cx, cy = np.cos(np.outer(RX["cells"], kx)), np.cos(np.outer(RY["cells"], ky))
    e = V[:, None, None] + HBAR ** 2 * (kx[None, :, None] ** 2 / (2 * mX[:, None, None]) +
                                         ky[None, None, :] ** 2 / (2 * mY[:, None, None])) / QE
    occ = 2 * deg / (1 + np.exp(np.clip(QE * (e - Ef) / (KB_RES * temp), -80, 80)))   # [node, kx, ky]
    rho = np.einsum("ak,nkl,bl->abn", cx, occ, cy) * dkx * dky / (2 * np.pi) ** 2
    return rho.reshape(RX["n"] * RY["n"], yn.size, order="F"), {"model": "material-default", "fermiLevelUsed": Ef}


def get_InflowBoundary_full2D(mat, f, EfL, EfR, Vxy=None):
    """{'source': (rhoBoundary, info), 'drain': ...} (get_InflowBoundary_full2D.m:1-56 with the
    reservoir model switch of :127-151)."""
    prm = mat["dg"]["params"]
    if Vxy is None:
        Vxy = mat.get("V", np.zeros((int(mat["Nx"]), int(mat["Ny"]))))
    model = str(_p(prm, "full2D_reservoirModel", "material-default")).strip().lower().replace("_", "-")
    masks = f.get("contact_masks") or {}
    if f.get("ytype") == "periodic" and not all(np.all(m) for m in masks.values()):
        raise WignerError(_lib.WG_ERR_ARG, "Periodic two-point contacts currently require full-width Source/Drain "
                          "masks.", "DG:Full2D:PeriodicContactMask")
    out = {}
    for side, ef in (("source", EfL), ("drain", EfR)):
        if model in ("contact-modes", "contact-mode", "modes"):
            out[side] = contact_mode_reservoir(mat, f, side, ef, Vxy)
        elif model in ("material-default", "default", "material"):
            out[side] = default_reservoir(mat, f, side, ef, Vxy)
        elif model in ("none", "zero", "off"):
            RX, RY = f["rel"]
            out[side] = (np.zeros((RX["n"] * RY["n"], f["axes"][1]["nd"])), {"model": "none"})
        else:
            raise WignerError(_lib.WG_ERR_ARG, "unknown full2D_reservoirModel %r" % model)
    for side in out:
        # reservoir data only on the contact pieces of the face (applyContactMask, get_InflowBoundary_full2D.m:23-24)
        m = masks.get(side)
        if m is not None and not np.all(m):
            rho, info = out[side]
            out[side] = (rho * m[None, :], dict(info, contactMask=np.asarray(m, dtype=bool)))
    if f.get("wall") is not None:
        # hard walls: the face data only on the active (rho_y, Y) samples (get_InflowBoundary_full2D.m:36-43)
        mask = np.repeat(f["wall"]["active"], f["rel"][0]["n"], axis=0)
        for side in out:
            rho, info = out[side]
            out[side] = (rho * mask, dict(info, hardWallSupportApplied=True))
    return out


def inflow_rhs(f, inflow):
    """The right-hand side of the Full-2D system from the Source/Drain reservoirs
    (get_Diff_full2D.m:405-430): scale_x sum_iy [e_iy (x) lift_L (x) A+ rho_src(:, iy) -
    e_iy (x) lift_R (x) A- rho_drn(:, iy)], state order (rho_x, rho_y, X, Y)."""
    AX, AY = f["axes"]
    RX, RY = f["rel"]
    Apx, Amx = f["split"][0], f["split"][1]
    sx = f["scales"][0]
    invM = np.linalg.inv(AX["M"])
    nl, nx = AX["nl"], AX["nd"]
    lift_l = np.zeros(nx); lift_l[:nl] = invM[:, 0] / AX["jac"][0]
    lift_r = np.zeros(nx); lift_r[nx - nl:] = invM[:, nl - 1] / AX["jac"][-1]
    src, drn = inflow["source"][0], inflow["drain"][0]
    nrx, nry = RX["n"], RY["n"]
    # kron(I_rho_y, A+/-_x) applied to every face column: rho_x is the fastest index
    inc_l = (Apx @ src.reshape(nrx, nry, -1, order="F").reshape(nrx, -1)).reshape(nrx, nry, -1)
    inc_r = (Amx @ drn.reshape(nrx, nry, -1, order="F").reshape(nrx, -1)).reshape(nrx, nry, -1)
    inc_l = inc_l.reshape(nrx * nry, -1, order="F")
    inc_r = inc_r.reshape(nrx * nry, -1, order="F")
    rhs = np.zeros((AY["nd"], nx, nrx * nry), dtype=complex)                 # [Y dof, X dof, relative]
    # the lifts live on the first and last X element only
    rhs[:, :nl, :] += sx * (lift_l[None, :nl, None] * inc_l.T[:, None, :])
    rhs[:, nx - nl:, :] -= sx * (lift_r[None, nx - nl:, None] * inc_r.T[:, None, :])
    return rhs.reshape(-1)
