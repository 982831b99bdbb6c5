"""Full-2D contact reservoirs and the source/drain inflow right-hand side (oracle; test
infrastructure only).

Restates in NumPy the reservoir data that the reference feeds into the Full-2D transport solve:

  contact_mode_reservoir    DG_code/core/get_ContactModeReservoirRho_full2D.m:1-151 on a periodic
                            Y cell (the Fourier-Galerkin contact modes of
                            get_PeriodicContactModes_full2D.m:1-70) or on a box (the transverse
                            contact problem of :153-302, :343-367), the contact-neutrality Fermi
                            level (:407-467, :483-621: bracket + bisection on the k_z-integrated
                            sheet density of the modes), the k_z window (:649-702), the
                            longitudinal occupation and its cosine transform (:304-329), the
                            density matrix phi_n(Y + rho_y/2) conj(phi_n(Y - rho_y/2)) at the Y
                            DG nodes
  default_reservoir         DG_code/core/get_DefaultReservoirRho_full2D.m:1-96: the separable
                            (k_x, k_y) Fermi distribution of the contact edge, cosine-transformed
                            to (rho_x, rho_y)
  inflow_rhs                DG_code/core/get_Diff_full2D.m:393-430 and :609-615: the Source and
                            Drain inflow parts scale_x kron(e_iy (x) lift, A+/- rho_boundary(:, iy))
                            of the system's right-hand side (full-width contacts)

Pinned against the reservoir data that the reference's recorded run stored
(2026-10-28_08-47/Sim_Res.mat: boundary.physical.XLeft/XRight.rhoBoundary with the mode energies
and Fermi levels of dataInfo.defaultReservoir), frozen in tests/golden/full2d_reservoir_golden.npz
by tests/golden/make_reservoir_golden.py.
"""
import numpy as np

HBAR = 1.054571817e-34
QE = 1.602176634e-19
KB = 1.38064852e-23          # the reservoir files' physicalConstants
M0 = 9.1093837015e-31


def _param(prm, name, default):
    v = prm.get(name, None)
    if v is None and isinstance(prm.get("full2D"), dict):
        v = prm["full2D"].get(name, None)
    return default if v is None else v


def make_k_grid(nk, length):
    """makeKGrid (get_ContactModeReservoirRho_full2D.m:704-708)."""
    nk = max(2, int(round(nk)))
    k = -2 * np.pi / length * (np.arange(1, nk + 1) - 0.5 * (nk + 1))
    return k, abs(k[1] - k[0])


def _constant_mass(mat, axis):
    """constantMass (get_PeriodicContactModes_full2D.m:72-95), relative units."""
    ref = "me_%s_ch" % axis
    m = mat[ref] if ref in mat else mat["me_x_ch"]
    if m < 1e-25:
        m = m / M0
    return float(m)


def periodic_contact_modes(mat, p, side, Vxy):
    """(energy [nm], coefficients, wave numbers, gridY, width) (get_PeriodicContactModes_full2D.m:9-57)."""
    prm = mat["dg"]["params"]
    gridY = np.asarray(mat["y"], dtype=float) * p["coordinateScale"]
    width = p["y"][-1] - p["y"][0]
    nunique = gridY.size - 1
    dy = width / nunique
    max_order = min((nunique - 1) // 2, (p["rhoY"]["nCells"] - 2) // 4)
    order = int(_param(prm, "full2D_periodicModeOrder", max_order))
    if order < 0 or order > max_order:
        raise ValueError("DG:Full2D:PeriodicModeOrder")
    ix = mat["Nx"] - 1 if side.lower() == "drain" else 0
    edge = np.asarray(Vxy, dtype=float).reshape(mat["Nx"], mat["Ny"])[ix, :]
    if abs(edge[0] - edge[-1]) > 1e-10 * max(1, np.abs(edge).max()):
        raise ValueError("DG:Full2D:NonperiodicPotential")
    my = _constant_mass(mat, "y")
    k = (2 * np.pi / width) * np.arange(-order, order + 1)
    basis = np.exp(1j * np.outer(gridY[:-1] - gridY[0], k)) / np.sqrt(width)
    H = np.diag(HBAR ** 2 * k ** 2 / (2 * my * M0 * QE)) + dy * (basis.conj().T @ (edge[:-1, None] * basis))
    H = (H + H.conj().T) / 2
    if np.abs(edge - edge[0]).max() < 1e-13 * max(1, abs(edge[0])):
        energy = edge[0] + HBAR ** 2 * k ** 2 / (2 * my * M0 * QE)
        ids = np.argsort(energy, kind="stable")
        energy = energy[ids]
        coef = np.eye(k.size)[:, ids]
    else:
        w, v = np.linalg.eigh(H)
        ids = np.argsort(w.real, kind="stable")
        energy, coef = w.real[ids], v[:, ids]
    return energy, coef, k, gridY, width


def sheet_density(ef, energy, mx, mz, temp, deg):
    """contactSheetDensity (:613-621) with the stable softplus of :623-631."""
    kbt = KB * temp
    eta = QE * (ef - np.real(energy)) / kbt
    dos = np.sqrt(np.real(mx) * np.real(mz))
    pref = deg * dos * kbt / (np.pi * HBAR ** 2)
    sp = np.where(eta > 40, eta, np.where(eta < -40, np.exp(np.minimum(eta, 0)), np.log1p(np.exp(np.clip(eta, -40, 40)))))
    by = pref * sp
    return by.sum(), by


def solve_neutrality(energy, mx, mz, target, temp, deg, prm, guess):
    """solveContactNeutrality (:533-611): bracket, then bisection to a relative 1e-10."""
    tol = _param(prm, "full2D_contactModeFermiTolerance", 1e-10)
    maxit = int(_param(prm, "full2D_contactModeFermiMaxIterations", 200))
    ktev = KB * temp / QE
    emin = np.min(np.real(energy))
    step = max(0.5, 20 * ktev)
    lo = emin - max(2, 80 * ktev)
    hi = emin + max(2, 80 * ktev)
    if np.isfinite(guess):
        lo = min(lo, guess - step)
        hi = max(hi, guess + step)
    dlo = sheet_density(lo, energy, mx, mz, temp, deg)[0]
    dhi = sheet_density(hi, energy, mx, mz, temp, deg)[0]
    for _ in range(50):
        if dlo <= target <= dhi:
            break
        step *= 2
        if dlo > target:
            lo -= step
            dlo = sheet_density(lo, energy, mx, mz, temp, deg)[0]
        if dhi < target:
            hi += step
            dhi = sheet_density(hi, energy, mx, mz, temp, deg)[0]
    if dlo > target or dhi < target:
        raise ValueError("DG:Full2D:ContactFermiBracketFailed")
    for _ in range(maxit):
        mid = 0.5 * (lo + hi)
        dm = sheet_density(mid, energy, mx, mz, temp, deg)[0]
        if abs(dm - target) / target <= tol:
            lo = hi = mid
            break
        if dm < target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def kz_grid(prm, mz, energy, ef, temp):
    """makeKzInfo (:649-702): 0 .. kz_max over the occupied window plus a thermal tail."""
    nkz = _param(prm, "full2D_contactMode_Nkz", _param(prm, "full2D_reservoir_Nkz", 1001))
    wmin = _param(prm, "full2D_contactModeKzEnergyWindow", 0.3)
    tail = _param(prm, "full2D_contactModeKzThermalTail", 10)
    tail_ev = tail * KB * temp / QE
    occupied = max(np.max(np.real(ef)) - np.min(np.real(energy)), 0.0)
    window = max(wmin, occupied + tail_ev)
    nkz = max(2, int(round(nkz)))
    mzref = np.max(np.real(mz))
    kzmax = np.sqrt(max(window, np.finfo(float).eps) * 2 * mzref * QE) / HBAR
    return np.linspace(0.0, kzmax, nkz)


def longitudinal_occupation(kx, e_mode, mx, mz, ef, temp, deg, kz):
    """longitudinalOccupation (:311-329), k_z integrated by the trapezoid rule."""
    ekx = HBAR ** 2 * kx ** 2 / (2 * mx * QE)
    if kz is None:
        arg = np.clip(QE * (e_mode + ekx - ef) / (KB * temp), -80, 80)
        return 2 * deg / (1 + np.exp(arg))
    ekz = HBAR ** 2 * kz ** 2 / (2 * mz * QE)
    arg = np.clip(QE * (e_mode + ekx[:, None] + ekz[None, :] - ef) / (KB * temp), -80, 80)
    fermi = 1 / (1 + np.exp(arg))
    trapz = getattr(np, "trapezoid", None) or np.trapz
    return 2 * deg * trapz(fermi, kz, axis=1) / np.pi


def box_contact_modes(mat, p, side, Vxy):
    """The non-periodic contact problem (get_ContactModeReservoirRho_full2D.m:153-302): the transverse
    Hamiltonian on the sorted material Y grid of the contact column (interior three-point rows with
    harmonic-mean masses; the first and last rows copy their neighbour's diagonal and outer coupling,
    the mode vanishing one step beyond the grid), or with hard walls the interior unknowns only (the
    mode vanishing at the walls); the nModes eigenpairs of smallest magnitude in ascending order,
    normalised to a unit trapezoid integral over y, the last grid value made nonnegative.  Constant
    masses.  Returns (energy, modes [nY x nModes] on the grid, grid, hard_wall)."""
    prm = mat["dg"]["params"]
    raw = np.asarray(mat["y"], dtype=float) * p["coordinateScale"]
    order = np.argsort(raw, kind="stable")
    grid = raw[order]
    nx, ny = int(mat["Nx"]), int(mat["Ny"])
    V = np.asarray(Vxy, dtype=float).reshape(nx, ny)[0 if side == "source" else nx - 1][order]
    my = _constant_mass(mat, "y")
    n = grid.size
    if n < 3:
        raise ValueError("DG:Full2D:ContactModeGridTooSmall")
    dy = np.mean(np.diff(grid))
    t0 = HBAR ** 2 / (2 * M0 * QE * dy ** 2)
    H = np.zeros((n, n))
    for i in range(1, n - 1):
        left, right = -2 * t0 / (my + my), -2 * t0 / (my + my)
        H[i, i - 1], H[i, i], H[i, i + 1] = left, -left - right + V[i], right
    H[0, 0], H[0, 1] = H[1, 1], H[1, 2]
    H[n - 1, n - 1], H[n - 1, n - 2] = H[n - 2, n - 2], H[n - 2, n - 3]
    hard = p.get("ytype") == "hard-wall"
    active = np.arange(n)
    if hard:
        tol = 64 * np.spacing(np.max(np.abs(grid)))
        if max(abs(grid[0] - p["y"][0]), abs(grid[-1] - p["y"][-1])) > tol:
            raise ValueError("DG:Full2D:HardWallContactDomainMismatch")
        active = np.arange(1, n - 1)
        H = H[np.ix_(active, active)]
    ngrid = H.shape[0]
    nm = int(mat["n_of_modes"]) if mat.get("n_of_modes") is not None else min(4, ngrid - 1)
    nm = int(round(_param(prm, "full2D_contactModeCount", nm)))
    nm = max(1, min(nm, ngrid))
    w, vec = np.linalg.eig(H)
    if nm < ngrid:                        # eigs(H, nModes, 'sm'): the smallest magnitudes
        keep = np.argsort(np.abs(w), kind="stable")[:nm]
        w, vec = w[keep], vec[:, keep]
    ids = np.argsort(np.real(w), kind="stable")[:nm]
    energy = np.real(w[ids])
    modes = np.zeros((n, nm))
    modes[active, :] = np.real(vec[:, ids])
    wts = np.zeros(n)
    wts[1:] += 0.5 * np.diff(grid)
    wts[:-1] += 0.5 * np.diff(grid)
    for im in range(nm):
        norm = np.sqrt(np.sum(wts * modes[:, im] ** 2))
        if norm > 0:
            modes[:, im] /= norm
        if modes[-1, im] < 0:
            modes[:, im] = -modes[:, im]
    return energy, modes, grid, hard


def box_mode_density(mode, grid, hard, yface, rho_y):
    """transverseModeDensity (:343-360): phi(Y + rho_y/2) phi(Y - rho_y/2) by linear interpolation,
    zero outside; the box modes continue to zero ghost nodes one grid step beyond the edges."""
    if hard:
        g, v = grid, mode
    else:
        dy = np.mean(np.diff(grid))
        g = np.concatenate([[grid[0] - dy], grid, [grid[-1] + dy]])
        v = np.concatenate([[0.0], mode, [0.0]])
    out = np.zeros((rho_y.size, yface.size))
    for iy in range(yface.size):
        plus = np.interp(yface[iy] + 0.5 * rho_y, g, v, left=0.0, right=0.0)
        minus = np.interp(yface[iy] - 0.5 * rho_y, g, v, left=0.0, right=0.0)
        out[:, iy] = plus * minus
    return out


def contact_mode_reservoir(mat, p, side, ef_input, Vxy):
    """(rhoBoundary [nRel x nYnodes], info) (get_ContactModeReservoirRho_full2D.m:35-151): the periodic
    branch on a periodic Y cell, the box contact problem otherwise."""
    prm = mat["dg"]["params"]
    temp = float(mat.get("Temp", 300))
    deg = float(np.ravel(mat.get("deg_factor", [1]))[0])
    periodic = p.get("ytype", "periodic") == "periodic"
    if periodic:
        energy, coef, kw, gridY, width = periodic_contact_modes(mat, p, side, Vxy)
    else:
        energy, modes, gridY, hard = box_contact_modes(mat, p, side, Vxy)
    nm = energy.size
    mx = _constant_mass(mat, "x") * M0 * np.ones(nm)     # constant mass: the harmonic mode average
    mz = _constant_mass(mat, "z") * M0 * np.ones(nm)
    nkx = _param(prm, "full2D_contactMode_Nkx", _param(prm, "full2D_reservoir_Nkx", p["rhoX"]["nCells"]))
    kx, dkx = make_k_grid(nkx, p["rhoX"]["length"])
    cosX = np.cos(np.outer(p["rhoX"]["cells"], kx))
    integrate = bool(_param(prm, "full2D_contactModeIntegrateKz", ("me_z" in mat) or ("me_z_ch" in mat)))
    model = str(_param(prm, "full2D_contactModeFermiModel", "contact-neutrality")).strip().lower().replace("_", "-")
    target = _param(prm, "full2D_%sContactSheetDensity" % side.lower(), np.nan)
    ef = float(ef_input)
    if model == "contact-neutrality" and integrate and np.isfinite(target) and target > 0:
        ef = solve_neutrality(energy, mx, mz, target, temp, deg, prm, float(ef_input))
    kz = kz_grid(prm, mz, energy, ef, temp) if integrate else None
    yface = p["Y"]["nodes"]
    rho_y = p["rhoY"]["cells"]
    nrel = p["rhoX"]["nCells"] * p["rhoY"]["nCells"]
    rho = np.zeros((nrel, yface.size), dtype=complex)
    ypl = yface[None, :] + 0.5 * rho_y[:, None]
    ymi = yface[None, :] - 0.5 * rho_y[:, None]
    for im in range(nm):
        fkx = longitudinal_occupation(kx, energy[im], mx[im], mz[im], ef, temp, deg, kz)
        rx = cosX @ fkx * dkx / (2 * np.pi)
        if periodic:
            php = np.exp(1j * np.outer(ypl.ravel(order="F") - gridY[0], kw)) @ coef[:, im] / np.sqrt(width)
            phm = np.exp(1j * np.outer(ymi.ravel(order="F") - gridY[0], kw)) @ coef[:, im] / np.sqrt(width)
            ry = (php * np.conj(phm)).reshape(ypl.shape, order="F")
        else:
            ry = box_mode_density(modes[:, im], gridY, hard, yface, rho_y)
        for iy in range(yface.size):
            rho[:, iy] += np.outer(rx, ry[:, iy]).ravel(order="F")
    # the +/- k plane waves of one energy pair up into real cosines; the stored data are real
    return rho, {"modeEnergy": energy, "fermiLevelUsed": ef, "kz": kz, "kx": kx}


def default_reservoir(mat, p, side, ef, Vxy):
    """(rhoBoundary [nRel x nYnodes]) (get_DefaultReservoirRho_full2D.m:15-96)."""
    prm = mat["dg"]["params"]
    temp = float(mat.get("Temp", 300))
    deg = float(np.ravel(mat.get("deg_factor", [1]))[0])
    kx, dkx = make_k_grid(_param(prm, "full2D_reservoir_Nkx", p["rhoX"]["nCells"]), p["rhoX"]["length"])
    ky, dky = make_k_grid(_param(prm, "full2D_reservoir_Nky", p["rhoY"]["nCells"]), p["rhoY"]["length"])
    cosX = np.cos(np.outer(p["rhoX"]["cells"], kx))
    cosY = np.cos(np.outer(p["rhoY"]["cells"], ky))
    yface = p["Y"]["nodes"]
    ix = mat["Nx"] - 1 if side.lower() == "drain" else 0
    gy = np.asarray(mat["y"], dtype=float) * p["coordinateScale"]

    def edge(field, default):
        f = mat.get(field)
        f = np.full((mat["Nx"], mat["Ny"]), default) if f is None else np.asarray(f, dtype=float).reshape(
            mat["Nx"], mat["Ny"])
        return np.interp(yface, gy, f[ix]) if gy.size > 1 else np.full(yface.shape, f[ix, 0])

    def kg(m):
        m = np.where(np.abs(m) > 1e-25, m * M0, m)
        return np.where(m <= 0, 0.041 * M0, m)
    V = np.interp(yface, gy, np.asarray(Vxy, dtype=float).reshape(mat["Nx"], mat["Ny"])[ix])
    mX = kg(edge("me_x", mat.get("me_x_ch", 0.041)))
    mY = kg(edge("me_y", mat.get("me_y_ch", 0.041)))
    rho = np.zeros((p["rhoX"]["nCells"] * p["rhoY"]["nCells"], yface.size))
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    for iy in range(yface.size):
        e = V[iy] + HBAR ** 2 * KX ** 2 / (2 * mX[iy] * QE) + HBAR ** 2 * KY ** 2 / (2 * mY[iy] * QE)
        arg = np.clip(QE * (e - ef) / (KB * temp), -80, 80)
        f = 2 * deg / (1 + np.exp(arg))
        rho[:, iy] = (cosX @ f @ cosY.T * dkx * dky / (2 * np.pi) ** 2).ravel(order="F")
    return rho


def inflow_rhs(p, rho_src, rho_drn, scale_x, Apx, Amx, left_lift, right_lift):
    """The Source / Drain inflow parts of the right-hand side (get_Diff_full2D.m:405-430 with
    assembleRhs :609-615), every Y face node a contact: rhs = sum_iy scale_x [kron(e_iy (x) lift_L,
    A+ rho_src(:, iy)) - kron(e_iy (x) lift_R, A- rho_drn(:, iy))], A+/- = kron(I_rho_y, A+/-_x)."""
    nry = p["rhoY"]["nCells"]
    nrel = p["rhoX"]["nCells"] * nry
    ncen = p["X"]["nDof"] * p["Y"]["nDof"]
    Ap = np.kron(np.eye(nry), Apx)
    Am = np.kron(np.eye(nry), Amx)
    rhs = np.zeros(ncen * nrel, dtype=complex)
    for iy in range(p["Y"]["nDof"]):
        e = np.zeros(p["Y"]["nDof"]); e[iy] = 1
        rhs += scale_x * np.kron(np.kron(e, left_lift), Ap @ rho_src[:, iy])
        rhs -= scale_x * np.kron(np.kron(e, right_lift), Am @ rho_drn[:, iy])
    return rhs
