"""Synthetic 1D resonant-tunnelling-diode device descriptions.

Host-side set-up in the role of the reference's device builders
(buildDevice.m:123-200, RTD/buildDevice2D_rtd.m): it produces the ``mat``
structure that ``solve_transport_DG_2D`` consumes, on a uniform material grid
``x = linspace(0, L, Nx)`` in nm with ``Nx = N_el*(N_K-1)+1`` so that every DG
element spans N_K-1 material cells (solve_transport_DG_2D.m:81-87).

Energies are in eV, lengths of the material grid in nm, ``Ly`` (the xi
correlation length) in m, masses in units of m0, as in the reference.
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class RTDSpec:
    """Double-barrier RTD along x, flat in the transverse directions."""
    length_nm: float = 60.0
    contact_nm: float = 15.0
    barrier_ev: float = 0.27
    barrier_nm: float = 3.0
    well_nm: float = 5.0
    doping_m3: float = 1e24            # 1e18 cm^-3
    m_rel: float = 0.067               # GaAs
    temp_k: float = 300.0
    eps_r: float = 12.9
    order: int = 2                     # DG order p, N_K = p + 1
    n_el: int = 120
    nk: int = 128
    n_xi: int = 0                      # 0 -> n_xi = nk
    l_xi_m: float = 30e-9
    fermi_offset_ev: float = 0.05      # E_F above the contact band edge
    extra: dict = field(default_factory=dict)

    @property
    def n_local(self):
        return self.order + 1

    @property
    def nx(self):
        return self.n_el * self.order + 1


def band_edge(spec: RTDSpec, x_nm: np.ndarray) -> np.ndarray:
    """Conduction band edge [eV]: barriers of height barrier_ev around a centred well."""
    c = spec.length_nm / 2
    half_w = spec.well_nm / 2
    ec = np.zeros_like(x_nm)
    left = (x_nm >= c - half_w - spec.barrier_nm) & (x_nm <= c - half_w)
    right = (x_nm >= c + half_w) & (x_nm <= c + half_w + spec.barrier_nm)
    ec[left | right] = spec.barrier_ev
    return ec


def bias_ramp(spec: RTDSpec, x_nm: np.ndarray) -> np.ndarray:
    """0 in the source contact, 1 in the drain contact, linear in between."""
    a, b = spec.contact_nm, spec.length_nm - spec.contact_nm
    return np.clip((x_nm - a) / (b - a), 0.0, 1.0)


def doping(spec: RTDSpec, x_nm: np.ndarray) -> np.ndarray:
    """Donor density [m^-3]: doped contacts, undoped active region."""
    nd = np.zeros_like(x_nm)
    nd[(x_nm <= spec.contact_nm) | (x_nm >= spec.length_nm - spec.contact_nm)] = spec.doping_m3
    return nd


def make_mat(spec: RTDSpec) -> dict:
    """The ``mat`` structure of one RTD (one valley, one mode, Ny = 1)."""
    nx = spec.nx
    x = np.linspace(0.0, spec.length_nm, nx)
    nxi = spec.n_xi or spec.nk
    mat = {
        "type": "RTD-1D",
        "Nx": nx,
        "Ny": 1,
        "dy": 1.0,
        "dx": spec.length_nm / (nx - 1),
        "x": x,
        "L_x": spec.length_nm,
        "me_x": np.full((1, nx, 1), spec.m_rel),
        "me_z_ch": spec.m_rel,
        "Temp": spec.temp_k,
        "deg_factor": np.array([1.0]),
        "n_of_valleys": 1,
        "n_of_modes": 1,
        "Vc": band_edge(spec, x),
        "Nd": doping(spec, x),
        "eps": np.full(nx, spec.eps_r),
        "ramp": bias_ramp(spec, x),
        "dg": {"params": {
            "N_K_chi": spec.n_local,
            "Xi_solver": "FV",
            "N_xi": nxi,
            "N": spec.nk,
            "Ly": spec.l_xi_m,
            "Q": "EXP",
            "permute_shell": True,
            "MPC": 1.0,
            "sl": 0,
            "st_init": False,
        }},
    }
    mat.update(spec.extra)
    return mat


def flatband_potential(mat: dict, bias: float) -> np.ndarray:
    """Esub for a fixed linear bias drop across the active region [eV]."""
    return np.asarray(mat["Vc"]) - bias * np.asarray(mat["ramp"])


def density_normalisation_nm(mat: dict, offset_ev: float = 0.05) -> float:
    """Transverse length dy [nm] that makes the contact's equilibrium density equal N_D.

    The 1D Wigner density is n_DG = sum_k f(k) dk / 2 pi with f the kz-integrated
    Fermi-Dirac occupation of the contact (verteilung.m:139-152), a sheet density;
    the volume density is n_DG |Vsub|^2 / dy (solve_transport_DG_2D.m:204).  This
    picks dy so that the flat-band contact at E_F - Ec = offset carries N_D.
    """
    h, m0, q, kb = 6.626e-34, 9.109e-31, 1.602e-19, 1.38e-23
    hb = h / 2 / np.pi
    prm = mat["dg"]["params"]
    nk, lxi = int(prm["N"]), float(prm["Ly"])
    k = -2 * np.pi / lxi * (np.arange(1, nk + 1) - 0.5 * (nk + 1))
    dk = abs(k[1] - k[0])
    m = float(np.asarray(mat["me_x"]).ravel()[0]) * m0
    me_z = float(mat["me_z_ch"])
    temp = float(mat["Temp"])
    vmax = float(np.max(mat["Vc"]))
    kz_max = np.sqrt(2 * 2 * m0 * me_z * q * (vmax + 0.3)) / hb
    kz = np.linspace(0.0, kz_max, 1001)
    ekz = hb ** 2 * kz ** 2 / 2 / m0 / me_z / q
    e = hb ** 2 * k ** 2 / 2 / m / q - offset_ev
    with np.errstate(over="ignore"):
        f = 2 / np.pi * (kz[1] - kz[0]) * np.sum(1 / (1 + np.exp(q * (e[:, None] + ekz[None, :]) / (kb * temp))), 1)
    n2d = np.sum(f) * dk / 2 / np.pi
    nd = float(np.max(mat["Nd"]))
    return n2d / nd / 1e-9


def contact_fermi_levels(mat: dict, bias: float, offset_ev: float = 0.05):
    """E_F,L = Vc(1) + offset, E_F,R = Vc(end) + offset - bias
    (RTD/solve2D_rtd_self_consistent.m:110-111 defaults)."""
    vc = np.asarray(mat["Vc"])
    return float(vc[0] + offset_ev), float(vc[-1] + offset_ev - bias)


@dataclass
class FETSpec:
    """Gated ultra-thin-body Si FET along x with a square cross-section.

    Subbands: the two valley types of a [100] Si wire (transport mass m_l with the
    cross-section confined by (m_t, m_t), degeneracy 2; transport mass m_t confined by
    (m_l, m_t), degeneracy 4) times the ``n_modes`` lowest particle-in-a-box modes of
    the ``width_nm`` x ``width_nm`` cross-section.  The longitudinal profile is a
    compact electrostatic model, not a Poisson solution: source at 0 eV, drain at
    -V_d, channel top at ``barrier_ev - gate_eff * V_g`` lowered towards the drain by
    ``dibl`` * V_d, joined by logistic steps of width ``step_nm`` at the junctions.
    """
    length_nm: float = 50.0
    sd_nm: float = 15.0               # source and drain extension lengths
    width_nm: float = 5.0
    oxide_nm: float = 1.0
    doping_m3: float = 1e26           # 1e20 cm^-3 in source and drain
    m_l: float = 0.98
    m_t: float = 0.19
    n_modes: int = 4
    barrier_ev: float = 0.45
    gate_eff: float = 0.8
    dibl: float = 0.1
    step_nm: float = 1.5
    temp_k: float = 300.0
    eps_r: float = 11.7
    order: int = 2
    n_el: int = 200
    nk: int = 256
    n_xi: int = 0
    l_xi_m: float = 30e-9
    fermi_offset_ev: float = 0.05

    @property
    def n_local(self):
        return self.order + 1

    @property
    def nx(self):
        return self.n_el * self.order + 1

    def valleys(self):
        """[(transport mass, (confinement masses)), ...] in units of m0."""
        return [(self.m_l, (self.m_t, self.m_t)), (self.m_t, (self.m_l, self.m_t))]


def fet_subband_offsets(spec: FETSpec) -> np.ndarray:
    """Confinement energies [n_valleys x n_modes] in eV: the lowest modes
    hbar^2 pi^2 (n^2 / m_y + l^2 / m_z) / (2 W^2) of each valley type."""
    h, m0, q = 6.626e-34, 9.109e-31, 1.602e-19
    hb = h / 2 / np.pi
    w = spec.width_nm * 1e-9
    out = []
    for _, (my, mz) in spec.valleys():
        e = sorted(hb ** 2 * np.pi ** 2 * (n * n / (my * m0) + l * l / (mz * m0)) / (2 * w * w) / q
                   for n in range(1, 5) for l in range(1, 5))
        out.append(e[:spec.n_modes])
    return np.asarray(out)


def fet_band_profile(spec: FETSpec, x_nm: np.ndarray, v_gate: float, v_drain: float) -> np.ndarray:
    """Longitudinal potential energy [eV] of the compact FET model (see FETSpec)."""
    s_src = 1 / (1 + np.exp(-(x_nm - spec.sd_nm) / spec.step_nm))
    s_drn = 1 / (1 + np.exp(-(x_nm - (spec.length_nm - spec.sd_nm)) / spec.step_nm))
    ch = spec.length_nm - 2 * spec.sd_nm
    top = spec.barrier_ev - spec.gate_eff * v_gate
    top = top - spec.dibl * v_drain * np.clip((x_nm - spec.sd_nm) / ch, 0.0, 1.0)
    return (1 - s_drn) * s_src * top + s_drn * (-v_drain)


def make_fet(spec: FETSpec, v_gate: float, v_drain: float):
    """(mat, Esub, Vsub, EfL, EfR) of one gate/drain point for ``solve_transport_DG_2D``:
    n_of_valleys = 2, n_of_modes = spec.n_modes, Ny = 1 (the mode's weight at the
    cross-section centre taken as 1 / W); E_F,L sits fermi_offset_ev above the
    source's lowest subband edge, E_F,R = E_F,L - V_d."""
    nx = spec.nx
    x = np.linspace(0.0, spec.length_nm, nx)
    nxi = spec.n_xi or spec.nk
    vals = spec.valleys()
    nv, nm = len(vals), spec.n_modes
    u = fet_band_profile(spec, x, v_gate, v_drain)
    esub = u[None, :, None] + fet_subband_offsets(spec)[:, None, :]
    vsub = np.full((nv, nx, nm, 1), 1.0 / np.sqrt(spec.width_nm))
    nd = np.where((x <= spec.sd_nm) | (x >= spec.length_nm - spec.sd_nm), spec.doping_m3, 0.0)
    mat = {
        "type": "UTB-FET-1D-modes",
        "Nx": nx,
        "Ny": 1,
        "dy": spec.width_nm,
        "dx": spec.length_nm / (nx - 1),
        "x": x,
        "L_x": spec.length_nm,
        "me_x": np.repeat(np.asarray([v[0] for v in vals])[:, None, None], nx, axis=1),
        "me_z_ch": spec.m_t,
        "Temp": spec.temp_k,
        "deg_factor": np.array([2.0, 4.0]),
        "n_of_valleys": nv,
        "n_of_modes": nm,
        "Vc": u,
        "Nd": nd,
        "eps": np.full(nx, spec.eps_r),
        "ramp": np.clip((x - spec.sd_nm) / (spec.length_nm - 2 * spec.sd_nm), 0.0, 1.0),
        "dg": {"params": {
            "N_K_chi": spec.n_local,
            "Xi_solver": "FV",
            "N_xi": nxi,
            "N": spec.nk,
            "Ly": spec.l_xi_m,
            "Q": "EXP",
            "permute_shell": True,
            "MPC": 1.0,
            "sl": 0,
            "st_init": False,
        }},
    }
    ef_l = float(esub[:, 0, :].min()) + spec.fermi_offset_ev   # above the source's lowest subband edge
    return mat, esub, vsub, ef_l, ef_l - v_drain


def utb_cross_section(spec: FETSpec, v_gate: float, v_drain: float, dy_nm: float = 0.1, oxide_offset_ev: float = 3.1,
                      me_y_ox: float = 0.5, bend_ev: float = 0.05):
    """Mode-space set-up of a double-gate ultra-thin-body FET with its confinement direction
    resolved: (x [nm], y [nm], me_y [nv x Nx x Ny], V [Nx x Ny] eV) on the grid
    y = -t_ox .. W + t_ox step dy, in the layout of the reference's device builders
    (buildDeviceCMS.m:116-152: the material table mapped onto (x, y), oxide with its
    own confinement mass and a conduction-band offset).  The body carries the compact
    longitudinal profile of ``fet_band_profile`` lowered towards both gate interfaces
    by ``bend_ev`` (a parabola) under the gate; valley v's body mass is its first
    confinement mass."""
    x = np.linspace(0.0, spec.length_nm, spec.nx)
    ny = int(round((spec.width_nm + 2 * spec.oxide_nm) / dy_nm)) + 1
    y = np.arange(ny) * dy_nm - spec.oxide_nm
    body = (y >= -1e-12) & (y <= spec.width_nm + 1e-12)
    u = fet_band_profile(spec, x, v_gate, v_drain)
    s_src = 1 / (1 + np.exp(-(x - spec.sd_nm) / spec.step_nm))
    s_drn = 1 / (1 + np.exp(-(x - (spec.length_nm - spec.sd_nm)) / spec.step_nm))
    gate = s_src * (1 - s_drn)
    yc = 0.5 * spec.width_nm
    bend = -bend_ev * gate[:, None] * ((y[None, :] - yc) / yc) ** 2
    V = np.where(body[None, :], u[:, None] + bend, u[:, None] + oxide_offset_ev)
    vals = spec.valleys()
    me_y = np.empty((len(vals), spec.nx, ny))
    for iv, (_, (my, _)) in enumerate(vals):
        me_y[iv] = np.where(body, my, me_y_ox)[None, :]
    return x, y, me_y, V


def make_utb_fet(spec: FETSpec, v_gate: float, v_drain: float, solve_subbands=None, dy_nm: float = 0.1, **kw):
    """(mat, Esub, Vsub, EfL, EfR) of ``make_fet`` with the subbands from the transverse
    eigensolve of ``utb_cross_section`` (solve_subbands.m:1-40) instead of the box
    formula: mat gains Ny, dy, y, me_y, V; Vsub is [nv x Nx x nm x Ny].  ``solve_subbands``
    maps mat -> (E, V) and defaults to the GPU solver."""
    if solve_subbands is None:
        from .subbands import solve_subbands
    mat, _, _, _, _ = make_fet(spec, v_gate, v_drain)
    x, y, me_y, V = utb_cross_section(spec, v_gate, v_drain, dy_nm=dy_nm, **kw)
    me_x = np.asarray(mat["me_x"], dtype=float)[:, :, :1]
    mat.update({"Ny": len(y), "dy": dy_nm, "y": y, "me_y": me_y, "V": V, "me_x": np.repeat(me_x, len(y), axis=2)})
    esub, vsub = solve_subbands(mat)
    ef_l = float(esub[:, 0, :].min()) + spec.fermi_offset_ev
    return mat, esub, vsub, ef_l, ef_l - v_drain
