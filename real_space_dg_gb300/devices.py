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
