"""Freeze the contact reservoirs of the reference's recorded Full-2D run into a small fixture.

Reads 2026-10-28_08-47/Sim_Res.mat of the reference project (run here, where the reference is
present; the fixture travels instead): the inputs of the Source/Drain contact-mode reservoirs (the
material Y grid, the contact-edge potentials of the last bias point, masses, temperature,
degeneracy and the DG parameters), the whole potential of that bias point (the Full-2D system the
benchmark solves), the density and current the reference's transport solve returned for it (with
its GMRES relative residual), and the outputs boundary.physical.XLeft/XRight.rhoBoundary with the
mode energies and Fermi levels the reference stored beside them; for the sweep's first bias point
(0 V) the device fields (Vc, eps, Nd, contact lengths), the converged potential and density and
the Gummel loop's per-iteration history; for the whole sweep the bias, the mean current, the Gummel
iterations and the GMRES iterations of every bias point.

    python tests/golden/make_reservoir_golden.py /path/to/reference
"""
import os
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    d = sio.loadmat(os.path.join(ref_root, "2026-10-28_08-47", "Sim_Res.mat"), squeeze_me=True,
                    struct_as_record=False)
    mat = d["mat"]
    prm = mat.dg.params
    pot = np.asarray(d["sweep"].potential)[:, :, -1]
    out = dict(y=np.asarray(mat.y, dtype=float), x=np.asarray(mat.x, dtype=float), Nx=int(mat.Nx), Ny=int(mat.Ny),
               v_source=pot[0], v_drain=pot[-1], potential=pot, bias=float(np.ravel(d["sweep"].bias)[-1]),
               density=np.asarray(d["sweep"].density, dtype=float)[:, :, -1],
               current=np.asarray(d["sweep"].current, dtype=float)[:, -1],
               relres=float(np.ravel(d["sweep"].relres)[-1]),
               me_x_ch=float(mat.me_x_ch), me_y_ch=float(mat.me_y_ch),
               me_z_ch=float(mat.me_z_ch), deg_factor=float(np.ravel(mat.deg_factor)[0]), Temp=float(mat.Temp))
    for name in ("N_K_X", "N_K_Y", "N_el_X", "N_el_Y", "N_rho_x", "N_rho_y", "L_rho_x", "L_rho_y",
                 "full2D_contactMode_Nkx", "full2D_contactMode_Nkz", "full2D_sourceContactSheetDensity",
                 "full2D_drainContactSheetDensity", "full2D_contactModeIntegrateKz"):
        out["prm_" + name] = float(getattr(prm, name))
    # the self-consistent sweep's first bias point: device fields, the converged potential and the
    # per-iteration history of the Gummel loop (solve2D_rtd_self_consistent.m)
    out.update(Vc=np.asarray(mat.Vc, dtype=float), eps=np.asarray(mat.eps, dtype=float),
               Nd=np.asarray(mat.Nd, dtype=float), Lc1=float(mat.Lc1), Lc2=float(mat.Lc2), dx=float(mat.dx),
               dy=float(mat.dy), potential0=np.asarray(d["sweep"].potential, dtype=float)[:, :, 0],
               density0=np.asarray(d["sweep"].density, dtype=float)[:, :, 0],
               iterations0=int(np.ravel(d["sweep"].iterations)[0]))
    # the whole recorded I-V sweep: bias, mean current (results.Id), Gummel iterations per bias
    out.update(sweep_bias=np.asarray(d["sweep"].bias, dtype=float),
               sweep_id=np.asarray(d["sweep"].current, dtype=float).mean(axis=0),
               sweep_iterations=np.asarray(d["sweep"].iterations, dtype=float),
               sweep_gmres=np.array([sum(h.gmresIterations for h in np.atleast_1d(hb))
                                     for hb in d["selfConsistency"].history], dtype=float))
    hist = d["selfConsistency"].history[0]
    out["history0"] = np.array([[h.gmresIterations, h.potentialDefect, h.densityChange, h.poissonPhysicalRelres]
                                for h in hist], dtype=float)
    for side, key in (("XLeft", "source"), ("XRight", "drain")):
        s = getattr(d["boundary"].physical, side)
        out["rho_" + key] = np.asarray(s.rhoBoundary, dtype=float)
        out["ef_input_" + key] = float(s.fermiLevelInput)
        out["ef_used_" + key] = float(s.fermiLevel)
        out["modes_" + key] = np.asarray(s.dataInfo.defaultReservoir.modeEnergy, dtype=float)
    np.savez_compressed(os.path.join(HERE, "full2d_reservoir_golden.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_reservoir_golden.py /path/to/reference")
    main(sys.argv[1])
