"""Generate the golden fixtures of the 1D Wigner path from the CPU oracle.

The reference (MATLAB) cannot run in this environment and ships no golden
vectors for its 1D k-basis path, so the fixtures are outputs of the oracle
restatement (oracle/dg1d.py) at small sizes.  They freeze the oracle's answer
so that regressions of either side are caught without re-running the oracle,
and they travel to the GPU machine with the tests.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from conftest import small_rtd  # noqa: E402
from oracle import dg1d, jacobi  # noqa: E402

CASES = {
    # name: (n_el, nk, order, n_xi, bias)
    "p2_nk32": (12, 32, 2, 0, 0.1),
    "p1_nk16_nxi20": (10, 16, 1, 20, 0.05),
    "p3_nk24": (8, 24, 3, 0, 0.2),
}


def deterministic_vector(n):
    """sin(i) + i cos(i), the reference's test vector (full2DDriftSystemSolveTest.m:613-615)."""
    i = np.arange(1, n + 1, dtype=float)
    return np.sin(i) + 1j * np.cos(i)


def make_case(name, n_el, nk, order, n_xi, bias):
    spec, mat, E, efl, efr, m = small_rtd(n_el=n_el, nk=nk, order=order, n_xi=n_xi, bias=bias)
    p = dg1d.init_params(mat, efl, efr, E, m)
    A, rhs = dg1d.get_sysm(mat, p, E)
    x = deterministic_vector(A.shape[0])
    rho = spla.spsolve(A.tocsc(), rhs)
    n_dg, j, rho_u = dg1d.observables(p, rho, dg1d.node_map(p, m))
    return dict(E=E, efl=efl, efr=efr, x_nm=mat["x"], m=m, Ax=A @ x, rhs=rhs, rho=rho, n_dg=n_dg, j=j,
                fnl=p["fnl"], fnr=p["fnr"], phi=p["phi"], k=p["k"],
                shape=np.array([n_el, nk, order, n_xi or nk]), bias=bias)


def main():
    out = {}
    for name, args in CASES.items():
        for key, val in make_case(name, *args).items():
            out[name + "/" + key] = val
    for n in (1, 2, 3, 4, 9):
        x, w = jacobi.jacobi_gl(0, 0, n)
        out["gl%d/x" % n] = x
        out["gl%d/w" % n] = w
    np.savez_compressed(os.path.join(HERE, "wigner1d_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "wigner1d_golden.npz"))


if __name__ == "__main__":
    main()
