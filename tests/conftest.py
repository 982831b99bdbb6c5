import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libwigner_gb300.so)")


@pytest.fixture(scope="session")
def built_lib():
    """Build libwigner_gb300.so in-tree (nvcc cross-compiles without a GPU)."""
    from real_space_dg_gb300 import build
    return build.build()


def small_rtd(n_el=12, nk=32, order=2, n_xi=0, bias=0.1, **kw):
    """A short RTD that the oracle's sparse LU solves in well under a second."""
    from real_space_dg_gb300 import devices
    import numpy as np
    args = dict(n_el=n_el, nk=nk, order=order, n_xi=n_xi, length_nm=30.0, contact_nm=8.0, well_nm=4.0,
                barrier_nm=2.0)
    args.update(kw)
    spec = devices.RTDSpec(**args)
    mat = devices.make_mat(spec)
    E = devices.flatband_potential(mat, bias)
    efl, efr = devices.contact_fermi_levels(mat, bias)
    m = np.full(mat["Nx"], spec.m_rel * 9.109e-31)
    return spec, mat, E, efl, efr, m
