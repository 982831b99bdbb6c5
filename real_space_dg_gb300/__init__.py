"""GB300-native (sm_103a) Wigner-transport solve.

A from-scratch CUDA implementation of the 1D phase-space Wigner solve of the
MATLAB simulator jonasneu1207/real_space_DG, behind a C ABI
(include/wigner_gb300.h, libwigner_gb300.so) with a Python mirror of the
reference's MATLAB interface (``solve_transport_DG_2D``).
"""
from ._lib import WignerError, load  # noqa: F401
from .transport import Problem1D, solve_transport_DG_2D  # noqa: F401
