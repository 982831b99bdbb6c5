"""CPU oracle for the Wigner-transport hot path (TEST INFRASTRUCTURE ONLY).

This package restates, in NumPy/SciPy, the MATLAB algorithm of the reference
simulator's 1D phase-space (x, xi->k) Wigner solve and its self-consistency
loop.  It is the parity checker for the CUDA library in ``real_space_dg_gb300``
and the timed CPU baseline of ``bench.py``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it.  The product path never calls into this package.

Parity status: the reference ships no golden vectors or unit tests for the 1D
k-basis path (its tests cover only the Full-2D operator) and MATLAB/Octave is
not available to run it.  The restatement is pinned by (i) the reference's own
closed-form facts (Gauss-Lobatto nodes/weights, mass/stiffness identities),
(ii) agreement of the two reference assembly forms that exist for the drift
operator (the index-table form of get_Drift_accel_trial_permutedShell.m and
the loop form of get_Drift.m), restated independently here, and (iii) the
reference's invariants restated for 1D (matrix-free == assembled, constant
potential => zero Wigner-potential term).  Against outputs of the reference
itself the oracle is "parity unpinned".
"""
