"""Serving: continuous batching of self-consistent bias points (wg_server_*).

Tolerances: a request gives the same result alone and inside a mix of other
requests and shapes -- bit-identical is expected (every slot's arithmetic is
independent of the others); the test allows 1e-12 V on the potential and 1e-10
relative on n and j.  Warm-started points reach the cold-start fixed points
within the Gummel tolerance (potential 1e-6 V: compared at 2e-5 V, current
1e-3 relative).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import small_rtd

pytestmark = pytest.mark.gpu

OPTS = dict(mixing=0.5, potentialTolerance=1e-6, densityTolerance=1e-5, maxIterations=150,
            transportTolerance=1e-10, transportMaxCycles=60, precision="mixed")


def _mats():
    from real_space_dg_gb300 import devices
    out = []
    for kw in (dict(n_el=10, nk=32, order=2), dict(n_el=12, nk=32, order=1)):
        spec, mat, *_ = small_rtd(**kw)
        out.append(dict(mat, dy_norm_nm=devices.density_normalisation_nm(mat)))
    return out


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def test_same_alone_and_in_the_mix(built_lib):
    from real_space_dg_gb300.rtd import RTDSweep
    from real_space_dg_gb300.serve import Server, serve_sweep
    matA, matB = _mats()
    with Server(OPTS, warm_start=False, max_slots=3) as S:
        alone = S.wait(S.submit(matA, 0.1, device_key=1))
    assert alone["state"] == "done" and alone["status"] == "fixed-point-converged", alone["error"]
    # the same point through the batch API with one problem
    R = RTDSweep(matA, 1, OPTS)
    try:
        R.set(0, 0.1)
        st, _ = R.run()
        phi_b, n_b, j_b = R.get(0)
    finally:
        R.close()
    assert st == 0
    assert np.abs(alone["phi"] - phi_b).max() <= 1e-12
    # a mix of two shapes arriving while earlier requests iterate
    jobs = [(matA, v, 1) for v in (0.0, 0.05, 0.1, 0.15, 0.2)] + [(matB, v, 2) for v in (0.05, 0.1, 0.15)]
    arrivals = np.arange(len(jobs)) * 0.03
    with Server(OPTS, warm_start=False, max_slots=3) as S:
        res, wall = serve_sweep(S, jobs, arrivals)
        stats = S.stats()
    assert all(r["state"] == "done" and r["status"] == "fixed-point-converged" for r in res), \
        [(r["state"], r["status"]) for r in res]
    mixed = res[2]
    assert np.abs(mixed["phi"] - alone["phi"]).max() <= 1e-12
    assert rel(mixed["n"], alone["n"]) <= 1e-10 and rel(mixed["j"], alone["j"]) <= 1e-10
    # continuous batching: a request entered a handle while another of that handle was running
    joined = any(a["handle"] == b["handle"] and b["t_admit"] < a["t_admit"] < b["t_done"]
                 for a in res for b in res if a is not b)
    assert joined
    # both shapes were on the device at the same time
    hA = [r for r in res[:5]]
    hB = [r for r in res[5:]]
    assert min(r["t_admit"] for r in hB) < max(r["t_done"] for r in hA)
    assert stats["failed"] == 0 and stats["done"] == len(jobs)


def test_memory_budget_admission(built_lib):
    from real_space_dg_gb300 import _lib
    from real_space_dg_gb300.serve import Server, serve_sweep
    from real_space_dg_gb300.transport import shape_from_mat
    lib = _lib.load()
    matA, matB = _mats()
    need = []
    for mat in (matA, matB):
        shp = shape_from_mat(mat)
        prm = _lib.WgParams(shp["n_el"], shp["n_local"], shp["nk"], shp["n_xi"], shp["l_xi"], 0.0, 1.0,
                            _lib.WG_PREC_MIXED, 50, 0.0, 40, 1e-3)
        b = C.c_double()
        assert lib.wg_problem_bytes(C.byref(prm), 2, C.byref(b)) == 0
        need.append(b.value)
    budget = max(need) * 1.05            # room for one two-slot handle at a time
    jobs = [(matA, v, 1) for v in (0.05, 0.1, 0.15)] + [(matB, v, 2) for v in (0.05, 0.1)]
    with Server(OPTS, mem_budget_bytes=budget, max_slots=2, idle_release_s=0.02) as S:
        res, _ = serve_sweep(S, jobs)
        stats = S.stats()
    assert all(r["state"] == "done" for r in res)
    assert stats["device_bytes_peak"] <= budget
    # the second shape waited for the first handle to be released
    first = min(res, key=lambda r: r["t_admit"])
    other = [r for r in res if r["handle"] != first["handle"]]
    same = [r for r in res if r["handle"] == first["handle"]]
    assert other and min(r["t_admit"] for r in other) >= max(r["t_done"] for r in same)


def test_warm_start_from_neighbouring_bias(built_lib):
    from real_space_dg_gb300.serve import Server
    matA, _ = _mats()
    biases = [0.0, 0.04, 0.08, 0.12, 0.16, 0.2]
    out = {}
    for warm in (False, True):
        with Server(OPTS, warm_start=warm, max_slots=2) as S:
            rs = [S.wait(S.submit(matA, v, device_key=7)) for v in biases]   # one after another: a sweep
        assert all(r["status"] == "fixed-point-converged" for r in rs)
        out[warm] = rs
    assert all(r["warm"] == 0 for r in out[False])
    assert all(r["warm"] == 2 for r in out[True][1:])      # slot with the neighbour's state resident
    its = {w: sum(r["info"]["iterations"] for r in out[w][1:]) for w in out}
    assert its[True] < its[False]
    for a, b in zip(out[True], out[False]):
        assert np.abs(a["phi"] - b["phi"]).max() < 2e-5
        assert rel(a["j"], b["j"]) < 1e-3
