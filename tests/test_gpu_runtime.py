"""CUDA-graph replay of the Arnoldi steps and the autotuned launch shapes.

Tolerances: a solve replayed from CUDA graphs equals the eagerly launched solve
bit for bit (the same kernels with the same arguments in the same order); the
FP32 xi stencil gives bit-identical results with 2 and 4 cells per thread (the
same FP32 operations per cell); the k-line preconditioner with any chunk length
matches the oracle's sequential sweep to 1e-12 (the chunks re-associate the
element recurrence, FP64).
"""
import numpy as np
import pytest

from conftest import small_rtd
from oracle import dg1d, krylov

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def det_vec(n):
    i = np.arange(1, n + 1, dtype=float)
    return np.sin(i) + 1j * np.cos(i)


def make(spec, **kw):
    from real_space_dg_gb300 import Problem1D
    return Problem1D(n_el=spec.n_el, n_local=spec.n_local, nk=spec.nk, n_xi=spec.n_xi or spec.nk,
                     l_xi=spec.l_xi_m, **kw)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_equals_eager_solve(built_lib, precision):
    """Solve 1 runs every Arnoldi chunk eagerly, solve 2 captures the chunks, solve 3
    replays them: all three give the same bits."""
    specs = [small_rtd(n_el=14, nk=32, order=2, bias=v) for v in (0.05, 0.2)]
    spec0 = specs[0][0]
    with make(spec0, batch=2, precision=precision, restart=12, inner_restart=8) as P:
        for b, (spec, mat, E, efl, efr, m) in enumerate(specs):
            P.set_potential(b, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        rhos = []
        for _ in range(3):
            st, info = P.solve(tol=1e-10, maxit=80)
            assert st == 0, info
            rhos.append(np.concatenate([P.rho(b) for b in range(2)]))
        stats = P.runtime_stats
    assert stats["graphs_disabled"] == 0 and stats["graphs_captured"] > 0 and stats["graph_replays"] > 0, stats
    assert np.array_equal(rhos[0], rhos[1]) and np.array_equal(rhos[0], rhos[2])


def test_stencil_cells_give_identical_bits(built_lib):
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=64, order=3)
    with make(spec, precision="mixed") as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        x = det_vec(P.N)
        out = {}
        for cells in (2, 4):
            P.set_launch_shapes(stencil_cells=cells)
            out[cells] = P.apply_lowprec(x)
    assert np.array_equal(out[2], out[4])


def test_kline_chunk_lengths_match_oracle(built_lib):
    spec, mat, E, efl, efr, m = small_rtd(n_el=24, nk=32, order=2)
    p = dg1d.init_params(mat, efl, efr, E, m)
    op = krylov.Operator1D(mat, p, E)
    ref = krylov.KLinePreconditioner(op, use_drift_diag=False)
    x = None
    with make(spec) as P:
        P.set_potential(0, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
        x = det_vec(P.N)
        want = ref.apply(x)
        for L in (1, 2, 3, 5, 8, 24):
            P.set_launch_shapes(kline_chunk=L)
            assert P.runtime_stats["kline_chunk"] == L
            assert rel(P.precondition(x), want) < 1e-12, L


def test_autotuner_picks_valid_shapes_and_caches_them(built_lib):
    spec, mat, E, efl, efr, m = small_rtd(n_el=40, nk=32, order=2)
    shapes = []
    for batch in (1, 3):
        with make(spec, batch=batch, precision="mixed") as P:
            for b in range(batch):
                P.set_potential(b, mat["x"], E, m, spec.m_rel, spec.temp_k, efl, efr)
            assert P.runtime_stats["tuned"] == 0
            st, _ = P.solve(tol=1e-10, maxit=80)
            assert st == 0
            s = P.runtime_stats
            assert s["tuned"] == 1 and s["stencil_cells"] in (2, 4)
            assert 1 <= s["kline_chunk"] <= spec.n_el and -(-spec.n_el // s["kline_chunk"]) <= 64
            shapes.append((s["kline_chunk"], s["stencil_cells"]))
    assert shapes[0] == shapes[1]          # one choice per shape, whatever the batch


def test_launch_shape_arguments_are_checked(built_lib):
    from real_space_dg_gb300 import WignerError
    spec, mat, E, efl, efr, m = small_rtd(n_el=10, nk=32, order=2)
    with make(spec) as P:
        for bad in (dict(kline_chunk=11), dict(kline_chunk=-1), dict(stencil_cells=3)):
            with pytest.raises(WignerError):
                P.set_launch_shapes(**bad)
