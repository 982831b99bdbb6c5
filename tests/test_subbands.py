"""Transverse subband eigensolve (solve_subbands.m): the oracle pinned to closed forms and to
shift-invert eigs (the algorithm behind the reference's eigs(Ht, n, 'sm')), and the CUDA
solver (libwigner_gb300.so, wg_subbands_*) against the oracle."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import subbands as S


def rand_mat(seed, nv=2, nx=24, ny=40, nm=6, shift=0.0, dy=0.25):
    """Seeded slices with random positive masses at every grid point (non-symmetric end
    rows) and random smooth potentials (eigenvalues of both signs)."""
    rng = np.random.default_rng(seed)
    me = rng.uniform(0.05, 0.6, (nv, nx, ny))
    yy = np.linspace(0.0, 1.0, ny)
    V = np.zeros((nx, ny))
    for ix in range(nx):
        c = rng.normal(size=4)
        V[ix] = 0.3 * (c[0] * np.sin(np.pi * yy) + c[1] * np.sin(2 * np.pi * yy) + c[2] * np.cos(3 * np.pi * yy)) \
            + shift + 0.2 * c[3]
    return dict(n_of_modes=nm, n_of_valleys=nv, Nx=nx, Ny=ny, dy=dy, me_y=me, V=V)


def utb_mat(nx_keep=40, v_gate=0.3, v_drain=0.4, nm=8):
    from real_space_dg_gb300 import devices
    spec = devices.FETSpec()
    x, y, me, V = devices.utb_cross_section(spec, v_gate, v_drain)
    sel = np.linspace(0, len(x) - 1, nx_keep).round().astype(int)
    return dict(n_of_modes=nm, n_of_valleys=me.shape[0], Nx=nx_keep, Ny=len(y), dy=0.1, me_y=me[:, sel],
                V=V[sel])


# ------------------------------------------------------------------------------------------ oracle

def test_oracle_box_spectrum_closed_form():
    E, V = S.solve_bandstructure(np.full(40, 0.19), np.full(40, 0.1), 0.25, 6)
    Eb, Vb = S.box_spectrum(40, 0.19, 0.25, 0.1, 6)
    assert np.abs(E - Eb).max() < 1e-12
    assert np.abs(V - Vb).max() < 1e-12


def test_oracle_hamiltonian_rows():
    """eval_transversal_Hamiltonian.m:20-37: harmonic-mean hopping, copied end rows."""
    rng = np.random.default_rng(1)
    m = rng.uniform(0.1, 0.5, 9)
    V = rng.normal(size=9)
    H = S.transversal_hamiltonian(m, V, 0.2)
    t0 = S.hopping_scale(0.2)
    for i in range(1, 8):
        assert H[i, i - 1] == -2 * t0 / (m[i - 1] + m[i])
        assert H[i, i + 1] == -2 * t0 / (m[i + 1] + m[i])
        assert abs(H[i, i] - (-(H[i, i - 1] + H[i, i + 1]) + V[i])) < 1e-12
    assert H[0, 0] == H[1, 1] and H[0, 1] == H[1, 2]
    assert H[8, 8] == H[7, 7] and H[8, 7] == H[7, 6]
    assert H[1, 0] != H[0, 1]                      # the end rows break the symmetry
    assert np.count_nonzero(H) == 3 * 9 - 2


@pytest.mark.parametrize("shift", [0.0, -1.0])
def test_oracle_matches_shift_invert_eigs(shift):
    """The oracle's dense eig + smallest-magnitude selection equals ARPACK shift-invert at 0 (what
    eigs(Ht, n, 'sm') computes) on slices with eigenvalues of both signs."""
    mat = rand_mat(3, nx=4, shift=shift)
    for ix in range(4):
        H = S.transversal_hamiltonian(mat["me_y"][0, ix], mat["V"][ix], mat["dy"])
        w, v = spla.eigs(sp.csc_matrix(H), k=6, sigma=0.0)
        order = np.argsort(w.real)
        E, Vo = S.solve_bandstructure(mat["me_y"][0, ix], mat["V"][ix], mat["dy"], 6)
        assert np.abs(E - w.real[order]).max() < 1e-10
        for k in range(6):
            u = np.real(v[:, order[k]])
            u = np.sign(u[-1]) * u / np.linalg.norm(u)
            assert np.abs(u - Vo[k]).max() < 1e-8


def test_oracle_smallest_magnitude_window():
    mat = rand_mat(0, nx=3, shift=-1.0)
    for ix in range(3):
        H = S.transversal_hamiltonian(mat["me_y"][1, ix], mat["V"][ix], mat["dy"])
        w = np.sort(np.linalg.eigvals(H).real)
        E, _ = S.solve_bandstructure(mat["me_y"][1, ix], mat["V"][ix], mat["dy"], 6)
        want = np.sort(w[np.argsort(np.abs(w))[:6]])
        assert (w < 0).any() and np.abs(E - want).max() < 1e-12


def test_oracle_cleanup_restores_flipped_vectors():
    """solve_subbands.m:22-40: a valley-1 vector anti-aligned with slice 1 is flipped back; slice 1
    and the other valleys are left alone."""
    mat = rand_mat(2, nx=6)
    _, Vs = S.solve_subbands(mat)
    bad = Vs.copy()
    hits = [(ix, m) for ix in range(1, 6) for m in range(6) if np.sum(Vs[0, 0, m] * Vs[0, ix, m]) > 0.5]
    assert hits
    for ix, m in hits:
        bad[0, ix, m] *= -1
    bad[0, 0, 2] *= -1
    bad[1, 3, 0] *= -1
    fixed = S.cleanup_signs(bad)
    for ix, m in hits:
        assert np.array_equal(fixed[0, ix, m], Vs[0, ix, m]) or np.sum(bad[0, 0, m] * bad[0, ix, m]) >= -0.5
    assert np.array_equal(fixed[0, 0], bad[0, 0]) and np.array_equal(fixed[1], bad[1])


# ------------------------------------------------------------------------------------------ GPU

@pytest.mark.gpu
def test_gpu_box_spectrum(built_lib):
    from real_space_dg_gb300.subbands import SubbandSolver
    nx, ny, nm = 5, 64, 10
    with SubbandSolver(1, nx, ny, nm) as s:
        E, V = s.solve(np.full((1, nx, ny), 0.19), np.full((nx, ny), 0.1), 0.25)
    Eb, Vb = S.box_spectrum(ny, 0.19, 0.25, 0.1, nm)
    assert np.abs(E[0] - Eb[None]).max() < 1e-11
    assert np.abs(V[0] - Vb[None]).max() < 1e-9


def _compare(mat, E, V):
    """Eigenvalues to 1e-10 eV, vectors to 1e-8.  The reference fixes each vector's sign by its
    last entry (solve_bandstructure.m:28-30); for a state localised away from that end the entry
    is at round-off level and its sign is arbitrary in any eigensolver, so such a vector -- and,
    through the clean-up, valley 1's vectors of that mode when slice 1's is such a vector -- is
    compared up to sign."""
    Eo, Vo = S.solve_subbands(mat)
    assert np.abs(E - Eo).max() < 1e-10
    amb = np.abs(Vo[..., -1]) < 1e-10
    amb[0] |= amb[0, 0][None, :]
    d = np.abs(V - Vo).max(axis=-1)
    d = np.where(amb, np.minimum(d, np.abs(V + Vo).max(axis=-1)), d)
    assert d.max() < 1e-8
    assert amb.mean() < 0.5
    return Eo, Vo


@pytest.mark.gpu
@pytest.mark.parametrize("seed,shift", [(0, 0.0), (0, -1.0), (3, 0.0), (4, -1.0)])
def test_gpu_matches_oracle_random_slices(built_lib, seed, shift):
    """Random masses and potentials: eigenvalues of both signs (the window around zero), the
    non-symmetric end rows, and valley-1 sign flips (the oracle flips vectors in these cases)."""
    from real_space_dg_gb300.subbands import solve_subbands
    mat = rand_mat(seed, shift=shift)
    E, V = solve_subbands(mat)
    Eo, Vo = _compare(mat, E, V)
    raw = np.stack([S.solve_bandstructure(mat["me_y"][0, ix], mat["V"][ix], mat["dy"], 6)[1]
                    for ix in range(mat["Nx"])])
    assert np.any(raw != Vo[0])


@pytest.mark.gpu
@pytest.mark.parametrize("v_gate", [0.0, 0.6])
def test_gpu_matches_oracle_utb_fet(built_lib, v_gate):
    from real_space_dg_gb300.subbands import solve_subbands
    mat = utb_mat(v_gate=v_gate)
    E, V = solve_subbands(mat)
    _compare(mat, E, V)


@pytest.mark.gpu
def test_gpu_limits_and_sizes(built_lib):
    """ny = 3 (the smallest Ht), nm = ny, and 32 modes on a wide grid."""
    from real_space_dg_gb300.subbands import solve_subbands
    for nv, nx, ny, nm in [(1, 2, 3, 3), (2, 3, 5, 5), (1, 3, 300, 32)]:
        mat = rand_mat(7, nv=nv, nx=nx, ny=ny, nm=nm, dy=0.5)
        E, V = solve_subbands(mat)
        _compare(mat, E, V)


@pytest.mark.gpu
def test_gpu_batch_matches_single_problems(built_lib):
    """A batch of problems (here three devices sharing the masses) in one launch equals the
    problems solved one by one, the sign clean-up included (per problem, against its own first
    slice)."""
    from real_space_dg_gb300.subbands import SubbandSolver, solve_subbands
    mats = [rand_mat(s_, nv=2, nx=10) for s_ in (0, 3, 4)]
    me = mats[0]["me_y"]
    V = np.stack([m["V"] for m in mats])
    with SubbandSolver(2, 10, mats[0]["Ny"], mats[0]["n_of_modes"], batch=3) as s:
        E, Vs = s.solve(me, V, mats[0]["dy"])
    for b, m in enumerate(mats):
        m = dict(m, me_y=me)
        E1, V1 = solve_subbands(m)
        assert np.array_equal(E[b], E1) and np.array_equal(Vs[b], V1)
        _compare(m, E[b], Vs[b])


@pytest.mark.gpu
def test_gpu_device_entry_matches_host(built_lib):
    import torch
    from real_space_dg_gb300.subbands import SubbandSolver
    mat = rand_mat(5)
    nv, nx, ny, nm = 2, mat["Nx"], mat["Ny"], mat["n_of_modes"]
    with SubbandSolver(nv, nx, ny, nm) as s:
        E, V = s.solve(mat["me_y"], mat["V"], mat["dy"])
        me = torch.tensor(mat["me_y"], device="cuda:0")
        pot = torch.tensor(mat["V"], device="cuda:0")
        Ed = torch.empty((nv, nx, nm), dtype=torch.float64, device="cuda:0")
        Vd = torch.empty((nv, nx, nm, ny), dtype=torch.float64, device="cuda:0")
        stream = torch.cuda.current_stream()
        s.solve_device(mat["dy"], me.data_ptr(), pot.data_ptr(), Ed.data_ptr(), Vd.data_ptr(), stream.cuda_stream)
        s.status(stream.cuda_stream)
        assert np.array_equal(Ed.cpu().numpy(), E) and np.array_equal(Vd.cpu().numpy(), V)


@pytest.mark.gpu
def test_gpu_argument_errors(built_lib):
    from real_space_dg_gb300 import WignerError
    from real_space_dg_gb300.subbands import SubbandSolver
    for shape in [(1, 4, 2, 1), (1, 4, 8, 9), (1, 4, 64, 33), (0, 4, 8, 2), (1, 4, 2000, 4)]:
        with pytest.raises(WignerError):
            SubbandSolver(*shape)
    with pytest.raises(WignerError):
        SubbandSolver(1, 4, 8, 2, batch=0)
    with SubbandSolver(1, 2, 8, 2) as s:
        me = np.full((1, 2, 8), 0.2)
        me[0, 1, 3] = -0.1
        with pytest.raises(WignerError):
            s.solve(me, np.zeros((2, 8)), 0.1)
        with pytest.raises(WignerError):
            s.solve(np.full((1, 2, 8), 0.2), np.full((2, 8), np.nan), 0.1)
        with pytest.raises(WignerError):
            s.solve(np.full((1, 2, 8), 0.2), np.zeros((2, 8)), 0.0)
        E, _ = s.solve(np.full((1, 2, 8), 0.2), np.zeros((2, 8)), 0.1)     # usable after the errors
        assert np.all(np.isfinite(E))


@pytest.mark.gpu
def test_gpu_utb_fet_feeds_transport(built_lib):
    """make_utb_fet: GPU subbands of the resolved cross-section -> solve_transport_DG_2D."""
    from real_space_dg_gb300 import devices
    from real_space_dg_gb300.transport import solve_transport_DG_2D
    spec = devices.FETSpec(n_el=40, nk=64, n_modes=2)
    mat, esub, vsub, efl, efr = devices.make_utb_fet(spec, 0.4, 0.2)
    Eo, Vo = S.solve_subbands(mat)
    assert np.abs(esub - Eo).max() < 1e-10 and np.abs(vsub - Vo).max() < 1e-8
    assert vsub.shape == (2, mat["Nx"], 2, mat["Ny"])
    DG = solve_transport_DG_2D(mat, esub, vsub, efl, efr, tol=1e-8, maxit=300, return_info=False)
    assert np.all(np.isfinite(DG["n"])) and np.all(np.isfinite(DG["j"]))
