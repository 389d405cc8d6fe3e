"""The fused, graph-replayed NVE runner against the per-step API and the oracle.

The runner (jmd_nve_run) fuses both half kicks, the drift and the skin test
into the force kernel and gates each step's rebuild with a device-side
conditional graph node.  Graph and direct launches must agree bit for bit;
against the per-step API (which checks the skin one step earlier, as the
reference loop does) and the FP64 oracle, trajectories agree to fp32 accuracy
over short runs.  The sorted run is tested with both of its private lists:
the segment-local list (16-bit slots of a shared-memory staged neighbourhood)
and the tiled int32 list.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import LJ_DT, fcc_system, lj_spec

pytestmark = pytest.mark.gpu


def _setup(cuda, n_cells=6, skin=0.3):
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(n_cells)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=skin, format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nve(efn, shift, LJ_DT)
    st = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    return R, P, L, nfn, efn, init, apply, st, nb


# (sort, layout) of a run: unsorted, sorted with the segment-local list
# (full or half lists), sorted with the tiled list
RUNS = [(False, None), (True, 'segment'), (True, 'half'), (True, 'tiled')]
RUN_IDS = ['unsorted', 'segment', 'half', 'tiled']


@pytest.mark.parametrize('sort,layout', RUNS, ids=RUN_IDS)
@pytest.mark.parametrize('steps', [1, 2, 7, 40])
def test_graph_equals_direct(cuda, steps, sort, layout):
    from jax_md_gb300 import simulate
    _, _, _, nfn, efn, init, apply, st_a, nb_a = _setup(cuda)
    _, _, _, nfn2, _, _, apply2, st_b, nb_b = _setup(cuda)
    simulate.run(apply, st_a, nb_a, steps, use_graph=True, sort=sort, layout=layout)
    simulate.run(apply2, st_b, nb_b, steps, use_graph=False, sort=sort, layout=layout)
    torch.cuda.synchronize()
    if layout == 'half':
        # half lists add reactions with float atomics: the summation order,
        # and so the last bits, may differ between any two runs, and the
        # difference grows over a run (forces reach ~15 on this lattice);
        # accuracy against the oracle is tested to 1e-4 elsewhere
        assert (st_a.position - st_b.position).abs().max().item() < 1e-5
        assert (st_a.momentum - st_b.momentum).abs().max().item() < 1e-3
        assert (st_a.force - st_b.force).abs().max().item() < 1e-3
    else:
        assert torch.equal(st_a.position, st_b.position)
        assert torch.equal(st_a.momentum, st_b.momentum)
        assert torch.equal(st_a.force, st_b.force)
        assert torch.equal(nb_a.idx, nb_b.idx)
    assert int(nb_a.error.code) == int(nb_b.error.code) == 0


def test_graph_replay_repeats(cuda):
    """A cached graph replayed twice equals one direct run of twice the length."""
    from jax_md_gb300 import simulate
    _, _, _, _, _, _, apply, st_a, nb_a = _setup(cuda)
    _, _, _, _, _, _, apply2, st_b, nb_b = _setup(cuda)
    simulate.run(apply, st_a, nb_a, 10)
    simulate.run(apply, st_a, nb_a, 10)
    for _ in range(2):
        simulate.run(apply2, st_b, nb_b, 10, use_graph=False)
    torch.cuda.synchronize()
    assert torch.equal(st_a.position, st_b.position)


@pytest.mark.parametrize('n_cells', [6, 10])
@pytest.mark.parametrize('sort,layout', RUNS, ids=RUN_IDS)
def test_runner_matches_per_step_api_and_oracle(cuda, sort, layout, n_cells):
    from jax_md_gb300 import simulate
    R, P, L, nfn, efn, init, apply, st, nb = _setup(cuda, n_cells=n_cells)
    _, _, _, nfn2, efn2, init2, apply2, st2, nb2 = _setup(cuda, n_cells=n_cells)
    steps = 40
    simulate.run(apply, st, nb, steps, sort=sort, layout=layout)
    for _ in range(steps):
        nb2 = nb2.update(st2.position)
        st2 = apply2(st2, neighbor=nb2)
    torch.cuda.synchronize()
    box = np.full(3, L)
    d = O.displacement(st.position.cpu().numpy(), st2.position.cpu().numpy(), box)
    assert np.abs(d).max() < (1e-4 if sort else 1e-5)
    # oracle trajectory
    spec = lj_spec()
    nl = O.NeighborListOracle(box, 2.5, 0.3)
    h = {'nb': nl.allocate(R)}

    def fn(X):
        h['nb'] = nl.update(X, h['nb'])
        return O.pair_energy_forces(spec, X, h['nb'].idx, O.DENSE, box)[1]
    Rd, Pd = R.astype(np.float64), P.astype(np.float64)
    F = fn(Rd)
    for _ in range(steps):
        Rd, Pd, F = O.velocity_verlet(fn, Rd, Pd, F, 1.0, LJ_DT, box)
    X = st.position.contiguous().cpu().numpy()
    d = O.displacement(X, Rd, box)
    assert np.abs(d).max() < 1e-4
    # forces of the final state against the oracle on the same positions
    _, Fx, _ = O.pair_energy_forces(spec, X, nb.idx.cpu().numpy(), O.DENSE, box)
    assert np.abs(st.force.cpu().numpy() - Fx).max() < 1e-4


def test_always_rebuild_mode(cuda):
    """dr_threshold = 0 rebuilds every step (partition.py:1141-1144)."""
    from jax_md_gb300 import simulate
    R, P, L, nfn, efn, init, apply, st, nb = _setup(cuda, skin=0.0)
    _, _, _, _, _, _, apply2, st2, nb2 = _setup(cuda, skin=0.0)
    simulate.run(apply, st, nb, 5)
    for _ in range(5):
        nb2 = nb2.update(st2.position)
        st2 = apply2(st2, neighbor=nb2)
    torch.cuda.synchronize()
    d = O.displacement(st.position.cpu().numpy(), st2.position.cpu().numpy(), np.full(3, L))
    assert np.abs(d).max() < 1e-5


def test_overflow_reallocates(cuda):
    """A list allocated too small overflows; run(neighbor_fn=...) restores and re-allocates."""
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(6)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3, format=partition.Dense,
                                                  capacity_multiplier=1.0)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)                      # no headroom over the lattice's occupancy
    init, apply = simulate.nve(efn, shift, LJ_DT)
    st = init(0, Rt, momenta=3.0 * torch.tensor(P, device=cuda), neighbor=nb)
    first = nb.max_occupancy
    st, nb2 = simulate.run(apply, st, nb, 300, neighbor_fn=nfn)
    torch.cuda.synchronize()
    assert not bool(nb2.did_buffer_overflow)
    assert nb2.max_occupancy > first
    assert torch.isfinite(st.position).all()


def test_sorted_run_returns_reference_order_list(cuda):
    """After a sorted run the caller's list is the reference's build at its reference positions."""
    from jax_md_gb300 import simulate
    R, P, L, nfn, efn, init, apply, st, nb = _setup(cuda, n_cells=8)
    simulate.run(apply, st, nb, 60, sort=True)
    torch.cuda.synchronize()
    box = np.full(3, L, np.float32)
    ref = nb.reference_position.contiguous().cpu().numpy()
    onl = O.NeighborListOracle(box, np.float32(2.5), np.float32(0.3))
    ob = onl.build(ref, nb.max_occupancy, 0, nb.cell_list_capacity)
    from tests.helpers import near_cutoff_pairs
    from tests.test_gpu_neighbor import _strict_equal_rows
    skip = near_cutoff_pairs(ref, box, float(np.float32(2.8)))
    assert _strict_equal_rows(nb.idx.cpu().numpy(), ob.idx, len(R), skip) == []
    # the list still covers the current positions (skin not exceeded since the rebuild)
    d = O.displacement(st.position.contiguous().cpu().numpy(), ref, box)
    assert ((d * d).sum(-1) <= (0.15 ** 2) * (1 + 1e-5) + 0.3 * 0.005).all()
    assert int(nb.error.code) == 0


def test_tiled_list_and_forces_match_row_major(cuda):
    """The engine's tiled layout holds the row-major list's entries in the same order per
    atom, and the thread-per-atom kernel gives the row-major kernel's forces."""
    import ctypes
    from jax_md_gb300 import _native as N, partition
    R, P, L, nfn, efn, init, apply, st, nb = _setup(cuda, n_cells=8)
    X = partition.padded_rows(torch.tensor(R, device=cuda))
    n = X.shape[0]
    plan = nb.plan
    depth = plan.ld
    tidx = torch.full((((n + 31) // 32) * 32 * depth,), -1, dtype=torch.int32, device=cuda)
    cnt = torch.zeros(n, dtype=torch.int32, device=cuda)
    occ = torch.zeros((), dtype=torch.int64, device=cuda)
    err = torch.zeros((), dtype=torch.uint8, device=cuda)
    ref = torch.zeros((n, 4), device=cuda)
    ws = torch.empty(plan.workspace.numel(), dtype=torch.uint8, device=cuda)
    L_ = N.lib()
    N.check(L_.jmd_neighbor_list_build_tiled(ctypes.byref(plan.nl), X.data_ptr(), n, tidx.data_ptr(),
                                             depth, cnt.data_ptr(), occ.data_ptr(), err.data_ptr(),
                                             ref.data_ptr(), None, ws.data_ptr(), ws.numel(),
                                             N.stream_ptr()))
    nb2 = nfn.allocate(X)
    assert torch.equal(cnt, nb2.nbr_count)
    t = tidx.reshape(-1, depth, 32).permute(0, 2, 1).reshape(-1, depth)[:n]
    rows = nb2.idx.cpu().numpy()
    tt = t.cpu().numpy()
    c = cnt.cpu().numpy()
    for i in range(0, n, 7):
        assert np.array_equal(tt[i, :c[i]], rows[i, :c[i]])
    species, pair = efn._resolve(X, {})
    sp = efn.geometry.space(3)
    F = torch.zeros((n, 4), device=cuda)
    N.check(L_.jmd_pair_forces_tiled(ctypes.byref(pair), ctypes.byref(sp), X.data_ptr(), None, n,
                                     tidx.data_ptr(), depth, nb2.max_occupancy, cnt.data_ptr(),
                                     F.data_ptr(), N.stream_ptr()))
    F0 = efn.forces(X, nb2)
    torch.cuda.synchronize()
    assert (F[:, :3] - F0).abs().max().item() < 2e-5


def _nvt_setup(cuda, n_cells=6, kT=0.722):
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(n_cells)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3, format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nvt_nose_hoover(efn, shift, LJ_DT, kT)
    st = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    return efn, init, apply, st, nb


@pytest.mark.parametrize('sort,layout', RUNS, ids=RUN_IDS)
def test_nvt_runner_matches_apply_loop(cuda, sort, layout):
    """simulate.run on a Nose-Hoover state (jmd_nvt_run / jmd_nvt_run_sorted)
    against the per-step apply_fn loop: same chain, same trajectory to fp32
    accuracy over 60 steps."""
    from jax_md_gb300 import simulate
    efn, init, apply, st_a, nb_a = _nvt_setup(cuda)
    _, _, apply_b, st_b, nb_b = _nvt_setup(cuda)
    steps = 60
    simulate.run(apply, st_a, nb_a, steps, sort=sort, layout=layout)
    for _ in range(steps):
        nb_b = nb_b.update(st_b.position)
        st_b = apply_b(st_b, neighbor=nb_b)
    torch.cuda.synchronize()
    assert (st_a.position - st_b.position).abs().max().item() < 1e-3
    assert (st_a.momentum - st_b.momentum).abs().max().item() < 1e-2
    ca, cb = st_a.chain.buffer.cpu().numpy(), st_b.chain.buffer.cpu().numpy()
    assert np.allclose(ca[:66], cb[:66], rtol=1e-3, atol=1e-6)


def test_nvt_runner_conserves_invariant(cuda):
    """The NVT invariant (simulate.py:672-701) of a 1000-step graph run drifts
    by less than 1e-3 per atom."""
    from jax_md_gb300 import simulate
    efn, init, apply, st, nb = _nvt_setup(cuda, n_cells=8)
    kT = 0.722
    H0 = float(simulate.nvt_nose_hoover_invariant(efn, st, kT, neighbor=nb))
    simulate.run(apply, st, nb, 1000)
    nb = nb.update(st.position)
    H1 = float(simulate.nvt_nose_hoover_invariant(efn, st, kT, neighbor=nb))
    n = st.position.shape[0]
    assert not bool(nb.did_buffer_overflow)
    assert abs(H1 - H0) / n < 1e-3, (H0, H1)
    T = float((st.momentum.double() ** 2).sum() / (3 * n))
    assert 0.5 < T < 1.0


@pytest.mark.parametrize('n_cells', [6, 10])
def test_segment_and_tiled_layouts_agree(cuda, n_cells):
    """The two private lists hold the same pairs: three steps from the same
    state give the same forces and positions to fp32 summation order (forces
    within the 1e-4 force tolerance: single pair forces reach ~50 on the
    jittered lattice)."""
    from jax_md_gb300 import simulate
    _, _, _, _, _, _, apply_a, st_a, nb_a = _setup(cuda, n_cells=n_cells)
    _, _, _, _, _, _, apply_b, st_b, nb_b = _setup(cuda, n_cells=n_cells)
    simulate.run(apply_a, st_a, nb_a, 3, layout='segment')
    simulate.run(apply_b, st_b, nb_b, 3, layout='tiled')
    torch.cuda.synchronize()
    assert (st_a.force - st_b.force).abs().max().item() < 1e-4
    assert (st_a.position - st_b.position).abs().max().item() < 1e-5
    assert simulate.last_run_status(st_a) == 0
    assert torch.equal(nb_a.idx, nb_b.idx)


@pytest.mark.parametrize('half', [False, True], ids=['full', 'half'])
@pytest.mark.parametrize('cells', [1, 2, 3, 4, 5, 8])
def test_segment_widths_match_oracle(cuda, cells, half):
    """Every segment width K gives forces within 1e-4 of the FP64 oracle at
    the run's own final positions (11 cells per side: K = 5 and 8 leave a
    shorter last segment in each row; K <= 3 stage in the CTA's periodic
    frame, wider segments take the minimum image per pair)."""
    from jax_md_gb300 import simulate
    spatial = pytest.importorskip('scipy.spatial')
    _, _, L, _, _, _, apply_a, st_a, nb_a = _setup(cuda, n_cells=20)
    threads = simulate.segment_threads_default(min(cells, 9), nb_a.plan.nl.cell_capacity)
    simulate.run(apply_a, st_a, nb_a, 5, layout=(cells, threads, 0, int(half)))
    torch.cuda.synchronize()
    assert simulate.last_run_status(st_a) == 0
    X = st_a.position.double().cpu().numpy()
    pairs = spatial.cKDTree(np.mod(X, L), boxsize=L).query_pairs(2.5, output_type='ndarray')
    idx = np.stack([pairs.min(1), pairs.max(1)])
    _, Fo, _ = O.pair_energy_forces(lj_spec(), X, idx, O.ORDERED_SPARSE, np.full(3, L))
    assert np.abs(st_a.force.cpu().numpy() - Fo).max() < 1e-4


def test_lazy_caller_list_is_built_when_read(cuda):
    """A sorted run leaves the caller's list for its first read; that read (or
    an update) gives the list an eager run returns."""
    from jax_md_gb300 import simulate
    _, _, _, _, _, _, apply_a, st_a, nb_a = _setup(cuda, n_cells=8)
    _, _, _, _, _, _, apply_b, st_b, nb_b = _setup(cuda, n_cells=8)
    simulate.run(apply_a, st_a, nb_a, 30, lazy_list=True)
    simulate.run(apply_b, st_b, nb_b, 30, lazy_list=False)
    assert nb_a.has_pending_build and not nb_b.has_pending_build
    assert torch.equal(nb_a.idx, nb_b.idx)
    assert not nb_a.has_pending_build
    # an update resolves the deferred build first, then tests the skin
    simulate.run(apply_a, st_a, nb_a, 30, lazy_list=True)
    simulate.run(apply_b, st_b, nb_b, 30, lazy_list=False)
    nb_a = nb_a.update(st_a.position)
    nb_b = nb_b.update(st_b.position)
    torch.cuda.synchronize()
    assert torch.equal(nb_a.idx, nb_b.idx)
    assert torch.equal(st_a.position, st_b.position)


@pytest.mark.parametrize('layout', ['segment', 'half', 'tiled'])
def test_sorted_engine_species_matches_per_step_api(cuda, layout):
    """A Kob-Andersen mixture (species matrices) through the sorted engine:
    the segment kernels read species from the private position rows."""
    from jax_md_gb300 import energy, partition, simulate, space
    rng = np.random.default_rng(3)
    n_side = 16
    L = float((n_side ** 3 / 1.2) ** (1 / 3))
    g = (np.arange(n_side) + 0.5) * (L / n_side)
    R = np.stack(np.meshgrid(g, g, g, indexing='ij'), -1).reshape(-1, 3)
    R = (R + rng.uniform(-0.05, 0.05, R.shape)).astype(np.float32) % np.float32(L)
    n = len(R)
    species = (rng.permutation(n) < int(0.2 * n)).astype(np.int32)
    sigma = torch.tensor([[1.0, 0.8], [0.8, 0.88]])
    eps = torch.tensor([[1.0, 1.5], [1.5, 0.5]])
    disp, shift = space.periodic(L)

    def make():
        nfn, efn = energy.lennard_jones_neighbor_list(
            disp, L, species=torch.tensor(species, device=cuda), sigma=sigma, epsilon=eps,
            dr_threshold=0.3, format=partition.Dense)
        Rt = torch.tensor(R, device=cuda)
        nb = nfn.allocate(Rt)
        init, apply = simulate.nve(efn, shift, 0.002)
        P = torch.tensor(O.maxwell_boltzmann(n, 3, 0.8, 4), device=cuda)
        return apply, init(0, Rt, momenta=P, neighbor=nb), nb
    apply_a, st_a, nb_a = make()
    apply_b, st_b, nb_b = make()
    simulate.run(apply_a, st_a, nb_a, 20, layout=layout)
    for _ in range(20):
        nb_b = nb_b.update(st_b.position)
        st_b = apply_b(st_b, neighbor=nb_b)
    torch.cuda.synchronize()
    d = O.displacement(st_a.position.cpu().numpy(), st_b.position.cpu().numpy(), np.full(3, L))
    assert np.abs(d).max() < 1e-4
    assert (st_a.momentum - st_b.momentum).abs().max().item() < 1e-3


def test_half_list_occupancy_and_overflow_follow_full_rows(cuda):
    """Half lists keep the Dense contract: the occupancy the run reports is
    the largest full row (own entries + the times an atom is listed by
    others), and a list allocated without headroom overflows as the full
    lists do."""
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(10)
    disp, shift = space.periodic(L)
    out = {}
    for layout in ('segment', 'half'):
        nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3,
                                                      format=partition.Dense,
                                                      capacity_multiplier=1.0)
        Rt = torch.tensor(R, device=cuda)
        nb = nfn.allocate(Rt)
        init, apply = simulate.nve(efn, shift, LJ_DT)
        st = init(0, Rt, momenta=3.0 * torch.tensor(P, device=cuda), neighbor=nb)
        simulate.run(apply, st, nb, 1, layout=layout, lazy_list=True)
        torch.cuda.synchronize()
        occ1 = int(nb.plan.occupancy)
        cnt1 = st._sorted.cnt.clone()
        simulate.run(apply, st, nb, 200, layout=layout, lazy_list=True)
        torch.cuda.synchronize()
        out[layout] = (occ1, cnt1, bool(nb.did_buffer_overflow))
    assert out['half'][0] == out['segment'][0]
    assert torch.equal(out['half'][1], out['segment'][1])
    assert out['half'][2] and out['segment'][2]


@pytest.mark.parametrize('layout', ['segment', 'half', 'tiled'])
def test_warm_start_rebuilds_when_the_caller_moves_atoms(cuda, layout):
    """A run that continues the previous run of the same state takes its
    first rebuild only when needed: after the caller moves a few atoms by
    half a lattice constant between runs (onto octahedral sites, far beyond
    the skin threshold), the next run's forces still match the FP64 oracle
    at its final positions, and an unchanged state continues as one run
    would."""
    from jax_md_gb300 import simulate
    spatial = pytest.importorskip('scipy.spatial')
    _, _, L, _, _, _, apply_a, st_a, nb_a = _setup(cuda, n_cells=10)
    simulate.run(apply_a, st_a, nb_a, 5, layout=layout)
    # move every 97th atom by a / 2 along x (wrapped), then continue
    with torch.no_grad():
        moved = torch.arange(0, st_a.position.shape[0], 97, device=cuda)
        st_a.position[moved, 0] = torch.remainder(st_a.position[moved, 0] + L / 20, L)
    simulate.run(apply_a, st_a, nb_a, 2, layout=layout)
    torch.cuda.synchronize()
    assert simulate.last_run_status(st_a) == 0
    X = st_a.position.double().cpu().numpy()
    pairs = spatial.cKDTree(np.mod(X, L), boxsize=L).query_pairs(2.5, output_type='ndarray')
    idx = np.stack([pairs.min(1), pairs.max(1)])
    _, Fo, _ = O.pair_energy_forces(lj_spec(), X, idx, O.ORDERED_SPARSE, np.full(3, L))
    F = st_a.force.cpu().numpy()
    # moved atoms may overlap their new neighbours: compare to the fp32
    # conditioning of the pair sums
    tol = 1e-4 + 4e-6 * np.abs(Fo).max()
    assert np.abs(F - Fo).max() < tol, np.abs(F - Fo).max()
    # an unchanged state: two warm runs of 4 steps against one run of 8
    _, _, _, _, _, _, apply_b, st_b, nb_b = _setup(cuda, n_cells=10)
    _, _, _, _, _, _, apply_c, st_c, nb_c = _setup(cuda, n_cells=10)
    simulate.run(apply_b, st_b, nb_b, 4, layout=layout)
    simulate.run(apply_b, st_b, nb_b, 4, layout=layout)
    simulate.run(apply_c, st_c, nb_c, 8, layout=layout)
    torch.cuda.synchronize()
    assert (st_b.position - st_c.position).abs().max().item() < 1e-5
    assert (st_b.momentum - st_c.momentum).abs().max().item() < 1e-3
