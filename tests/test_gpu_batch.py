"""Batched uneven systems against the FP64 oracle, system by system.

Each system of a batch must get the results of its own single-system call:
neighbour sets of partition.neighbor_list (sorted rows, pairs within 1e-6 of
the cutoff excluded), forces and energies of smap.pair_neighbor_list, FIRE
steps of minimize.fire_descent and velocity-Verlet steps of simulate.nve.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import near_cutoff_pairs

pytestmark = pytest.mark.gpu

SS_SIGMA = np.array([[1.0, 1.2], [1.2, 1.4]])
SIZES_2D = [64, 150, 401, 1000, 97, 2500]


def _ss_batch(cuda, sizes=SIZES_2D, seed=0, capacity_multiplier=1.25):
    from jax_md_gb300 import batch, energy, space
    systems = [O.bidisperse_2d(n, phi=0.84, seed=seed + k) for k, n in enumerate(sizes)]
    Rs = [torch.tensor(R, device=cuda) for R, L, s in systems]
    bt = batch.pack(Rs, [float(L) for R, L, s in systems], species=[s for R, L, s in systems])
    disp, _ = space.periodic(float(systems[0][1]))
    _, efn = energy.soft_sphere_neighbor_list(disp, float(systems[0][1]),
                                              torch.tensor(systems[0][2], device=cuda),
                                              sigma=SS_SIGMA)
    fns = batch.neighbor_list(1.4, 0.2, capacity_multiplier=capacity_multiplier)
    nb = fns.allocate(bt)
    return systems, bt, fns, nb, batch.BatchPairEnergy(efn)


def _lj_batch(cuda, cells=(6, 7, 8), seed=0):
    from jax_md_gb300 import batch, energy, space
    systems = [O.fcc_lattice(c, 0.8442, 0.05, seed + k) for k, c in enumerate(cells)]
    Rs = [torch.tensor(R, device=cuda) for R, L in systems]
    bt = batch.pack(Rs, [float(L) for R, L in systems])
    disp, _ = space.periodic(float(systems[0][1]))
    _, efn = energy.lennard_jones_neighbor_list(disp, float(systems[0][1]), dr_threshold=0.3)
    fns = batch.neighbor_list(2.5, 0.3)
    nb = fns.allocate(bt)
    return systems, bt, fns, nb, batch.BatchPairEnergy(efn)


def _check_sets(bt, nb, systems, cutoff, dim):
    for b, sysb in enumerate(systems):
        R, L = sysb[0], float(sysb[1])
        box = np.full(dim, L)
        got = nb.dense(b)
        nl = O.NeighborListOracle(box, cutoff, 0.0, fmt=O.DENSE)
        ref = O.neighbor_sets(nl.build(R), len(R))
        near = near_cutoff_pairs(R, box, cutoff)
        for i in range(len(R)):
            g = {int(j) for j in got[i] if j < len(R)}
            r = set(ref[i])
            diff = {(i, j) for j in g ^ r}
            assert diff <= near, (b, i, sorted(g ^ r))


def test_batch_neighbor_sets_2d_uneven(cuda):
    systems, bt, fns, nb, _ = _ss_batch(cuda)
    torch.cuda.synchronize()
    assert not nb.did_buffer_overflow
    _check_sets(bt, nb, systems, 1.6, 2)


def test_batch_neighbor_sets_3d(cuda):
    systems, bt, fns, nb, _ = _lj_batch(cuda)
    assert not nb.did_buffer_overflow
    _check_sets(bt, nb, systems, 2.8, 3)


def test_batch_neighbor_sets_small_boxes(cuda):
    """Boxes of 1, 2 and 3 list cutoffs per side (the reference's all-pairs
    candidates below three cells) give the oracle's sets."""
    systems, bt, fns, nb, ef = _lj_batch(cuda, cells=(3, 4, 6))
    assert nb.grid.cps[:, 0].tolist() == [1, 2, 3]
    assert not nb.did_buffer_overflow
    _check_sets(bt, nb, systems, 2.8, 3)
    F = ef.forces(bt, nb)
    torch.cuda.synchronize()
    for b, (R, L) in enumerate(systems):
        F0 = O.pair_energy_forces(O.PairSpec(kind='lj'), R, nb.dense(b), O.DENSE, np.full(3, L))[1]
        assert np.abs(bt.split(F[:, :3])[b].cpu().numpy() - F0).max() < 1e-4


@pytest.mark.parametrize('kind', ['soft_sphere_2d', 'lj_3d'])
def test_batch_forces_and_energies(cuda, kind):
    if kind == 'soft_sphere_2d':
        systems, bt, fns, nb, ef = _ss_batch(cuda)
        specs = [O.PairSpec(kind='soft_sphere', sigma=SS_SIGMA, species=s) for R, L, s in systems]
        dim = 2
    else:
        systems, bt, fns, nb, ef = _lj_batch(cuda)
        specs = [O.PairSpec(kind='lj') for _ in systems]
        dim = 3
    e = torch.empty(bt.n_systems, dtype=torch.float64, device=cuda)
    F = ef.forces(bt, nb, energies=e)
    torch.cuda.synchronize()
    Fb = bt.split(F[:, :dim])
    for b, sysb in enumerate(systems):
        R, L = sysb[0], float(sysb[1])
        box = np.full(dim, L)
        idx = nb.dense(b)
        E0, F0, _ = O.pair_energy_forces(specs[b], R, idx, O.DENSE, box)
        scale = O.pair_force_abs_sum(specs[b], R, idx, O.DENSE, box)
        err = np.abs(Fb[b].cpu().numpy() - F0).max(1)
        assert np.all(err <= 1e-4 + 4e-6 * scale), (b, err.max())
        assert abs(float(e[b]) - E0) <= 1e-5 * abs(E0) + 1e-6, (b, float(e[b]), E0)


def test_batch_fire_matches_oracle_steps(cuda):
    from jax_md_gb300 import batch
    systems, bt, fns, nb, ef = _ss_batch(cuda, sizes=[64, 300, 777])
    run = batch.BatchRunner(bt, fns, nb, ef)
    run.fire_init(f_tol=0.0)
    steps = 25
    run.fire(steps)
    torch.cuda.synchronize()
    fs = run.fire_state.view(-1, 8).cpu().numpy()
    Rb = bt.split(bt.R)
    for b, (R, L, s) in enumerate(systems):
        box = np.full(2, float(L))
        spec = O.PairSpec(kind='soft_sphere', sigma=SS_SIGMA, species=s)
        nl = O.NeighborListOracle(box, 1.4, 0.2, fmt=O.DENSE)
        h = {'nb': nl.allocate(R)}

        def fn(X):
            h['nb'] = nl.update(X, h['nb'])
            return O.pair_energy_forces(spec, X, h['nb'].idx, O.DENSE, box)[1]
        Rd = R.astype(np.float64)
        st = O.FireO(Rd, np.zeros_like(Rd), fn(Rd), 1.0, 0.1, 0.1, 0)
        for _ in range(steps):
            st = O.fire_step(fn, st, box)
        assert abs(fs[b, 0] - st.dt) < 1e-5 * max(1.0, st.dt), (b, fs[b, 0], st.dt)
        assert abs(fs[b, 1] - st.alpha) < 1e-5, (b, fs[b, 1], st.alpha)
        assert int(fs[b, 2]) == st.n_pos
        d = O.displacement(Rb[b].cpu().numpy(), st.R, box)
        assert np.abs(d).max() < 1e-3, (b, np.abs(d).max())


def test_batch_minimize_to_tolerance(cuda):
    from jax_md_gb300 import batch
    systems, bt, fns, nb, ef = _ss_batch(cuda, sizes=[64, 200, 512, 128])
    run = batch.BatchRunner(bt, fns, nb, ef)
    E0 = run.potential().cpu().numpy()
    steps = run.minimize(f_tol=1e-4, max_steps=20000, chunk=500)
    torch.cuda.synchronize()
    assert int(run.n_done.item()) == bt.n_systems, steps
    assert not nb.did_buffer_overflow
    # the stopping test used the forces after each system's last step
    fmax_stop = run.fire_state.view(-1, 8)[:, 6].cpu().numpy()
    assert np.all(fmax_stop < 1e-4)
    E1 = run.potential().cpu().numpy()
    assert np.all(E1 < E0)


def test_batch_nve_matches_oracle(cuda):
    from jax_md_gb300 import batch
    systems, bt, fns, nb, ef = _lj_batch(cuda)
    run = batch.BatchRunner(bt, fns, nb, ef, dt=0.005)
    P0 = [O.maxwell_boltzmann(len(R), 3, 0.722, 10 + b) for b, (R, L) in enumerate(systems)]
    run.momentum.zero_()
    run.momentum[:, :3] = torch.tensor(np.concatenate(P0), device=cuda)
    steps = 50
    run.nve(steps)
    torch.cuda.synchronize()
    Rb = bt.split(bt.R)
    Pb = bt.split(run.momentum[:, :3])
    spec = O.PairSpec(kind='lj')
    for b, (R, L) in enumerate(systems):
        box = np.full(3, float(L))
        nl = O.NeighborListOracle(box, 2.5, 0.3, fmt=O.DENSE)
        h = {'nb': nl.allocate(R)}

        def fn(X):
            h['nb'] = nl.update(X, h['nb'])
            return O.pair_energy_forces(spec, X, h['nb'].idx, O.DENSE, box)[1]
        X, P = R.astype(np.float64), P0[b].astype(np.float64)
        F = fn(X)
        for _ in range(steps):
            X, P, F = O.velocity_verlet(fn, X, P, F, 1.0, 0.005, box)
        d = O.displacement(Rb[b].cpu().numpy(), X, box)
        assert np.abs(d).max() < 1e-3, (b, np.abs(d).max())
        assert np.abs(Pb[b].cpu().numpy() - P).max() < 1e-2


def test_batch_nve_graph_equals_direct(cuda):
    """The graph-replayed run and direct launches give identical states."""
    from jax_md_gb300 import batch
    out = []
    for use_graph in (True, False):
        systems, bt, fns, nb, ef = _lj_batch(cuda, cells=(6, 7))
        run = batch.BatchRunner(bt, fns, nb, ef, dt=0.005)
        run.set_momenta(0.722, seed=4)
        run.nve(30, use_graph=use_graph)
        out.append((bt.position.clone(), run.momentum.clone()))
    torch.cuda.synchronize()
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])


def test_batch_overflow_flag(cuda):
    systems, bt, fns, nb, _ = _ss_batch(cuda, sizes=[64, 150])
    small = fns._make(bt, nb.grid, 2)
    fns._build(small, bt.position)
    torch.cuda.synchronize()
    assert small.did_buffer_overflow
    assert int(small.occupancy.item()) == nb.occupancy.item()


KA_SIG = np.array([[1.0, 0.8], [0.8, 0.88]])
KA_EPS = np.array([[1.0, 1.5], [1.5, 0.5]])


def _ka_system(n_cells, seed):
    R, L = O.fcc_lattice(n_cells, 0.8442, 0.05, seed)
    n = len(R)
    Lk = float(np.float32((n / 1.2) ** (1 / 3)))
    R = np.mod(R / float(L) * Lk, Lk).astype(np.float32)
    rng = np.random.default_rng(seed)
    species = np.zeros(n, np.int32)
    species[rng.permutation(n)[: n // 5]] = 1
    P = (rng.standard_normal((n, 3)) * np.sqrt(0.8)).astype(np.float32)
    P -= P.mean(0, keepdims=True)
    return R, P, Lk, species


def _ka_batch(cuda, cells=(6, 7, 6)):
    from jax_md_gb300 import batch, energy, space
    systems = [_ka_system(c, 20 + k) for k, c in enumerate(cells)]
    bt = batch.pack([torch.tensor(R, device=cuda) for R, P, L, s in systems],
                    [L for R, P, L, s in systems], species=[s for R, P, L, s in systems])
    disp, _ = space.periodic(systems[0][2])
    _, efn = energy.lennard_jones_neighbor_list(disp, systems[0][2],
                                                torch.tensor(systems[0][3], device=cuda),
                                                sigma=KA_SIG, epsilon=KA_EPS, dr_threshold=0.3)
    fns = batch.neighbor_list(2.5, 0.3)
    nb = fns.allocate(bt, extra_capacity=8)
    return systems, bt, fns, nb, batch.BatchPairEnergy(efn)


def _ka_oracle_final_energies(systems, sig, eps, steps, dt=0.005, kT=None):
    """PE_b / N_b of each system after `steps` NVE steps, or
    Nose-Hoover steps (chain 5, tau = 100 dt) at kT when kT is given."""
    out = []
    for R, P, L, s in systems:
        box = np.full(3, L)
        spec = O.PairSpec(kind='lj', sigma=sig, epsilon=eps, species=s)
        nl = O.NeighborListOracle(box, 2.5 * np.max(sig), 0.3)
        h = {'nb': nl.allocate(R)}

        def fn(X):
            h['nb'] = nl.update(X, h['nb'])
            return O.pair_energy_forces(spec, X, h['nb'].idx, O.DENSE, box)[1]
        X, Pd = R.astype(np.float64), P.astype(np.float64)
        F = fn(X)
        c = O.nhc_init(3 * len(R), O.kinetic_energy(Pd), kT, 100 * dt, 5) if kT else None
        for _ in range(steps):
            if kT:
                X, Pd, F, c = O.nvt_nose_hoover_step(fn, X, Pd, F, 1.0, c, dt, kT, box)
            else:
                X, Pd, F = O.velocity_verlet(fn, X, Pd, F, 1.0, dt, box)
        out.append(O.pair_energy_forces(spec, X, nl.build(X).idx, O.DENSE, box)[0] / len(R))
    return np.array(out)


def test_batch_energy_gradients(cuda):
    systems, bt, fns, nb, ef = _ka_batch(cuda)
    sig = torch.tensor(KA_SIG, dtype=torch.float32, device=cuda, requires_grad=True)
    eps = torch.tensor(KA_EPS, dtype=torch.float32, device=cuda, requires_grad=True)
    R = bt.R.clone().requires_grad_(True)
    E = ef.energy_fn_autograd(bt, nb)(R, sigma=sig, epsilon=eps)
    w = torch.tensor([0.5, -1.0, 2.0], dtype=torch.float64, device=cuda)
    (E * w).sum().backward()
    F = ef.forces(bt, nb)[:, :3]
    wa = w[bt.atom_sys.long()].to(torch.float32)[:, None]
    assert torch.allclose(R.grad, -F * wa, atol=1e-6)
    h = 1e-6
    for mat, g in (('sigma', sig.grad), ('epsilon', eps.grad)):
        for a, b in ((0, 1), (1, 1)):
            vals = []
            for sgn in (1, -1):
                sm, em = KA_SIG.copy(), KA_EPS.copy()
                (sm if mat == 'sigma' else em)[a, b] += sgn * h
                tot = 0.0
                for k, (Rk, Pk, Lk, sk) in enumerate(systems):
                    spec = O.PairSpec(kind='lj', sigma=sm, epsilon=em, species=sk)
                    tot += float(w[k]) * O.pair_energy_forces(spec, Rk, nb.dense(k), O.DENSE,
                                                              np.full(3, Lk))[0]
                vals.append(tot)
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(float(g[a, b]) - fd) <= 1e-4 * max(1.0, abs(fd)), (mat, a, b, float(g[a, b]), fd)


@pytest.mark.parametrize('k', [7, None], ids=['checkpointed', 'stored'])
def test_batch_trajectory_gradient_matches_fd(cuda, k):
    """Gradient of mean_b PE_b(x_n)/N_b after 20 NVE steps of an uneven KA
    batch with respect to the shared sigma_AB, epsilon_AB (and R0 along a
    direction), against FP64 central differences of the oracle."""
    from jax_md_gb300 import batch
    systems, bt, fns, nb, ef = _ka_batch(cuda)
    steps = 20
    traj = batch.BatchTrajectory(bt, fns, nb, ef, 0.005, steps, checkpoint_every=k)
    sig = torch.tensor(KA_SIG, dtype=torch.float32, device=cuda, requires_grad=True)
    eps = torch.tensor(KA_EPS, dtype=torch.float32, device=cuda, requires_grad=True)
    R0 = bt.R.clone().requires_grad_(True)
    P0 = torch.tensor(np.concatenate([P for R, P, L, s in systems]), device=cuda)
    xn, pn = traj(R0, P0, sigma=sig, epsilon=eps)
    x4 = torch.nn.functional.pad(xn.detach(), (0, 1)).contiguous()
    nb = fns.update(x4, nb)
    E = ef.energy_fn_autograd(bt, nb)(xn, sigma=sig, epsilon=eps)
    sizes = torch.tensor(bt.sizes, dtype=torch.float64, device=cuda)
    loss = (E / sizes).mean()
    loss.backward()
    L0 = _ka_oracle_final_energies(systems, KA_SIG, KA_EPS, steps).mean()
    assert abs(float(loss) - L0) <= 1e-4 * abs(L0)
    hh = 1e-4
    for mat, g in (('sigma', sig.grad), ('epsilon', eps.grad)):
        for a, b in ((0, 1), (0, 0)):
            lp = []
            for sgn in (1, -1):
                sm, em = KA_SIG.copy(), KA_EPS.copy()
                (sm if mat == 'sigma' else em)[a, b] += sgn * hh
                lp.append(_ka_oracle_final_energies(systems, sm, em, steps).mean())
            fd = (lp[0] - lp[1]) / (2 * hh)
            assert abs(float(g[a, b]) - fd) <= 1e-3 * max(abs(fd), 1e-2), (mat, a, b, float(g[a, b]), fd)
    v = np.random.default_rng(9).standard_normal((bt.n, 3))
    v /= np.linalg.norm(v)
    e_r = 1e-4
    sp = []
    for sgn in (1, -1):
        shifted = []
        for kk, (R, P, L, s) in enumerate(systems):
            r = bt.rows(kk)
            shifted.append(((R + sgn * e_r * v[r]).astype(np.float64), P, L, s))
        sp.append(_ka_oracle_final_energies(shifted, KA_SIG, KA_EPS, steps).mean())
    fd = (sp[0] - sp[1]) / (2 * e_r)
    ad = float((R0.grad.cpu().numpy() * v).sum())
    assert abs(ad - fd) <= 1e-3 * max(abs(fd), 1e-2), (ad, fd)


def test_batch_autotune(cuda):
    """The batch autotuner times every launch shape, leaves the runner's state
    as it found it, and the forces do not depend on the force CTA size."""
    from jax_md_gb300 import batch
    systems, bt, fns, nb, ef = _ss_batch(cuda, sizes=[64, 300, 777])
    run = batch.BatchRunner(bt, fns, nb, ef)
    run.fire_init(0.0)
    x0 = bt.position.clone()
    r = batch.autotune(run, steps=5)
    assert len(r['ms']) == len(batch.FORCE_BLOCKS) * len(batch.FIRE_THREADS)
    assert r['best'][0] in batch.FORCE_BLOCKS and r['best'][1] in batch.FIRE_THREADS
    assert torch.equal(bt.position, x0)
    F = {}
    for fb in batch.FORCE_BLOCKS:
        batch.set_launch(fb, 1024)
        F[fb] = ef.forces(bt, nb).clone()
    torch.cuda.synchronize()
    assert torch.equal(F[64], F[128]) and torch.equal(F[128], F[256])
    batch.set_launch(*r['best'])


def _lj_oracle_nvt(R, P0, L, steps, kT=0.722, dt=0.005):
    box = np.full(3, float(L))
    spec = O.PairSpec(kind='lj')
    nl = O.NeighborListOracle(box, 2.5, 0.3, fmt=O.DENSE)
    h = {'nb': nl.allocate(R)}

    def fn(X):
        h['nb'] = nl.update(X, h['nb'])
        return O.pair_energy_forces(spec, X, h['nb'].idx, O.DENSE, box)[1]
    X, P = R.astype(np.float64), P0.astype(np.float64)
    F = fn(X)
    c = O.nhc_init(3 * len(R), O.kinetic_energy(P), kT, 100 * dt, 5)
    for _ in range(steps):
        X, P, F, c = O.nvt_nose_hoover_step(fn, X, P, F, 1.0, c, dt, kT, box)
    return X, P, c


def test_batch_nvt_matches_oracle(cuda):
    """Every system of a batched Nose-Hoover run, each with its own chain,
    against the oracle's NVT step (simulate.py:649-667) over 50 steps
    (positions, momenta, chain momenta), and each system's invariant
    (simulate.py:672-701) conserved."""
    from jax_md_gb300 import batch
    systems, bt, fns, nb, ef = _lj_batch(cuda, cells=(4, 5, 6))
    run = batch.BatchRunner(bt, fns, nb, ef, dt=0.005)
    P0 = [O.maxwell_boltzmann(len(R), 3, 0.722, 30 + b) for b, (R, L) in enumerate(systems)]
    run.momentum.zero_()
    run.momentum[:, :3] = torch.tensor(np.concatenate(P0), device=cuda)
    run.nvt_init(0.722)
    H0 = run.nvt_invariant()
    steps = 50
    run.nvt(steps)
    H1 = run.nvt_invariant()
    torch.cuda.synchronize()
    Rb = bt.split(bt.R)
    Pb = bt.split(run.momentum[:, :3])
    chain = run.chain.cpu().numpy()
    for b, (R, L) in enumerate(systems):
        X, P, c = _lj_oracle_nvt(R, P0[b], L, steps)
        d = O.displacement(Rb[b].cpu().numpy(), X, np.full(3, float(L)))
        assert np.abs(d).max() < 1e-3, (b, np.abs(d).max())
        assert np.abs(Pb[b].cpu().numpy() - P).max() < 1e-2
        err = np.abs(chain[b, 16:21] - c.p_xi).max()
        assert err <= 1e-2 * max(1.0, np.abs(c.p_xi).max()), (b, chain[b, 16:21], c.p_xi)
    sizes = torch.tensor(bt.sizes, dtype=torch.float64, device=cuda)
    assert float(((H1 - H0).abs() / sizes).max()) < 1e-3, (H0, H1)


def test_batch_nvt_graph_equals_direct(cuda):
    """The graph-replayed batched NVT run and direct launches give identical
    positions, momenta and chains."""
    from jax_md_gb300 import batch
    out = []
    for use_graph in (True, False):
        systems, bt, fns, nb, ef = _lj_batch(cuda, cells=(5, 6))
        run = batch.BatchRunner(bt, fns, nb, ef, dt=0.005)
        run.set_momenta(0.722, seed=4)
        run.nvt_init(0.722)
        run.nvt(30, use_graph=use_graph)
        out.append((bt.position.clone(), run.momentum.clone(), run.chain.clone()))
    torch.cuda.synchronize()
    assert all(torch.equal(a, b) for a, b in zip(*out))


@pytest.mark.parametrize('k', [None, 5], ids=['stored', 'checkpointed'])
def test_batch_nvt_trajectory_gradient_matches_fd(cuda, k):
    """Gradient of mean_b PE_b(x_n)/N_b after 12 batched Nose-Hoover steps (a
    chain per system, kT = 0.6) with respect to the shared sigma_AB,
    epsilon_AB and along random directions of R0 and P0, against FP64 central
    differences of the oracle's NVT step; every step recorded, or checkpoints
    every 5 steps with replayed segments."""
    from jax_md_gb300 import batch
    systems, bt, fns, nb, ef = _ka_batch(cuda)
    steps, kT = 12, 0.6
    traj = batch.BatchNvtTrajectory(bt, fns, nb, ef, 0.005, kT, steps, checkpoint_every=k)
    sig = torch.tensor(KA_SIG, dtype=torch.float32, device=cuda, requires_grad=True)
    eps = torch.tensor(KA_EPS, dtype=torch.float32, device=cuda, requires_grad=True)
    R0 = bt.R.clone().requires_grad_(True)
    P0 = torch.tensor(np.concatenate([P for R, P, L, s in systems]), device=cuda).requires_grad_(True)
    xn, pn = traj(R0, P0, sigma=sig, epsilon=eps)
    x4 = torch.nn.functional.pad(xn.detach(), (0, 1)).contiguous()
    nb = fns.update(x4, nb)
    E = ef.energy_fn_autograd(bt, nb)(xn, sigma=sig, epsilon=eps)
    sizes = torch.tensor(bt.sizes, dtype=torch.float64, device=cuda)
    loss = (E / sizes).mean()
    loss.backward()
    L0 = _ka_oracle_final_energies(systems, KA_SIG, KA_EPS, steps, kT=kT).mean()
    assert abs(float(loss.detach()) - L0) <= 1e-4 * abs(L0)
    hh = 1e-4
    for mat, g in (('sigma', sig.grad), ('epsilon', eps.grad)):
        lp = []
        for sgn in (1, -1):
            sm, em = KA_SIG.copy(), KA_EPS.copy()
            (sm if mat == 'sigma' else em)[0, 1] += sgn * hh
            lp.append(_ka_oracle_final_energies(systems, sm, em, steps, kT=kT).mean())
        fd = (lp[0] - lp[1]) / (2 * hh)
        assert abs(float(g[0, 1]) - fd) <= 1e-3 * max(abs(fd), 1e-2), (mat, float(g[0, 1]), fd)
    rng = np.random.default_rng(11)
    e = 1e-4
    for which, grad in (('R', R0.grad), ('P', P0.grad)):
        v = rng.standard_normal((bt.n, 3))
        v /= np.linalg.norm(v)
        sp = []
        for sgn in (1, -1):
            shifted = []
            for kk, (R, P, L, s) in enumerate(systems):
                r = bt.rows(kk)
                if which == 'R':
                    shifted.append(((R + sgn * e * v[r]).astype(np.float64), P, L, s))
                else:
                    shifted.append((R, (P + sgn * e * v[r]).astype(np.float64), L, s))
            sp.append(_ka_oracle_final_energies(shifted, KA_SIG, KA_EPS, steps, kT=kT).mean())
        fd = (sp[0] - sp[1]) / (2 * e)
        ad = float((grad.cpu().numpy() * v).sum())
        assert abs(ad - fd) <= 1e-3 * max(abs(fd), 1e-2), (which, ad, fd)
