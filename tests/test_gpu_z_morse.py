"""Morse pairs (energy.morse x multiplicative_isotropic_cutoff, energy.py:346-440)
on the GPU against the FP64 oracle: forces, energies and virials in every list
format and memory layout, species matrices of sigma / epsilon / alpha, the
graph-replayed NVE engine, the force VJP with its sigma / epsilon gradients,
and a batch of uneven systems.

Tolerances as for LJ (tests/test_gpu_pair.py): forces within 1e-4 +
4e-6 x sum_j |F_ij| max-abs (the fp32 condition of the force sum), the
virial within 1e-6 of its largest component; energies within 1e-5 relative,
since the reference's own float32 form eps (1 - e)^2 - eps loses digits for
the many small outer-shell pairs (it is kept for parity).

The file sorts after the other GPU test files (and before the allocation-free
test, which must come last): these are the newest GPU tests, and a failure
here leaves the earlier files' results intact in a run that stops at the
first failure.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import fcc_system

pytestmark = pytest.mark.gpu

FORCE_ATOL = 1e-4
COND_RTOL = 4e-6
ENERGY_RTOL = 1e-5


def _spec(species=None, sigma=1.0, epsilon=5.0, alpha=5.0):
    return O.PairSpec(kind='morse', sigma=sigma, epsilon=epsilon, alpha=alpha, r_onset=2.0,
                      r_cutoff=2.5, species=species)


def _force_ok(F, Fo, spec, R, idx, fmt, box):
    err = np.abs(np.asarray(F) - Fo).max(axis=1)
    scale = O.pair_force_abs_sum(spec, R, idx, fmt, box)
    return bool(np.all(err <= FORCE_ATOL + COND_RTOL * scale)), float(err.max())


def _setup(cuda, n_cells=8, fmt='Dense', seed=0, species=None, **params):
    from jax_md_gb300 import energy, partition, space
    R, P, L = fcc_system(n_cells, seed)
    disp, shift = space.periodic(L)
    sp = torch.tensor(species, device=cuda) if species is not None else None
    nfn, efn = energy.morse_neighbor_list(disp, L, sp, dr_threshold=0.3,
                                          format=getattr(partition, fmt), **params)
    Rt = torch.tensor(R, device=cuda)
    return R, P, L, shift, nfn, efn, Rt, nfn.allocate(Rt)


@pytest.mark.parametrize('layout', ['float4', 'contiguous'])
def test_morse_dense_forces_energy_virial(cuda, layout):
    from jax_md_gb300 import partition
    R, P, L, shift, nfn, efn, Rt, nb = _setup(cuda)
    X = partition.padded_rows(Rt) if layout == 'float4' else Rt
    E, F, _, W = efn.compute(X, nb, virial=True)
    idx = nb.idx.cpu().numpy()
    box = np.full(3, L)
    Eo, Fo, Wo = O.pair_energy_forces(_spec(), R, idx, O.DENSE, box)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo), (float(E), Eo)
    ok, err = _force_ok(F.cpu().numpy(), Fo, _spec(), R, idx, O.DENSE, box)
    assert ok, err
    w = W.cpu().numpy()
    wo = np.array([Wo[0, 0], Wo[1, 1], Wo[2, 2], Wo[0, 1], Wo[0, 2], Wo[1, 2]])
    assert np.abs(w - wo).max() <= 1e-6 * np.abs(wo).max()


@pytest.mark.parametrize('fmt,code', [('Sparse', O.SPARSE), ('OrderedSparse', O.ORDERED_SPARSE)])
def test_morse_sparse_formats(cuda, fmt, code):
    """The reference's default format for morse_neighbor_list is OrderedSparse."""
    R, P, L, shift, nfn, efn, Rt, nb = _setup(cuda, n_cells=6, fmt=fmt)
    E, F, _, _ = efn.compute(Rt, nb)
    idx = nb.idx.cpu().numpy()
    box = np.full(3, L)
    Eo, Fo, _ = O.pair_energy_forces(_spec(), R, idx, code, box)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    ok, err = _force_ok(F.cpu().numpy(), Fo, _spec(), R, idx, code, box)
    assert ok, err


def test_morse_species_matrices(cuda):
    """Binary Morse with sigma / epsilon / alpha species matrices."""
    rng = np.random.default_rng(5)
    R, _, _ = fcc_system(7, 1)
    species = (rng.uniform(size=len(R)) < 0.3).astype(np.int32)
    sig = np.array([[1.0, 1.1], [1.1, 1.2]])
    eps = np.array([[5.0, 3.0], [3.0, 4.0]])
    alp = np.array([[5.0, 4.0], [4.0, 6.0]])
    R, P, L, shift, nfn, efn, Rt, nb = _setup(cuda, n_cells=7, seed=1, species=species,
                                              sigma=sig, epsilon=eps, alpha=alp)
    E, F, _, _ = efn.compute(Rt, nb)
    spec = _spec(species, sig, eps, alp)
    idx = nb.idx.cpu().numpy()
    box = np.full(3, L)
    Eo, Fo, _ = O.pair_energy_forces(spec, R, idx, O.DENSE, box)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    ok, err = _force_ok(F.cpu().numpy(), Fo, spec, R, idx, O.DENSE, box)
    assert ok, err


def test_morse_nve_run_matches_oracle(cuda):
    """30 steps of simulate.run (one CUDA graph, cell-ordered engine) against
    the oracle's velocity Verlet with its own list rebuilds."""
    from jax_md_gb300 import simulate
    R, P, L, shift, nfn, efn, Rt, nb = _setup(cuda, n_cells=6)
    init, apply = simulate.nve(efn, shift, 0.005)
    st = init(0, Rt, momenta=torch.tensor(P, device=cuda) * 0.5, neighbor=nb)
    steps = 30
    st, nb = simulate.run(apply, st, nb, steps)
    torch.cuda.synchronize()
    box = np.full(3, L)
    nl = O.NeighborListOracle(box, 2.5, 0.3, fmt=O.DENSE)
    h = {'nb': nl.allocate(R)}

    def fn(X):
        h['nb'] = nl.update(X, h['nb'])
        return O.pair_energy_forces(_spec(), X, h['nb'].idx, O.DENSE, box)[1]
    X, Pd = R.astype(np.float64), P.astype(np.float64) * 0.5
    F = fn(X)
    for _ in range(steps):
        X, Pd, F = O.velocity_verlet(fn, X, Pd, F, 1.0, 0.005, box)
    d = O.displacement(st.position[:, :3].cpu().numpy(), X, box)
    assert np.abs(d).max() < 1e-3, np.abs(d).max()
    assert np.abs(st.momentum[:, :3].cpu().numpy() - Pd).max() < 2e-2
    assert not bool(nb.did_buffer_overflow)


def test_morse_force_vjp_and_parameter_gradients(cuda):
    """(dF/dR)^T lambda against the oracle's analytic form, and
    d(lambda . F)/d(sigma, epsilon), dE/d(sigma, epsilon) against FP64 central
    differences (the Morse radii do not move with sigma)."""
    from jax_md_gb300.smap import _bins_to_grads
    R, P, L, shift, nfn, efn, Rt, nb = _setup(cuda, n_cells=5, seed=3)
    idx = nb.idx.cpu().numpy()
    box = np.full(3, L)
    lam = np.random.default_rng(7).standard_normal(R.shape).astype(np.float32)
    gR, bins, _ = efn.force_vjp(Rt, nb, torch.tensor(lam, device=cuda))
    go, _, _ = O.pair_force_vjp(_spec(), R, idx, O.DENSE, lam.astype(np.float64), box)
    assert np.abs(gR.cpu().numpy() - go).max() <= 5e-5 * np.abs(go).max()
    ebins = efn.energy_param_grad(Rt, nb)
    one = torch.tensor(1.0, device=cuda)
    gs, ge = _bins_to_grads(bins, None, one, one)
    es, ee = _bins_to_grads(ebins, None, one, one)
    h = 1e-6
    for name, g, eg in (('sigma', float(gs), float(es)), ('epsilon', float(ge), float(ee))):
        vals = []
        for sgn in (1, -1):
            kw = {'sigma': 1.0, 'epsilon': 5.0}
            kw[name] += sgn * h
            E, F, _ = O.pair_energy_forces(_spec(**kw), R, idx, O.DENSE, box)
            vals.append((float((lam * F).sum()), E))
        fd = (vals[0][0] - vals[1][0]) / (2 * h)
        fde = (vals[0][1] - vals[1][1]) / (2 * h)
        assert abs(g - fd) <= 2e-4 * max(1.0, abs(fd)), (name, g, fd)
        assert abs(eg - fde) <= 2e-4 * max(1.0, abs(fde)), (name, eg, fde)


def test_morse_batched_forces(cuda):
    """A batch of uneven Morse systems: each system's forces and energy equal
    its own single-system oracle values."""
    from jax_md_gb300 import batch, energy, space
    systems = [O.fcc_lattice(c, 0.8442, 0.05, 10 + k) for k, c in enumerate((4, 6, 5))]
    bt = batch.pack([torch.tensor(R, device=cuda) for R, L in systems],
                    [float(L) for R, L in systems])
    disp, _ = space.periodic(float(systems[0][1]))
    _, efn = energy.morse_neighbor_list(disp, float(systems[0][1]), dr_threshold=0.3)
    fns = batch.neighbor_list(2.5, 0.3)
    nb = fns.allocate(bt)
    ef = batch.BatchPairEnergy(efn)
    F = ef.forces(bt, nb)
    E = ef.energies(bt, nb)
    torch.cuda.synchronize()
    Fb = bt.split(F[:, :3])
    for b, (R, L) in enumerate(systems):
        box = np.full(3, float(L))
        nl = O.NeighborListOracle(box, 2.5, 0.3, fmt=O.DENSE)
        idx = nl.allocate(R).idx
        Eo, Fo, _ = O.pair_energy_forces(_spec(), R, idx, O.DENSE, box)
        assert abs(float(E[b]) - Eo) <= ENERGY_RTOL * abs(Eo)
        ok, err = _force_ok(Fb[b].cpu().numpy(), Fo, _spec(), R, idx, O.DENSE, box)
        assert ok, (b, err)
