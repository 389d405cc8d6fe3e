"""Pair energies, forces and virials on the GPU against the FP64 oracle.

Tolerances (fp32 kernels vs the f64 oracle on identical fp32 positions):
per-atom forces within 1e-4 eps/sigma max-abs, total energy within 1e-6
relative, virial within 1e-6 relative of its largest component.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import GOLDEN, fcc_system, lj_spec

pytestmark = pytest.mark.gpu

FORCE_ATOL = 1e-4
ENERGY_RTOL = 1e-6
# fp32 force sums carry rounding of the order of 1e-6 x sum_j |F_ij|; on
# artificially overlapped configurations (pair forces ~1e3) the tolerance is
# scaled by that condition number.
COND_RTOL = 4e-6


def _force_ok(F, Fo, spec, R, idx, fmt, box):
    err = np.abs(np.asarray(F) - Fo).max(axis=1)
    scale = O.pair_force_abs_sum(spec, R, idx, fmt, box)
    return np.all(err <= FORCE_ATOL + COND_RTOL * scale), float(err.max())


def _equilibrated(n_cells, steps, cuda, seed=0):
    """LJ configuration after `steps` NVE steps from the FCC start (melting run)."""
    from jax_md_gb300 import energy, partition, simulate, space
    from tests.helpers import fcc_system
    R, P, L = fcc_system(n_cells, seed)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3, format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nve(efn, shift, 0.005)
    st = init(0, Rt, momenta=torch.tensor(P, device=cuda) * 1.5, neighbor=nb)
    for _ in range(steps):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    return st.position.contiguous().cpu().numpy(), L


def _lj_setup(cuda, n_cells=10, fmt='Dense', seed=0, disorder=0.0):
    from jax_md_gb300 import energy, partition, space
    R, P, L = fcc_system(n_cells, seed)
    if disorder:
        rng = np.random.default_rng(seed + 7)
        R = np.mod(R + rng.uniform(-disorder, disorder, R.shape), L).astype(np.float32)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, sigma=1.0, epsilon=1.0,
                                                  dr_threshold=0.3,
                                                  format=getattr(partition, fmt))
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    return R, L, Rt, nb, efn


def _oracle(R, L, nb_idx, fmt):
    return O.pair_energy_forces(lj_spec(), R, nb_idx, fmt, np.full(3, L))


@pytest.mark.parametrize('layout', ['float4', 'contiguous'])
def test_lj_dense_lattice_start(cuda, layout):
    """The plain LJ workload's own start (FCC + 0.05 jitter), N=4000: 1e-4 max-abs."""
    R, L, Rt, nb, efn = _lj_setup(cuda)
    X = Rt if layout == 'contiguous' else __import__('jax_md_gb300').partition.padded_rows(Rt)
    E, F, _, W = efn.compute(X, nb, virial=True)
    Eo, Fo, Wo = _oracle(R, L, nb.idx.cpu().numpy(), O.DENSE)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    err = np.abs(F.cpu().numpy() - Fo).max()
    assert err < FORCE_ATOL, err
    w = W.cpu().numpy()
    wo = np.array([Wo[0, 0], Wo[1, 1], Wo[2, 2], Wo[0, 1], Wo[0, 2], Wo[1, 2]])
    assert np.abs(w - wo).max() <= 1e-6 * np.abs(wo).max()


def test_lj_dense_equilibrated_liquid(cuda):
    """A melted LJ configuration (hot start, 400 steps), identical positions: 1e-4 max-abs."""
    from jax_md_gb300 import energy, partition, space
    R, L = _equilibrated(8, 400, cuda)
    disp, _ = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3, format=partition.Dense)
    Rt = partition.padded_rows(torch.tensor(R, device=cuda))
    nb = nfn.allocate(Rt)
    E, F, _, W = efn.compute(Rt, nb, virial=True)
    Eo, Fo, Wo = _oracle(R, L, nb.idx.cpu().numpy(), O.DENSE)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    err = np.abs(F.cpu().numpy() - Fo).max()
    assert err < FORCE_ATOL, (err, np.abs(Fo).max())


@pytest.mark.parametrize('layout', ['float4', 'contiguous'])
def test_lj_dense_overlapped_conditioned(cuda, layout):
    """Overlapped start (pair forces ~1e3): error within the fp32 conditioning bound."""
    R, L, Rt, nb, efn = _lj_setup(cuda, disorder=0.25)
    X = Rt if layout == 'contiguous' else __import__('jax_md_gb300').partition.padded_rows(Rt)
    E, F, _, W = efn.compute(X, nb, virial=True)
    idx = nb.idx.cpu().numpy()
    Eo, Fo, Wo = _oracle(R, L, idx, O.DENSE)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    ok, err = _force_ok(F.cpu().numpy(), Fo, lj_spec(), R, idx, O.DENSE, np.full(3, L))
    assert ok, err


@pytest.mark.parametrize('tpa', [4, 8, 16, 32])
def test_threads_per_atom_agree(cuda, tpa):
    from jax_md_gb300 import _native as N
    R, L, Rt, nb, efn = _lj_setup(cuda, n_cells=6, disorder=0.2)
    N.check(N.lib().jmd_set_pair_threads_per_atom(tpa))
    try:
        E, F, _, _ = efn.compute(Rt, nb)
    finally:
        N.lib().jmd_set_pair_threads_per_atom(8)
    idx = nb.idx.cpu().numpy()
    Eo, Fo, _ = _oracle(R, L, idx, O.DENSE)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    ok, err = _force_ok(F.cpu().numpy(), Fo, lj_spec(), R, idx, O.DENSE, np.full(3, L))
    assert ok, err


@pytest.mark.parametrize('tpa', [4, 8, 16])
def test_float4_threads_per_atom_agree(cuda, tpa):
    from jax_md_gb300 import _native as N, partition
    R, L, Rt, nb, efn = _lj_setup(cuda, n_cells=6, disorder=0.2)
    X = partition.padded_rows(Rt)
    N.check(N.lib().jmd_set_dense_threads_per_atom(tpa))
    try:
        E, F, _, _ = efn.compute(X, nb)
    finally:
        N.lib().jmd_set_dense_threads_per_atom(8)
    idx = nb.idx.cpu().numpy()
    Eo, Fo, _ = _oracle(R, L, idx, O.DENSE)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    ok, err = _force_ok(F.cpu().numpy(), Fo, lj_spec(), R, idx, O.DENSE, np.full(3, L))
    assert ok, err


@pytest.mark.parametrize('fmt,code', [('Sparse', O.SPARSE), ('OrderedSparse', O.ORDERED_SPARSE)])
def test_lj_sparse_formats(cuda, fmt, code):
    R, L, Rt, nb, efn = _lj_setup(cuda, n_cells=6, fmt=fmt, disorder=0.2)
    E, F, _, W = efn.compute(Rt, nb, virial=True)
    idx = nb.idx.cpu().numpy()
    Eo, Fo, Wo = _oracle(R, L, idx, code)
    assert abs(float(E) - Eo) <= ENERGY_RTOL * abs(Eo)
    ok, err = _force_ok(F.cpu().numpy(), Fo, lj_spec(), R, idx, code, np.full(3, L))
    assert ok, err


def test_per_particle_energy(cuda):
    from jax_md_gb300 import energy, space
    R, P, L = fcc_system(6)
    disp, _ = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3, per_particle=True,
                                                  format=__import__('jax_md_gb300').partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    e = efn(Rt, nb).cpu().numpy()
    eo, _, _ = O.pair_energy_forces(lj_spec(), R, nb.idx.cpu().numpy(), O.DENSE, np.full(3, L),
                                    per_particle=True)
    np.testing.assert_allclose(e, eo, rtol=1e-5, atol=1e-5)


def test_autograd_backward_is_minus_force(cuda):
    R, L, Rt, nb, efn = _lj_setup(cuda, n_cells=5, disorder=0.2)
    Rg = Rt.clone().requires_grad_(True)
    E = efn(Rg, nb)
    E.backward()
    F = efn.forces(Rt, nb)
    torch.testing.assert_close(Rg.grad, -F, rtol=0, atol=0)


def test_lammps_fixture_on_gpu(cuda):
    """Golden LAMMPS LJ dump: truncated LJ at 2.5 over all pairs, tol 5e-5."""
    from jax_md_gb300 import energy, quantity, smap, space
    g = np.load(GOLDEN / 'lammps_lj_stress.npz')
    box = float(g['box'])
    R = torch.tensor((g['fractional_position'] * box).astype(np.float32), device=cuda)
    V = torch.tensor(g['velocity'].astype(np.float32), device=cuda)
    disp, _ = space.periodic(box)
    efn = smap.pair(energy.truncated(energy.lennard_jones, 2.5), disp)
    E = float(efn(R)) / len(R)
    assert abs(E - float(g['energy_per_atom'])) < 5e-5
    S = quantity.stress(efn, R, box, velocity=V).cpu().numpy()
    np.testing.assert_allclose(S, g['stress'], atol=5e-5, rtol=5e-5)


def test_jammed_soft_sphere_on_gpu(cuda):
    """Golden jammed packing: energy and pressure (quantity_test.py:134-150, f32 tol 2e-5)."""
    from jax_md_gb300 import energy, quantity, space
    g = np.load(GOLDEN / 'jammed_soft_sphere_2d.npz')
    L = np.diag(g['box']).astype(np.float32)
    disp, _ = space.periodic(L)
    R = torch.tensor(g['real_position'].astype(np.float32), device=cuda)
    sp = torch.tensor(g['species'], device=cuda)
    efn = energy.soft_sphere_pair(disp, sp, g['sigma'])
    E = float(efn(R))
    assert abs(E - float(g['energy'])) < 2e-5 * max(1.0, abs(float(g['energy'])))
    P = float(quantity.pressure(efn, R, g['box']))
    assert abs(P - float(g['pressure'])) < 2e-5


def test_soft_sphere_neighbor_list_species(cuda):
    """Bidisperse 2D soft spheres through the neighbour-list builder vs the oracle."""
    from jax_md_gb300 import energy, partition, space
    R, L, species = O.bidisperse_2d(2000, seed=4)
    sigma = np.array([[1.0, 1.2], [1.2, 1.4]])
    disp, _ = space.periodic(float(L))
    nfn, efn = energy.soft_sphere_neighbor_list(disp, float(L), torch.tensor(species, device=cuda),
                                                sigma=sigma, format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    E, F, _, W = efn.compute(Rt, nb, virial=True)
    spec = O.PairSpec(kind='soft_sphere', sigma=sigma, species=species)
    Eo, Fo, Wo = O.pair_energy_forces(spec, R, nb.idx.cpu().numpy(), O.DENSE, np.full(2, L))
    assert abs(float(E) - Eo) <= 1e-5 * abs(Eo)
    assert np.abs(F.cpu().numpy() - Fo).max() < FORCE_ATOL
    w = W.cpu().numpy()
    assert np.abs(w - np.array([Wo[0, 0], Wo[1, 1], Wo[0, 1]])).max() <= 1e-5 * np.abs(Wo).max()


def test_kob_andersen_species(cuda):
    """Binary LJ with species matrices (global cutoff 2.5 max sigma, energy.py:319-320)."""
    from jax_md_gb300 import energy, partition, space
    R, P, L = fcc_system(8, seed=2)           # lattice start: no overlaps
    rng = np.random.default_rng(2)
    species = (rng.uniform(size=len(R)) < 0.2).astype(np.int32)
    sigma = np.array([[1.0, 0.8], [0.8, 0.88]])
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    disp, _ = space.periodic(float(L))
    nfn, efn = energy.lennard_jones_neighbor_list(disp, float(L), torch.tensor(species, device=cuda),
                                                  sigma=sigma, epsilon=eps, dr_threshold=0.3,
                                                  format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    E, F, _, _ = efn.compute(Rt, nb)
    spec = O.PairSpec(kind='lj', sigma=sigma, epsilon=eps, species=species)
    Eo, Fo, _ = O.pair_energy_forces(spec, R, nb.idx.cpu().numpy(), O.DENSE, np.full(3, L))
    assert abs(float(E) - Eo) <= 1e-5 * abs(Eo)
    assert np.abs(F.cpu().numpy() - Fo).max() < FORCE_ATOL
