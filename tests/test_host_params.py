"""Per-particle parameter arrays on the host (no GPU): the reference's
default combinator 0.5 (p_i + p_j) (smap.py:833-838) is mapped exactly onto
the species table the kernels read, for up to 8 distinct values."""
import numpy as np
import pytest
import torch

from jax_md_gb300 import energy, partition, smap, space
from oracle import md_oracle as O
from tests.helpers import fcc_system


def test_table_of_bidisperse_diameters():
    d = np.array([1.0, 1.4, 1.4, 1.0, 1.4])
    params, species, S = smap._per_particle_table({'sigma': d, 'epsilon': 1.0})
    assert S == 2 and species.tolist() == [0, 1, 1, 0, 1]
    np.testing.assert_allclose(params['sigma'], [[1.0, 1.2], [1.2, 1.4]], rtol=1e-7)
    assert params['epsilon'] == 1.0
    assert smap._per_particle_table({'sigma': 1.0}) is None


def test_table_reproduces_per_particle_energies():
    """The species-matrix form of the table gives the oracle's per-particle
    energies and forces (to the float32 rounding of the pairwise means)."""
    rng = np.random.default_rng(8)
    R, _, L = fcc_system(4, 9)
    box = np.full(3, L)
    n = len(R)
    sig = rng.choice([0.9, 1.0, 1.15], n)
    eps = rng.choice([1.0, 2.0], n)
    params, species, S = smap._per_particle_table({'sigma': sig, 'epsilon': eps})
    assert S <= 6
    a = O.all_pairs_energy_forces(O.PairSpec(kind='lj', sigma=sig, epsilon=eps), R, box)
    b = O.all_pairs_energy_forces(O.PairSpec(kind='lj', sigma=params['sigma'],
                                             epsilon=params['epsilon'], species=species), R, box)
    assert abs(a[0] - b[0]) <= 1e-6 * abs(a[0])
    np.testing.assert_allclose(a[1], b[1], rtol=1e-5, atol=1e-5 * np.abs(a[1]).max())


def test_resolve_maps_static_and_dynamic_arrays():
    disp, _ = space.periodic(10.0)
    d = np.array([1.0, 1.4, 1.0, 1.4])
    _, efn = energy.soft_sphere_neighbor_list(disp, 10.0, sigma=d, format=partition.Dense)
    species, p = efn._resolve(torch.zeros((4, 2)), {})
    assert p.n_species == 2 and species.tolist() == [0, 1, 0, 1]
    assert abs(p.sigma[0][1] - 1.2) < 1e-6 and abs(p.sigma[1][1] - 1.4) < 1e-6
    species, p = efn._resolve(torch.zeros((4, 2)), {'sigma': np.array([1.0, 1.0, 1.2, 1.2])})
    assert species.tolist() == [0, 0, 1, 1] and abs(p.sigma[0][1] - 1.1) < 1e-6


def test_continuous_per_particle_arrays_go_to_the_generic_kernels():
    """More distinct per-particle values than the species table holds: the
    pair struct carries per-atom arrays (sigma[0][0] = max sigma, the cutoff
    scale), no species, and the energy reports it (the engine falls back to
    the per-step loop)."""
    disp, _ = space.periodic(10.0)
    sig = np.linspace(1.0, 1.5, 12)
    eps = np.linspace(0.5, 2.0, 12)
    _, efn = energy.soft_sphere_neighbor_list(disp, 10.0, sigma=sig, epsilon=eps,
                                              format=partition.Dense)
    assert efn.has_particle_arrays()
    species, pair = efn._resolve(torch.zeros((12, 2)), {})
    assert species is None and pair.n_species == 0
    assert pair.particle_sigma and pair.particle_epsilon
    assert abs(pair.sigma[0][0] - 1.5) < 1e-6
    # arrays the species table can hold stay on the species path
    _, efn2 = energy.soft_sphere_neighbor_list(disp, 10.0, sigma=np.array([1.0, 1.4, 1.0]),
                                               format=partition.Dense)
    assert not efn2.has_particle_arrays()
    with pytest.raises(NotImplementedError, match='alpha'):
        smap._per_particle_table({'alpha': np.linspace(2.0, 3.0, 12)})


def test_unsupported_per_particle_cases():
    disp, _ = space.periodic(10.0)
    _, efn = energy.soft_sphere_neighbor_list(disp, 10.0, sigma=np.array([1.0, 1.4, 1.0]),
                                              format=partition.Dense)
    with pytest.raises(ValueError, match='one entry per atom'):
        efn._resolve(torch.zeros((5, 2)), {})
    with pytest.raises(NotImplementedError, match='species array'):
        efn._resolve(torch.zeros((3, 2)), {'species': torch.tensor([0, 1, 0])})
    with pytest.raises(NotImplementedError, match='species matrices'):
        smap._per_particle_table({'sigma': np.ones(3), 'epsilon': np.ones((2, 2))})
    with pytest.raises(NotImplementedError, match='per-particle'):
        smap._param_tensor(torch.ones(3, requires_grad=True))
