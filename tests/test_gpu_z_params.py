"""Per-particle parameter arrays on the GPU (combined as 0.5 (p_i + p_j),
smap.py:833-838, run through the species table): the golden jammed
soft-sphere packing given as per-particle diameters, and a bidisperse LJ
neighbour list with per-particle sigma and epsilon against the oracle.

The file sorts after the other GPU test files (and before the
allocation-free test, which must come last): its tests are among the
newest, and a failure here leaves the earlier files' results intact in a run
that stops at the first failure.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import GOLDEN, fcc_system

pytestmark = pytest.mark.gpu


def test_jammed_soft_sphere_per_particle_diameters(cuda):
    """quantity_test.py:134-150's golden packing with its species matrix
    replaced by per-particle diameters d_i = sigma[s_i, s_i] (the matrix is
    additive: sigma_01 = (sigma_00 + sigma_11) / 2): the golden energy and
    pressure, f32 tolerance 2e-5."""
    from jax_md_gb300 import energy, quantity, space
    g = np.load(GOLDEN / 'jammed_soft_sphere_2d.npz')
    sig = g['sigma']
    assert abs(sig[0, 1] - 0.5 * (sig[0, 0] + sig[1, 1])) < 1e-12
    d = np.diag(sig)[g['species']]
    L = np.diag(g['box']).astype(np.float32)
    disp, _ = space.periodic(L)
    R = torch.tensor(g['real_position'].astype(np.float32), device=cuda)
    efn = energy.soft_sphere_pair(disp, None, d)
    E = float(efn(R))
    assert abs(E - float(g['energy'])) < 2e-5 * max(1.0, abs(float(g['energy'])))
    P = float(quantity.pressure(efn, R, g['box']))
    assert abs(P - float(g['pressure'])) < 2e-5


def test_lj_neighbor_list_per_particle_sigma_epsilon(cuda):
    """LJ with per-particle sigma in {0.95, 1.0, 1.05} and epsilon in {1, 1.5}
    (radii from max sigma, energy.py:319-320) through a Dense list: forces
    within 1e-4 max-abs and energy within 1e-5 relative of the oracle's
    per-particle evaluation."""
    from jax_md_gb300 import energy, partition, space
    R, P, L = fcc_system(7, 3)
    rng = np.random.default_rng(12)
    sig = rng.choice([0.95, 1.0, 1.05], len(R))
    eps = rng.choice([1.0, 1.5], len(R))
    disp, _ = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, sigma=sig, epsilon=eps,
                                                  dr_threshold=0.3, format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    E, F, _, _ = efn.compute(Rt, nb)
    spec = O.PairSpec(kind='lj', sigma=sig, epsilon=eps)
    Eo, Fo, _ = O.pair_energy_forces(spec, R, nb.idx.cpu().numpy(), O.DENSE, np.full(3, L))
    assert abs(float(E) - Eo) <= 1e-5 * abs(Eo)
    assert np.abs(F.cpu().numpy() - Fo).max() < 1e-4
