"""Per-particle parameter arrays on the GPU (combined as 0.5 (p_i + p_j),
smap.py:833-838): through the species table (up to 8 distinct values: the
golden jammed soft-sphere packing given as per-particle diameters, a
bidisperse LJ list) and as per-atom arrays read by the generic pair kernels
(continuous values: polydisperse soft spheres and LJ in every list format,
and an NVE run of them) against the oracle.

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


@pytest.mark.parametrize('fmt', ['Dense', 'Sparse', 'OrderedSparse'])
def test_polydisperse_soft_spheres_continuous_diameters(cuda, fmt):
    """2-D soft spheres with diameters uniform in [1.0, 1.4] (every atom its
    own value: per-atom arrays, no species table), packing fraction 0.84:
    energy within 1e-6 relative, forces within 1e-4 + 4e-6 sum_j |F_ij|
    (overlapped packing) and the virial of the oracle."""
    from jax_md_gb300 import energy, partition, quantity, space
    rng = np.random.default_rng(21)
    n = 1200
    d = rng.uniform(1.0, 1.4, n)
    L = float(np.sqrt(np.sum(np.pi * d ** 2 / 4) / 0.84))
    R = (rng.uniform(0, L, (n, 2))).astype(np.float32)
    disp, _ = space.periodic(L)
    nfn, efn = energy.soft_sphere_neighbor_list(disp, L, sigma=d, dr_threshold=0.2,
                                                format=getattr(partition, fmt))
    assert efn.has_particle_arrays()
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    E, F, _, W = efn.compute(Rt, nb, virial=True)
    spec = O.PairSpec(kind='soft_sphere', sigma=d, epsilon=1.0, alpha=2.0)
    ofmt = {'Dense': O.DENSE, 'Sparse': O.SPARSE, 'OrderedSparse': O.ORDERED_SPARSE}[fmt]
    Eo, Fo, Wo = O.pair_energy_forces(spec, R, nb.idx.cpu().numpy(), ofmt, np.full(2, L))
    assert abs(float(E) - Eo) <= 1e-6 * abs(Eo)
    scale = O.pair_force_abs_sum(spec, R, nb.idx.cpu().numpy(), ofmt, np.full(2, L))
    err = np.abs(F.cpu().numpy() - Fo).max(1)
    assert np.all(err <= 1e-4 + 4e-6 * scale), err.max()
    w = W.cpu().numpy()
    assert np.abs(w - np.array([Wo[0, 0], Wo[1, 1], Wo[0, 1]])).max() <= 1e-6 * np.abs(Wo).max()


def test_lj_continuous_sigma_epsilon_and_run(cuda):
    """3-D LJ with sigma uniform in [0.92, 1.08] and epsilon in [0.7, 1.3]
    per atom (radii from max sigma): forces within 1e-4 and energy within
    1e-6 relative of the oracle; simulate.run of such an energy takes the
    per-step loop and equals it step for step."""
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(7, 4)
    rng = np.random.default_rng(13)
    sig = rng.uniform(0.92, 1.08, len(R))
    eps = rng.uniform(0.7, 1.3, len(R))
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, sigma=sig, epsilon=eps,
                                                  dr_threshold=0.3, format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    E, F, _, _ = efn.compute(Rt, nb)
    spec = O.PairSpec(kind='lj', sigma=sig, epsilon=eps)
    Eo, Fo, _ = O.pair_energy_forces(spec, R, nb.idx.cpu().numpy(), O.DENSE, np.full(3, L))
    assert abs(float(E) - Eo) <= 1e-6 * abs(Eo)
    assert np.abs(F.cpu().numpy() - Fo).max() < 1e-4
    init, apply = simulate.nve(efn, shift, 0.004)
    st_a = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    nb_b = nfn.allocate(Rt)
    st_b = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb_b)
    st_a, nb = simulate.run(apply, st_a, nb, 15)
    for _ in range(15):
        nb_b = nb_b.update(st_b.position)
        st_b = apply(st_b, neighbor=nb_b)
    torch.cuda.synchronize()
    assert torch.equal(st_a.position, st_b.position)
    assert torch.equal(st_a.momentum, st_b.momentum)
