"""Host-side logic of smap (no GPU): parameter packing into the pair struct
(scalars, species matrices, the potentials' own defaults) and the mapping of
the kernels' gradient bins onto sigma / epsilon (the cutoff-scale bin is
credited to the largest sigma, as jax.grad through jnp.max does,
energy.py:319-320)."""
import numpy as np
import pytest
import torch

from jax_md_gb300 import _native as N
from jax_md_gb300 import energy, smap


def test_param_matrix_packing():
    m = smap._param_matrix(2.5, 0, 'sigma')
    assert m.shape == (8, 8) and np.all(m == 2.5)
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    m = smap._param_matrix(torch.tensor(sig), 2, 'sigma')
    np.testing.assert_allclose(m[:2, :2], sig)
    with pytest.raises(NotImplementedError):
        smap._param_matrix(sig, 0, 'sigma')            # a matrix needs species
    with pytest.raises(ValueError):
        smap._param_matrix(np.ones((9, 9)), 9, 'sigma')
    with pytest.raises(ValueError):
        smap._param_matrix(np.ones((2, 2, 2)), 2, 'sigma')


def test_pair_struct_defaults_per_potential():
    lj = energy.multiplicative_isotropic_cutoff(energy.lennard_jones, 2.0, 2.5)
    p = smap.make_pair_struct(lj, {}, 0)
    assert p.kind == N.LJ and (p.sigma[0][0], p.epsilon[0][0]) == (1.0, 1.0)
    assert (p.r_onset, p.r_cutoff) == (2.0, 2.5)
    p = smap.make_pair_struct(energy.soft_sphere, {'sigma': 1.4}, 0)
    assert p.kind == N.SOFT_SPHERE and p.alpha[0][0] == 2.0
    assert abs(p.sigma[0][0] - 1.4) < 1e-6
    p = smap.make_pair_struct(energy.truncated(energy.lennard_jones, 2.5), {}, 0)
    assert p.kind == N.LJ_TRUNCATED and p.r_cutoff == 2.5


def test_bins_to_grads_shapes_and_cutoff_credit():
    bins = torch.zeros(130, dtype=torch.float64)
    bins[0 * 8 + 1] = 2.0      # d/d sigma[0][1]
    bins[1 * 8 + 0] = 3.0      # d/d sigma[1][0]
    bins[64 + 1 * 8 + 1] = 5.0 # d/d epsilon[1][1]
    bins[128] = 7.0            # cutoff scale max(sigma)
    sig = torch.tensor([[1.0, 0.8], [0.8, 1.2]])
    eps = torch.tensor([[1.0, 1.5], [1.5, 0.5]])
    gs, ge = smap._bins_to_grads(bins, None, sig, eps)
    np.testing.assert_array_equal(gs.numpy(), [[0.0, 2.0], [3.0, 7.0]])   # credit at argmax
    np.testing.assert_array_equal(ge.numpy(), [[0.0, 0.0], [0.0, 5.0]])
    s0, e0 = smap._bins_to_grads(bins, None, torch.tensor(1.0), torch.tensor(1.0))
    assert float(s0) == 0.0 + 7.0 and float(e0) == 0.0
    none_s, none_e = smap._bins_to_grads(bins, None, None, None)
    assert none_s is None and none_e is None
