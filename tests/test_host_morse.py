"""Host side of the Morse potential (no GPU): the pair parameters the
builders hand to the kernels, the elementwise function against the oracle,
and the C ABI's argument checks."""
import ctypes
import math

import numpy as np
import pytest
import torch

from jax_md_gb300 import _native as N
from jax_md_gb300 import energy, partition, smap, space
from oracle import md_oracle as O


def test_morse_neighbor_list_pair_parameters():
    """energy.py:400-440: defaults eps 5, alpha 5; radii 2.0 / 2.5 as given
    (not multiples of sigma); the list cutoff is r_cutoff."""
    disp, _ = space.periodic(10.0)
    nfn, efn = energy.morse_neighbor_list(disp, 10.0, sigma=1.3, dr_threshold=0.4)
    p = smap.make_pair_struct(efn.fn, efn.params, 0)
    assert p.kind == N.MORSE and p.per_pair_cutoff == 0
    assert (p.r_onset, p.r_cutoff) == (2.0, 2.5)
    assert math.isclose(p.sigma[0][0], 1.3, rel_tol=1e-7)
    assert p.epsilon[0][0] == 5.0 and p.alpha[0][0] == 5.0
    assert efn.fn.kind == N.MORSE and nfn is not None


def test_plain_morse_defaults_and_unbounded_range():
    """The bare elementwise function keeps energy.morse's defaults
    (energy.py:346-352) and has no cutoff (infinite radii)."""
    p = smap.make_pair_struct(energy.morse, {}, 0)
    assert p.kind == N.MORSE and p.epsilon[0][0] == 5.0 and p.alpha[0][0] == 5.0
    assert p.r_cutoff > 1e38 and p.r_onset == p.r_cutoff


def test_morse_species_matrices_packed():
    sig = np.array([[1.0, 1.1], [1.1, 1.2]])
    alp = np.array([[5.0, 4.0], [4.0, 6.0]])
    disp, _ = space.periodic(10.0)
    _, efn = energy.morse_neighbor_list(disp, 10.0, torch.zeros(4, dtype=torch.int32), sigma=sig,
                                        alpha=alp, format=partition.Dense)
    species, p = efn._resolve(torch.zeros((4, 3)), {})
    assert p.n_species == 2 and species is not None
    assert math.isclose(p.sigma[1][0], 1.1, rel_tol=1e-7) and p.alpha[1][1] == 6.0
    assert p.epsilon[0][1] == 5.0


def test_morse_elementwise_matches_oracle():
    r = np.linspace(0.6, 2.6, 201)
    cut = energy.multiplicative_isotropic_cutoff(energy.morse, 2.0, 2.5)
    got = cut(torch.tensor(r), sigma=1.1, epsilon=3.0, alpha=4.0).numpy()
    U, _, _ = O.pair_terms(O.PairSpec(kind='morse', sigma=1.1, epsilon=3.0, alpha=4.0), r)
    np.testing.assert_allclose(got, U, rtol=1e-12, atol=1e-12)
    bare = energy.morse(torch.tensor(r)).numpy()
    np.testing.assert_allclose(bare, O.morse(r)[0], rtol=1e-12, atol=1e-12)


def test_morse_per_pair_cutoff_rejected():
    """Morse radii are absolute: the C ABI refuses per-pair (sigma-scaled)
    radii before touching any buffer."""
    disp, _ = space.periodic(10.0)
    _, efn = energy.morse_neighbor_list(disp, 10.0)
    p = smap.make_pair_struct(efn.fn, efn.params, 0)
    p.per_pair_cutoff = 1
    sp = N.Space()
    sp.dim, sp.periodic = 3, 1
    L = N.lib()
    rc = L.jmd_pair_forces(ctypes.byref(p), ctypes.byref(sp), N.DENSE, None, 4, None, 0, None, 0,
                           0, None, None, 4, None, None, None, None, 0, None)
    assert rc != 0 and b'Morse' in L.jmd_last_error()
    p.per_pair_cutoff = 0
    p.kind = 4
    rc = L.jmd_pair_forces(ctypes.byref(p), ctypes.byref(sp), N.DENSE, None, 4, None, 0, None, 0,
                           0, None, None, 4, None, None, None, None, 0, None)
    assert rc != 0 and b'unknown pair potential' in L.jmd_last_error()
