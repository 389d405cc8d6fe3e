"""simulate.initialize_momenta / canonicalize_momenta (simulate.py:141-165)
and the Langevin key split (simulate.py:1157) on CPU tensors: the momenta
follow Maxwell-Boltzmann in distribution (temperature, zero net momentum,
mass scaling), and one key gives independent O-step and momentum streams."""
import math

import numpy as np
import pytest
import torch

from jax_md_gb300 import simulate


@pytest.mark.parametrize('dim', [2, 3])
def test_momenta_are_maxwell_boltzmann(dim):
    n, kT = 200000, 0.722
    R = torch.zeros((n, dim))
    P = simulate.initialize_momenta(R, 1.0, 3, kT)
    assert P.shape == (n, dim) and P.dtype == torch.float32
    # centred: zero net momentum, to the float32 rounding of the subtracted
    # mean (the uncentred mean's standard error is sqrt(kT / N) = 1.9e-3)
    assert torch.abs(P.double().mean(0)).max() < 1e-7
    # temperature sum p^2 / m / (N d) = kT within five standard errors
    T = float((P.double() ** 2).sum() / (n * dim))
    assert abs(T - kT) < 5 * kT * math.sqrt(2.0 / (n * dim))
    # each component is normal: fourth moment 3 (kT)^2
    k4 = float((P.double() ** 4).mean())
    assert abs(k4 - 3 * kT ** 2) < 5 * kT ** 2 * math.sqrt(96.0 / (n * dim))


def test_momenta_scale_with_sqrt_mass():
    n, kT = 100000, 1.3
    R = torch.zeros((n, 3))
    m = torch.where(torch.arange(n) % 2 == 0, torch.tensor(1.0), torch.tensor(9.0))
    P = simulate.initialize_momenta(R, m, 11, kT)
    for mass in (1.0, 9.0):
        sel = P[m == mass].double()
        var = float((sel ** 2).mean())
        assert abs(var - mass * kT) < 5 * mass * kT * math.sqrt(2.0 / sel.numel())
    # kinetic temperature of the whole system, sum p^2 / m / (N d)
    T = float((P.double() ** 2 / m[:, None].double()).sum() / (3 * n))
    assert abs(T - kT) < 5 * kT * math.sqrt(2.0 / (3 * n))


def test_single_particle_is_not_centred():
    R = torch.zeros((1, 3))
    P = simulate.initialize_momenta(R, 1.0, 5, 1.0)
    assert float(torch.abs(P).sum()) > 0


def test_seeds_reproduce_and_differ():
    R = torch.zeros((1000, 3))
    a = simulate.initialize_momenta(R, 1.0, 7, 1.0)
    b = simulate.initialize_momenta(R, 1.0, 7, 1.0)
    c = simulate.initialize_momenta(R, 1.0, 8, 1.0)
    assert torch.equal(a, b) and not torch.equal(a, c)
    g = torch.Generator().manual_seed(7)
    d = simulate.initialize_momenta(R, 1.0, g, 1.0)
    assert torch.equal(a, d)


def test_canonicalize_momenta():
    st = simulate.NVEState(torch.zeros((4, 3)), torch.zeros((4, 3)), torch.zeros((4, 3)), 1.0)
    assert simulate.canonicalize_momenta(st, None) is st
    p = torch.ones((4, 3))
    assert torch.equal(simulate.canonicalize_momenta(st, p).momentum, p)


def test_langevin_key_split_gives_independent_streams():
    s0 = simulate.split_key(5, 0)
    s1 = simulate.split_key(5, 1)
    assert s0 != s1 and s0 != 5 and s1 != 5
    assert 0 <= s0 < 2 ** 64 and 0 <= s1 < 2 ** 64
    assert simulate.split_key(5, 0) == s0          # deterministic
    assert simulate.split_key(6, 0) != s0
    g = torch.Generator().manual_seed(5)
    assert simulate.split_key(g, 0) == s0          # a Generator keys by its seed
    assert simulate.split_key(None, 0) == simulate.split_key(0, 0)
    seeds = {simulate.split_key(k, j) for k in range(200) for j in range(2)}
    assert len(seeds) == 400
