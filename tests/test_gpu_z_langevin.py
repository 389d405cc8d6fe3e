"""Langevin dynamics (simulate.nvt_langevin, BAOAB, simulate.py:1102-1171) on
the GPU.  The O step draws its normals from a counter-based generator, so the
oracle replays a device run exactly from (seed, step, atom): the O step
alone, and a BAOAB LJ run step by step.  The reference's own statistical
test (the damped harmonic oscillator, simulate_test.py:872-915) checks the
dynamics in distribution.

The file sorts after the other GPU test files (and before the
allocation-free test, which must come last): its tests are among the
newest, and a failure here leaves the earlier files' results intact in a run
that stops at the first failure.
"""
import ctypes
import math

import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import fcc_system

pytestmark = pytest.mark.gpu


def test_langevin_o_step_replays_exactly(cuda):
    """jmd_langevin_o_step: its draws equal the oracle's restatement of the
    generator (exact float32 uniforms, float32 Box-Muller: 2e-6) and
    p <- c1 p + c2 sqrt(m) xi holds."""
    from jax_md_gb300 import _native as N
    n, seed, step = 5000, 2024, 17
    rng = np.random.default_rng(1)
    p0 = rng.standard_normal((n, 3)).astype(np.float32)
    m = rng.uniform(0.5, 4.0, n).astype(np.float32)
    P = torch.zeros((n, 4), dtype=torch.float32, device=cuda)
    P[:, :3] = torch.tensor(p0, device=cuda)
    mt = torch.tensor(m, device=cuda)
    noise = torch.zeros((n, 4), dtype=torch.float32, device=cuda)
    c1, c2 = np.float32(math.exp(-0.3 * 0.01)), np.float32(0.7)
    N.check(N.lib().jmd_langevin_o_step(P.data_ptr(), 4, n, 3, mt.data_ptr(), 1.0, float(c1),
                                        float(c2), seed, step, noise.data_ptr(), N.stream_ptr()),
            'langevin_o_step')
    torch.cuda.synchronize()
    _, z = O.langevin_normals(seed, step, n)
    np.testing.assert_allclose(noise.cpu().numpy(), z, rtol=2e-6, atol=2e-6)
    want = float(c1) * p0.astype(np.float64) + float(c2) * np.sqrt(m.astype(np.float64))[:, None] * z[:, :3]
    np.testing.assert_allclose(P[:, :3].cpu().numpy(), want, rtol=1e-5, atol=1e-5)


def test_langevin_lj_run_matches_oracle_replay(cuda):
    """Ten BAOAB steps of LJ (N = 500, kT 0.722, gamma 0.5) through
    simulate.nvt_langevin against the oracle's BAOAB step fed the draws of
    the same (seed, step): positions within 1e-4, momenta within 1e-3."""
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(5, 4)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3, format=partition.Dense)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    dt, kT, gamma, seed, steps = 0.005, 0.722, 0.5, 99, 10
    init, apply = simulate.nvt_langevin(efn, shift, dt, kT, gamma=gamma)
    st = init(seed, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    for _ in range(steps):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    torch.cuda.synchronize()
    assert st.step == steps
    box = np.full(3, L)
    nl = O.NeighborListOracle(box, 2.5, 0.3, fmt=O.DENSE)
    h = {'nb': nl.allocate(R)}

    def fn(X):
        h['nb'] = nl.update(X, h['nb'])
        return O.pair_energy_forces(O.PairSpec(kind='lj'), X, h['nb'].idx, O.DENSE, box)[1]
    X, Pd = R.astype(np.float64), P.astype(np.float64)
    F = fn(X)
    for k in range(steps):
        _, z = O.langevin_normals(st.seed, k, len(R))
        X, Pd, F = O.nvt_langevin_step(fn, X, Pd, F, 1.0, dt, kT, gamma, box, z[:, :3])
    d = O.displacement(st.position[:, :3].cpu().numpy(), X, box)
    assert np.abs(d).max() < 1e-4, np.abs(d).max()
    assert np.abs(st.momentum[:, :3].cpu().numpy() - Pd).max() < 1e-3


def test_langevin_harmonic_matches_theory(cuda):
    """simulate_test.py:872-915 on the device: 200,000 independent 1-D
    oscillators (100,000 particles in 2-D; alpha 1, mass 3, gamma 3,
    kT 0.25, dt 1e-4) from x = 1 with thermal momenta; after 1000 steps the
    mean position and the momentum autocorrelation follow the analytic
    solution within four standard errors plus 1e-3 relative."""
    from jax_md_gb300 import simulate, space
    alpha, mass, gamma, kT, dt, steps, n = 1.0, 3.0, 3.0, 0.25, 1e-4, 1000, 100000
    _, shift = space.free()
    init, apply = simulate.nvt_langevin(lambda R, **kw: 0.5 * alpha * (R * R).sum(), shift, dt, kT,
                                        gamma=gamma)
    g = torch.Generator(device=cuda).manual_seed(5)
    P0 = torch.randn((n, 2), generator=g, device=cuda) * math.sqrt(kT * mass)
    st = init(11, torch.ones((n, 2), device=cuda), mass=mass, momenta=P0)
    P0 = st.momentum.clone()
    for _ in range(steps):
        st = apply(st)
    torch.cuda.synchronize()
    X = st.position.double().cpu().numpy().reshape(-1)
    pp = (st.momentum.double() * P0.double()).cpu().numpy().reshape(-1)
    d = math.sqrt(gamma ** 2 / 4 - alpha / mass)
    b1, b2 = gamma / 2 + d, gamma / 2 - d
    A, B = -b2 / (b1 - b2), b1 / (b1 - b2)
    Z = kT / (2 * d * mass)
    t = steps * dt
    pos = A * math.exp(-b1 * t) + B * math.exp(-b2 * t)
    mom = Z * (-b2 * math.exp(-b2 * t) + b1 * math.exp(-b1 * t)) * mass ** 2
    m = X.size
    assert abs(X.mean() - pos) <= 4 * X.std() / math.sqrt(m) + 1e-3 * abs(pos), (X.mean(), pos)
    assert abs(pp.mean() - mom) <= 4 * pp.std() / math.sqrt(m) + 1e-3 * abs(mom), (pp.mean(), mom)
