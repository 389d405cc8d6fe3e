"""NVE / NVT integration on the GPU against the FP64 oracle.

Short trajectories are compared step by step with the f64 oracle run from the
same fp32 inputs (before chaotic divergence sets in); longer runs check energy
conservation (NVE drift) and the Nose-Hoover invariant.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import LJ_DT, LJ_KT, fcc_system, lj_spec

pytestmark = pytest.mark.gpu


def _lj(cuda, n_cells, fmt='Dense'):
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(n_cells)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3,
                                                  format=getattr(partition, fmt))
    return R, P, L, disp, shift, nfn, efn


def _oracle_nve(R, P, L, steps):
    box = np.full(3, L)
    spec = lj_spec()
    nl = O.NeighborListOracle(box, 2.5, 0.3)
    nb = nl.allocate(R)
    Rd, Pd = R.astype(np.float64), P.astype(np.float64)
    state = {'nb': nb}

    def fn(X):
        state['nb'] = nl.update(X, state['nb'])
        return O.pair_energy_forces(spec, X, state['nb'].idx, O.DENSE, box)[1]
    F = fn(Rd)
    for _ in range(steps):
        Rd, Pd, F = O.velocity_verlet(fn, Rd, Pd, F, 1.0, LJ_DT, box)
    return Rd, Pd


def test_nve_short_trajectory_matches_oracle(cuda):
    from jax_md_gb300 import simulate
    R, P, L, disp, shift, nfn, efn = _lj(cuda, 6)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nve(efn, shift, LJ_DT)
    st = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    steps = 40
    for _ in range(steps):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    assert not bool(nb.did_buffer_overflow)
    Ro, Po = _oracle_nve(R, P, L, steps)
    d = O.displacement(st.position.cpu().numpy(), Ro, np.full(3, L))
    assert np.abs(d).max() < 1e-4
    assert np.abs(st.momentum.cpu().numpy() - Po).max() < 1e-3


def test_nve_energy_drift(cuda):
    from jax_md_gb300 import quantity, simulate
    R, P, L, disp, shift, nfn, efn = _lj(cuda, 10)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nve(efn, shift, LJ_DT)
    st = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)

    def H():
        return float(efn.energy_f64(st.position, nb) + quantity._ke_f64(st.momentum))
    H0 = H()
    for _ in range(1000):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    assert not bool(nb.did_buffer_overflow)
    drift = abs(H() - H0) / len(R)
    assert drift < 2e-3, drift


def test_nvt_matches_oracle_and_conserves_invariant(cuda):
    from jax_md_gb300 import simulate
    R, P, L, disp, shift, nfn, efn = _lj(cuda, 5)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nvt_nose_hoover(efn, shift, LJ_DT, LJ_KT, chain_length=5)
    st = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    H0 = float(simulate.nvt_nose_hoover_invariant(efn, st, LJ_KT, neighbor=nb))
    # oracle, 20 steps
    box = np.full(3, L)
    spec = lj_spec()
    nl = O.NeighborListOracle(box, 2.5, 0.3)
    onb = nl.allocate(R)
    holder = {'nb': onb}

    def fn(X):
        holder['nb'] = nl.update(X, holder['nb'])
        return O.pair_energy_forces(spec, X, holder['nb'].idx, O.DENSE, box)[1]
    Rd, Pd = R.astype(np.float64), P.astype(np.float64)
    F = fn(Rd)
    c = O.nhc_init(Rd.size, O.kinetic_energy(Pd), LJ_KT, float(np.float32(LJ_DT * 100)), 5)
    for k in range(20):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
        Rd, Pd, F, c = O.nvt_nose_hoover_step(fn, Rd, Pd, F, 1.0, c, LJ_DT, LJ_KT, box)
    np.testing.assert_allclose(st.chain.momentum.cpu().numpy(), c.p_xi, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(st.chain.position.cpu().numpy(), c.xi, rtol=1e-4, atol=1e-6)
    assert np.abs(st.momentum.cpu().numpy() - Pd).max() < 1e-3
    for _ in range(480):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    H1 = float(simulate.nvt_nose_hoover_invariant(efn, st, LJ_KT, neighbor=nb))
    assert abs(H1 - H0) / len(R) < 5e-4
