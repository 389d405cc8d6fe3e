"""NPT Nose-Hoover (simulate.npt_nose_hoover) on the GPU against the oracle.

The golden jammed soft-sphere packing in its periodic_general cell, as the
reference's test_npt_nose_hoover_jammed (tests/simulate_test.py:360-400):
20 steps step by step against the FP64 oracle from the same momenta, then
800 steps with the extended Hamiltonian conserved to the reference's
float32 tolerance and the pressure near its target; and an LJ liquid whose
neighbour list follows the cell through the ``box`` keyword.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import GOLDEN, fcc_system, lj_spec

pytestmark = pytest.mark.gpu


def _jammed(cuda):
    from jax_md_gb300 import energy, space
    g = np.load(GOLDEN / 'jammed_soft_sphere_2d.npz')
    box = g['box'].astype(np.float32).astype(np.float64)
    disp, shift = space.periodic_general(torch.tensor(box))
    E = energy.soft_sphere_pair(disp, torch.tensor(g['species'], device=cuda),
                                sigma=g['sigma'])
    spec = O.PairSpec(kind='soft_sphere', sigma=g['sigma'], epsilon=1.0, alpha=2.0,
                      species=g['species'])

    def force_stress(R, cell):
        e, F, W = O.all_pairs_energy_forces(spec, R, O.PeriodicGeneral(cell))
        return e, F, float(np.trace(W))
    R = g['fractional_position'].astype(np.float32)
    return g, box, shift, E, force_stress, R


def test_npt_steps_match_oracle(cuda):
    from jax_md_gb300 import simulate
    g, box, shift, E, fs, R = _jammed(cuda)
    kT, dt, Pt = 1e-3, 1e-3, float(g['pressure'])
    P = O.maxwell_boltzmann(len(R), 2, kT, seed=3)
    init, apply = simulate.npt_nose_hoover(E, shift, dt, Pt, kT)
    st = init(0, torch.tensor(R, device=cuda), box, momenta=torch.tensor(P, device=cuda))
    s = O.npt_init(fs, R.astype(np.float64), P.astype(np.float64), box, 1.0, kT, dt)
    assert abs(st.dUdV - s['dUdV']) <= 1e-5 * max(1.0, abs(s['dUdV']))
    for _ in range(20):
        st = apply(st)
        s = O.npt_nose_hoover_step(fs, s, Pt, kT, dt)
    cell, _ = O.npt_box(s)
    d = O.PeriodicGeneral(cell).displacement(st.position.cpu().numpy(), s['R'])
    assert np.abs(d).max() < 1e-4, np.abs(d).max()
    assert np.abs(st.momentum.cpu().numpy() - s['P']).max() < 1e-4
    assert abs(st.box_position - s['R_b']) <= 1e-6 + 1e-3 * abs(s['R_b'])
    assert abs(st.box_momentum - s['P_b']) <= 1e-3 * max(abs(s['P_b']), 1e-3)
    np.testing.assert_allclose(simulate.npt_box(st), cell, rtol=1e-6)


def test_npt_jammed_conserves_invariant_and_pressure(cuda):
    """tests/simulate_test.py:360-400: 800 steps, invariant within the
    reference's float32 tolerance (1e-3), pressure within 5% (+0.05)."""
    from jax_md_gb300 import quantity, simulate
    g, box, shift, E, fs, R = _jammed(cuda)
    kT, dt, Pt = 1e-3, 1e-3, float(g['pressure'])
    init, apply = simulate.npt_nose_hoover(E, shift, dt, Pt, kT)
    st = init(7, torch.tensor(R, device=cuda), box)
    H0 = simulate.npt_nose_hoover_invariant(E, st, Pt, kT)
    for k in range(800):
        st = apply(st)
        if k % 40 == 39:
            H = simulate.npt_nose_hoover_invariant(E, st, Pt, kT)
            assert abs(H - H0) <= 1e-3 + 1e-3 * abs(H0), (k, H, H0)
            cell = simulate.npt_box(st)
            ke = quantity._ke_f64(st.momentum, st.mass)
            p = float(quantity.pressure(E, st.position, cell, ke))
            assert abs(p - Pt) <= 0.05 + 0.05 * abs(Pt), (k, p, Pt)


def test_npt_with_neighbor_list_follows_the_cell(cuda):
    """An LJ liquid (N = 500) under NPT with a fractional neighbour list
    updated with the current cell every step (update(R, box=npt_box(state)),
    partition.py:1123-1139) follows the FP64 oracle's all-pairs NPT run for
    20 steps."""
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(5)
    T = (np.eye(3) * L).astype(np.float32).astype(np.float64)
    U = (R.astype(np.float64) / L).astype(np.float32)
    disp, shift = space.periodic_general(torch.tensor(T))
    nfn, efn = energy.lennard_jones_neighbor_list(disp, T, dr_threshold=0.3,
                                                  fractional_coordinates=True,
                                                  format=partition.Dense)
    kT, dt, Pt = 0.722, 0.005, 1.0
    Ut = torch.tensor(U, device=cuda)
    nb = nfn.allocate(Ut)
    init, apply = simulate.npt_nose_hoover(efn, shift, dt, Pt, kT)
    st = init(0, Ut, T, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    spec = lj_spec()

    def fs(X, cell):
        e, F, W = O.all_pairs_energy_forces(spec, X, O.PeriodicGeneral(cell))
        return e, F, float(np.trace(W))
    s = O.npt_init(fs, U.astype(np.float64), P.astype(np.float64), T, 1.0, kT, dt)
    for _ in range(20):
        nb = nb.update(st.position, box=simulate.npt_box(st))
        st = apply(st, neighbor=nb)
        s = O.npt_nose_hoover_step(fs, s, Pt, kT, dt)
    assert not bool(nb.did_buffer_overflow)
    cell, _ = O.npt_box(s)
    d = O.PeriodicGeneral(cell).displacement(st.position.cpu().numpy(), s['R'])
    assert np.abs(d).max() < 1e-4, np.abs(d).max()
    assert np.abs(st.momentum.cpu().numpy() - s['P']).max() < 1e-3
    assert abs(st.box_position - s['R_b']) <= 1e-6 + 1e-3 * abs(s['R_b'])
