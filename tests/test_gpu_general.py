"""periodic_general cells (fractional coordinates) on the GPU against the oracle.

Restates the reference's general-cell tests (tests/partition_test.py:462-669):
random triclinic cells, neighbour lists binned in the unit cube with the
fractional cell size, pair energies through the cell, resized cells through
the ``box`` keyword; plus a short NVE trajectory in a sheared cell compared
with the FP64 oracle step by step.
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import LJ_DT, fcc_system, lj_spec, near_cutoff_pairs

pytestmark = pytest.mark.gpu


def _triclinic(rng, L):
    """Upper-triangular cell from edges in [L/2, 3L] and angles in [45, 125]
    degrees (the construction of partition_test.py:536-560), rounded to
    float32 so the kernels and the oracle use the same cell."""
    while True:
        a, b, c = rng.uniform(0.5 * L, 3 * L, 3)
        al, be, ga = np.radians(rng.uniform(45.0, 125.0, 3))
        xx, yy, xy, xz = a, b * np.sin(ga), b * np.cos(ga), c * np.cos(be)
        yz = (b * c * np.cos(al) - xy * xz) / yy
        zz2 = c * c - xz * xz - yz * yz
        if zz2 > 0:
            T = np.array([[xx, xy, xz], [0.0, yy, yz], [0.0, 0.0, np.sqrt(zz2)]])
            return T.astype(np.float32).astype(np.float64)


def _cells(seed, count, N, rho, cutoff, need_cells=True):
    rng = np.random.default_rng(seed)
    L = (N / rho) ** (1 / 3)
    out = []
    while len(out) < count:
        T = _triclinic(rng, L)
        if need_cells and not O.fractional_cell_size(T, cutoff) < np.float32(1 / 3):
            continue
        U = rng.uniform(0, 1, (N, 3)).astype(np.float32)
        out.append((T, U))
    return out


@pytest.mark.parametrize('fmt', [0, 1, 2], ids=['Dense', 'Sparse', 'OrderedSparse'])
def test_general_cell_lists_match_oracle(cuda, fmt):
    from jax_md_gb300 import partition, space
    f = [partition.Dense, partition.Sparse, partition.OrderedSparse][fmt]
    r_cut, skin = 2.0, 0.25
    cutoff = float(np.float32(np.float32(r_cut) + np.float32(skin)))
    for T, U in _cells(21 + fmt, 4, 400, 0.2, cutoff):
        disp, _ = space.periodic_general(torch.tensor(T))
        fns = partition.neighbor_list(disp, T, r_cut, skin, fractional_coordinates=True, format=f)
        nb = fns.allocate(torch.tensor(U, device=cuda))
        sp = O.PeriodicGeneral(T)
        onl = O.NeighborListOracle(T, np.float32(r_cut), np.float32(skin), fmt=fmt, space=sp,
                                   fractional=True)
        onb = onl.allocate(U)
        assert onb.use_cell_list and nb.cell_list_capacity is not None
        assert int(nb.error.code) == onb.error
        skip = near_cutoff_pairs(U, sp, cutoff)
        got = nb.idx.cpu().numpy()
        if fmt == 0 and not skip:
            np.testing.assert_array_equal(got, onb.idx)  # entry order included
        gs = O.neighbor_sets(O.NeighborListO(got, U, 0, None, 0, fmt, True), len(U))
        ws = O.neighbor_sets(onb, len(U))
        for i in range(len(U)):
            assert [j for j in gs[i] if (i, j) not in skip] == \
                   [j for j in ws[i] if (i, j) not in skip]


def _soft(sigma=2.5):
    return O.PairSpec(kind='soft_sphere', sigma=sigma, epsilon=1.0, alpha=2.0)


def test_general_cell_energy_and_forces_match_oracle(cuda):
    """Pair energy over the fractional list equals the all-pairs energy
    through the cell (partition_test.py:565-605); forces and virial match the
    oracle's.  Soft spheres of diameter 2.5 (bounded at overlap, as random
    positions need)."""
    from jax_md_gb300 import energy, partition, space
    spec = _soft()
    for T, U in _cells(31, 4, 500, 0.3, 2.7):
        disp, _ = space.periodic_general(torch.tensor(T))
        nfn, efn = energy.soft_sphere_neighbor_list(disp, T, sigma=2.5, dr_threshold=0.2,
                                                    fractional_coordinates=True,
                                                    format=partition.Dense)
        Ut = torch.tensor(U, device=cuda)
        nb = nfn.allocate(Ut)
        assert nb.cell_list_capacity is not None
        e, F, _, W = efn.compute(Ut, nb, virial=True)
        E_all, F_all, W_all = O.all_pairs_energy_forces(spec, U, O.PeriodicGeneral(T))
        assert abs(E_all) > 0.25
        assert abs(float(e) - E_all) <= 1e-5 * max(1.0, abs(E_all)), (float(e), E_all)
        assert np.abs(F.cpu().numpy() - F_all).max() <= 1e-4 * max(1.0, np.abs(F_all).max())
        w = W.cpu().numpy()
        wo = np.array([W_all[0, 0], W_all[1, 1], W_all[2, 2], W_all[0, 1], W_all[0, 2],
                       W_all[1, 2]])
        assert np.abs(w - wo).max() <= 1e-5 * np.abs(wo).max()


@pytest.mark.parametrize('factor', [0.5, 2.0])
def test_general_cell_resize(cuda, factor):
    """update(R, box=factor T) and energy(R, box=factor T)
    (partition_test.py:607-669): a grown cell gives the all-pairs energy
    through the new cell; a shrunk one raises cell_size_too_small."""
    from jax_md_gb300 import energy, partition, space
    spec = _soft()
    checked = 0
    for T, U in _cells(41, 4, 400, 0.05, 2.7, need_cells=False):
        disp, _ = space.periodic_general(torch.tensor(T))
        # dr_threshold 0: every update rebuilds, as in the reference's test
        nfn, efn = energy.soft_sphere_neighbor_list(disp, T, sigma=2.5, dr_threshold=0.0,
                                                    fractional_coordinates=True,
                                                    format=partition.Dense,
                                                    capacity_multiplier=1.0)
        Ut = torch.tensor(U, device=cuda)
        nb = nfn.allocate(Ut)
        Tn = (T * factor).astype(np.float32).astype(np.float64)
        nb = nb.update(Ut, box=torch.tensor(Tn))
        if factor > 1:
            e = float(efn(Ut, nb, box=torch.tensor(Tn)))
            E_all = O.all_pairs_energy_forces(spec, U, O.PeriodicGeneral(Tn))[0]
            assert abs(e - E_all) <= 1e-5 * max(1.0, abs(E_all)), (e, E_all)
            assert not bool(nb.cell_size_too_small)
            checked += 1
        elif nb.cell_list_capacity is not None:
            assert bool(nb.cell_size_too_small)
            checked += 1
    assert checked > 0


def test_general_cell_nve_matches_oracle(cuda):
    """40 velocity-Verlet steps of an FCC LJ solid in a sheared cell
    (fractional positions, shift u <- mod(u + T^-1 dR, 1)), step by step
    against the FP64 oracle from the same float32 start; then simulate.run
    over the same steps gives the same state."""
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(7)
    T = np.array([[L, 0.08 * L, -0.05 * L], [0.0, L, 0.06 * L], [0.0, 0.0, L]])
    T = T.astype(np.float32).astype(np.float64)
    U = (R.astype(np.float64) / L).astype(np.float32)
    disp, shift = space.periodic_general(torch.tensor(T))
    nfn, efn = energy.lennard_jones_neighbor_list(disp, T, dr_threshold=0.3,
                                                  fractional_coordinates=True,
                                                  format=partition.Dense)
    Ut = torch.tensor(U, device=cuda)
    nb = nfn.allocate(Ut)
    init, apply = simulate.nve(efn, shift, LJ_DT)
    st = init(0, Ut, momenta=torch.tensor(P, device=cuda), neighbor=nb)
    st2 = st.copy()
    steps = 40
    for _ in range(steps):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    assert not bool(nb.did_buffer_overflow)
    # oracle: the same loop in FP64
    sp = O.PeriodicGeneral(T)
    spec = lj_spec()
    nl = O.NeighborListOracle(T, 2.5, 0.3, space=sp, fractional=True)
    state = {'nb': nl.allocate(U)}

    def fn(X):
        state['nb'] = nl.update(X, state['nb'])
        return O.pair_energy_forces(spec, X, state['nb'].idx, O.DENSE, sp)[1]
    Ud, Pd = U.astype(np.float64), P.astype(np.float64)
    F = fn(Ud)
    for _ in range(steps):
        Ud, Pd, F = O.velocity_verlet(fn, Ud, Pd, F, 1.0, LJ_DT, sp)
    d = sp.displacement(st.position.cpu().numpy(), Ud)   # real-space difference
    assert np.abs(d).max() < 1e-4, np.abs(d).max()
    assert np.abs(st.momentum.cpu().numpy() - Pd).max() < 1e-3
    # simulate.run takes the same per-step loop for general cells
    nb2 = nfn.allocate(st2.position)
    st2, nb2 = simulate.run(apply, st2, nb2, steps)
    assert torch.equal(st2.position, st.position)
    assert torch.equal(st2.momentum, st.momentum)
