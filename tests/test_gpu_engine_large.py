"""The sorted engine at the benchmark's size: LJ on FCC 60^3 x 4 = 864,000
atoms (35 cells per side), NVE through simulate.run with the segment-local
private list, checked against the FP64 oracle:

* every atom's force at the final positions within 1e-4 and the total energy
  within 1e-6 relative (oracle pairs from a periodic k-d tree);
* the caller's Dense list returned by the run, in the reference's entry
  order, on a seeded sample of 2,000 atoms (pairs within 1e-6 of the list
  cutoff compared as sets), and the run's occupancy and error bits;
* the same run with the tiled int32 list, and the energy drift.

The k-d tree only finds the pairs; distances, the potential and the sums are
the oracle's (oracle/md_oracle.py).
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import LJ_DT, fcc_system, lj_spec

pytestmark = pytest.mark.gpu

N_CELLS = 60          # 864,000 atoms
STEPS = 30


@pytest.fixture(scope='module')
def lj864k(cuda):
    from jax_md_gb300 import energy, partition, simulate, space
    R, P, L = fcc_system(N_CELLS)
    disp, shift = space.periodic(L)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, dr_threshold=0.3, format=partition.Dense)
    out = {}
    for layout in ('segment', 'half', 'tiled'):
        Rt = torch.tensor(R, device=cuda)
        nb = nfn.allocate(Rt)
        init, apply = simulate.nve(efn, shift, LJ_DT)
        st = init(0, Rt, momenta=torch.tensor(P, device=cuda), neighbor=nb)
        E0 = float(efn.energy_f64(st.position, nb)) + float(simulate.kinetic_energy(st))
        simulate.run(apply, st, nb, STEPS, layout=layout)
        torch.cuda.synchronize()
        out[layout] = (st, nb, E0, simulate.last_run_status(st))
    return R, L, efn, out


def _oracle_pairs(X, L, r):
    spatial = pytest.importorskip('scipy.spatial')
    tree = spatial.cKDTree(np.mod(X, L), boxsize=L)
    pairs = tree.query_pairs(r, output_type='ndarray')
    return tree, pairs


@pytest.mark.parametrize('layout', ['segment', 'half'])
def test_forces_and_energy_match_oracle(lj864k, layout):
    R, L, efn, out = lj864k
    st, nb, _, status = out[layout]
    assert status == 0
    X = st.position[:, :3].double().cpu().numpy()
    _, pairs = _oracle_pairs(X, L, 2.5)
    # OrderedSparse-style (receiver, sender) pairs with i > j: each pair once
    idx = np.stack([pairs.min(1), pairs.max(1)])
    Eo, Fo, _ = O.pair_energy_forces(lj_spec(), X, idx, O.ORDERED_SPARSE, np.full(3, L))
    F = st.force[:, :3].double().cpu().numpy()
    err = np.abs(F - Fo).max()
    assert err < 1e-4, err
    E = float(efn.energy_f64(st.position, nb))
    assert abs(E - Eo) <= 1e-6 * abs(Eo), (E, Eo)


def test_returned_list_matches_oracle_rows(lj864k):
    R, L, efn, out = lj864k
    st, nb, _, _ = out['segment']
    n = R.shape[0]
    ref = nb.reference_position[:, :3].contiguous().cpu().numpy()
    box = np.full(3, L, np.float32)
    onl = O.NeighborListOracle(box, np.float32(2.5), np.float32(0.3))
    atoms = np.sort(np.random.default_rng(11).choice(n, 2000, replace=False))
    want, counts = onl.dense_rows(ref, atoms, nb.cell_list_capacity)
    got = nb.idx.cpu().numpy()[atoms]
    cut = float(np.float32(2.8))
    tree, _ = _oracle_pairs(ref.astype(np.float64), L, cut)
    bad = []
    for k, i in enumerate(atoms):
        near = set()
        for j in tree.query_ball_point(ref[i].astype(np.float64), cut + 1e-5):
            d = O.displacement(ref[i].astype(np.float64), ref[j].astype(np.float64), np.full(3, L))
            if abs(np.sqrt((d * d).sum()) - cut) < 1e-6:
                near.add(int(j))
        g, w = got[k], want[k][:got.shape[1]]
        if near & set(int(j) for j in np.concatenate([g, w]) if j < n):
            gs = sorted(int(j) for j in g if j < n and int(j) not in near)
            ws = sorted(int(j) for j in w if j < n and int(j) not in near)
            if gs != ws:
                bad.append(int(i))
        elif not np.array_equal(g, w):
            bad.append(int(i))
    assert bad == []
    assert int(counts.max()) <= nb.max_occupancy
    assert int(nb.error.code) == 0


@pytest.mark.parametrize('layout', ['segment', 'half'])
def test_layouts_agree_and_energy_is_conserved(lj864k, layout):
    """The segment (full or half lists) and tiled runs agree to fp32 rounding
    over the run; the segment run conserves energy."""
    from jax_md_gb300 import simulate
    R, L, efn, out = lj864k
    (sa, na, E0, _), (sb, nbb, _, _) = out[layout], out['tiled']
    d = O.displacement(sa.position[:, :3].cpu().numpy(), sb.position[:, :3].cpu().numpy(),
                       np.full(3, L))
    assert np.abs(d).max() < 1e-4
    E1 = float(efn.energy_f64(sa.position, na)) + float(simulate.kinetic_energy(sa))
    assert abs(E1 - E0) / R.shape[0] < 1e-3, (E0, E1)
