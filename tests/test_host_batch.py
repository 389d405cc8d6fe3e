"""Host-side logic of the batched form and the adjoint (no GPU): packing,
per-system cell grids (partition.py:146-188 per system), argument checks."""
import numpy as np
import pytest
import torch

from jax_md_gb300 import batch


def _pos(n, dim, L, seed):
    return torch.tensor(np.random.default_rng(seed).uniform(0, L, (n, dim)), dtype=torch.float32)


def test_pack_offsets_species_and_wrap():
    Rs = [_pos(5, 2, 10.0, 0), _pos(3, 2, 7.0, 1) + 7.0, _pos(4, 2, 12.0, 2)]
    sp = [np.zeros(5), np.ones(3), np.zeros(4)]
    bt = batch.pack(Rs, [10.0, 7.0, [12.0, 12.0]], species=sp, device='cpu')
    assert bt.n == 12 and bt.n_systems == 3 and bt.sizes == [5, 3, 4]
    assert bt.offsets.tolist() == [0, 5, 8, 12]
    assert bt.sys_offset.tolist() == [0, 5, 8, 12]
    assert bt.atom_sys.tolist() == [0] * 5 + [1] * 3 + [2] * 4
    assert bt.species.tolist() == [0] * 5 + [1] * 3 + [0] * 4
    # positions are wrapped into each system's own box, float4 rows
    assert bt.position.shape == (12, 4)
    assert float(bt.R[5:8].max()) < 7.0 and float(bt.R[5:8].min()) >= 0.0
    assert torch.equal(bt.position[:, 2:], torch.zeros(12, 2))
    assert [t.shape[0] for t in bt.split(bt.R)] == [5, 3, 4]


def test_pack_rejects_bad_input():
    with pytest.raises(ValueError):
        batch.pack([], [], device='cpu')
    with pytest.raises(ValueError):
        batch.pack([_pos(3, 2, 5.0, 0), _pos(3, 3, 5.0, 1)], [5.0, 5.0], device='cpu')
    with pytest.raises(ValueError):
        batch.pack([_pos(3, 2, 5.0, 0)], [-1.0], device='cpu')
    with pytest.raises(ValueError):
        batch.pack([_pos(3, 2, 5.0, 0)], [5.0], species=[np.zeros(2)], device='cpu')


def test_cell_grids_per_system():
    """cells_per_side = floor(L / cutoff) per system and axis (at least 1),
    cell_size = L / cells_per_side in float32, global cell offsets."""
    Rs = [_pos(10, 3, 20.0, 0), _pos(10, 3, 5.0, 1), _pos(10, 3, 8.5, 2)]
    bt = batch.pack(Rs, [20.0, 5.0, 8.5], device='cpu')
    g = batch._Grid(bt, 2.8)
    assert g.cps[:, 0].tolist() == [7, 1, 3]
    assert g.cps[:, :3].prod(1).tolist() == [343, 1, 27]
    assert g.cell_offset.tolist() == [0, 343, 344, 371]
    assert g.total_cells == 371 and g.max_cells == 343
    assert np.allclose(g.cs[:, 0].numpy(), np.float32([20.0 / 7, 5.0, 8.5 / 3]))
    assert g.struct.n_systems == 3 and g.struct.n_atoms == 30 and g.struct.dim == 3


def test_cell_grid_limit():
    bt = batch.pack([_pos(10, 3, 100.0, 0)], [100.0], device='cpu')
    with pytest.raises(ValueError, match='24576 cells'):
        batch._Grid(bt, 2.8)   # 35^3 = 42875 cells


def test_neighbor_list_constants_match_single_system():
    """The batched list keeps partition.neighbor_list's float32 cutoff and
    skin arithmetic (partition.py:880-884, 1146-1154)."""
    fns = batch.neighbor_list(2.5, 0.3)
    assert fns.cutoff == float(np.float32(np.float32(2.5) + np.float32(0.3)))
    assert fns.threshold_sq == float(np.float32((np.float32(0.3) / np.float32(2)) ** 2))
    assert batch.neighbor_list(2.5, 0.0).threshold_sq < 0   # rebuild every step


def test_trajectory_segments():
    """Checkpoint segments of the adjoint cover the run exactly."""
    from jax_md_gb300 import adjoint, energy, partition, space
    disp, shift = space.periodic(10.0)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, 10.0, format=partition.Dense)
    tr = adjoint.nve_trajectory(efn, nfn, shift, 0.005, 23, checkpoint_every=5)
    buf_segments = [(s0, min(s0 + 5, 23)) for s0 in range(0, 23, 5)]
    assert tr.segment_length(100) == 5
    assert buf_segments[-1] == (20, 23) and sum(b - a for a, b in buf_segments) == 23
    with pytest.raises(ValueError):
        adjoint.nve_trajectory(efn, nfn, shift, 0.005, 0)


def test_chain_init_matches_oracle():
    """Per-system Nose-Hoover chains of a batch: the layout of
    jmd_nhc_half_step (xi[16] p[16] Q[16] spare[16] KE kT) holding each
    system's own simulate.py:436-442 initial chain (dof = n_b * dim)."""
    from oracle import md_oracle as O
    Rs = [_pos(5, 3, 10.0, 0), _pos(3, 3, 7.0, 1), _pos(8, 3, 12.0, 2)]
    bt = batch.pack(Rs, [10.0, 7.0, 12.0], device='cpu')
    c = batch._nhc_constants(0.005, 4, 2, 3, None)
    assert c.tau == float(np.float32(np.float32(0.005) * 100))
    ke = torch.tensor([1.5, 2.0, 0.25], dtype=torch.float64)
    kT = [0.6, 0.7, 0.8]
    chain = batch._chain_init(bt, ke, torch.tensor(kT, dtype=torch.float64), c).numpy()
    assert chain.shape == (3, 66)
    for b, n in enumerate(bt.sizes):
        ref = O.nhc_init(3 * n, float(ke[b]), kT[b], c.tau, 4)
        assert np.allclose(chain[b, 32:36], ref.Q)
        assert np.all(chain[b, 36:48] == 0) and np.all(chain[b, :32] == 0)
        assert chain[b, 64] == float(ke[b]) and chain[b, 65] == kT[b]
    # a scalar kT is shared by every system
    same = batch._chain_init(bt, ke, 0.5, c).numpy()
    assert np.all(same[:, 65] == 0.5)


def test_nose_hoover_argument_checks():
    with pytest.raises(ValueError):
        batch._nhc_constants(0.005, 1, 2, 3, None)
    with pytest.raises(ValueError):
        batch._nhc_constants(0.005, 5, 2, 4, None)
    with pytest.raises(ValueError):
        batch._nhc_constants(0.005, 5, 0, 3, None)
    bt = batch.pack([_pos(4, 3, 10.0, 0)], [10.0], device='cpu')
    with pytest.raises(NotImplementedError):
        batch.BatchNvtTrajectory(bt, None, None, None, 0.005, 1.0, 10, chain_length=8)
    with pytest.raises(ValueError):
        batch.BatchNvtTrajectory(bt, None, None, None, 0.005, 1.0, 0)
