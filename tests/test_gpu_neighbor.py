"""Neighbour and cell lists on the GPU against the FP64 oracle.

Dense lists must be identical to the oracle's (which restates the reference's
candidate order), entry order included; pairs whose f64 distance lies within
1e-6 of the list cutoff are excluded from the strict comparison and checked
separately (their decision may flip between fp32 and fp64).
"""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O
from tests.helpers import fcc_system, near_cutoff_pairs, random_box

pytestmark = pytest.mark.gpu

FMT = {0: 'Dense', 1: 'Sparse', 2: 'OrderedSparse'}


def _gpu_list(R, box, r_cut, skin, fmt, cuda, **kw):
    from jax_md_gb300 import partition, space
    disp, _ = space.periodic(box.tolist() if hasattr(box, 'tolist') else box)
    f = getattr(partition, FMT[fmt])
    fns = partition.neighbor_list(disp, box.tolist() if hasattr(box, 'tolist') else box, r_cut,
                                  skin, format=f, **kw)
    Rt = torch.tensor(R, device=cuda)
    return fns, fns.allocate(Rt), Rt


def _strict_equal_rows(got, want, N, skip_pairs):
    """Compares Dense rows entry by entry unless a row touches a near-cutoff pair."""
    bad = []
    for i in range(N):
        g = got[i]
        w = want[i]
        touched = any((i, int(j)) in skip_pairs for j in np.concatenate([g, w]) if j < N)
        if touched:
            gs = sorted(int(j) for j in g if j < N and (i, int(j)) not in skip_pairs)
            ws = sorted(int(j) for j in w if j < N and (i, int(j)) not in skip_pairs)
            if gs != ws:
                bad.append(i)
        elif not np.array_equal(g, w):
            bad.append(i)
    return bad


@pytest.mark.parametrize('dim', [2, 3])
@pytest.mark.parametrize('fmt', [0, 1, 2])
def test_random_box_matches_oracle(cuda, dim, fmt):
    box = np.array([9.0, 3.25] if dim == 2 else [9.0, 4.0, 7.25], np.float32)
    R = random_box(1000, dim, box, seed=dim)
    r_cut, skin = 0.55, 0.06
    fns, nb, Rt = _gpu_list(R, box, r_cut, skin, fmt, cuda)
    onl = O.NeighborListOracle(box, np.float32(r_cut), np.float32(skin), fmt=fmt)
    onb = onl.allocate(R)
    skip = near_cutoff_pairs(R, box, float(np.float32(np.float32(r_cut) + np.float32(skin))))
    assert nb.idx.shape == onb.idx.shape or skip
    assert int(nb.error.code) == onb.error
    got = nb.idx.cpu().numpy()
    if fmt == 0:
        assert _strict_equal_rows(got, onb.idx, len(R), skip) == []
    else:
        if not skip:
            np.testing.assert_array_equal(got, onb.idx)
        gs = O.neighbor_sets(O.NeighborListO(got, R, 0, None, 0, fmt, True), len(R))
        ws = O.neighbor_sets(onb, len(R))
        for i in range(len(R)):
            a = [j for j in gs[i] if (i, j) not in skip]
            b = [j for j in ws[i] if (i, j) not in skip]
            assert a == b


def test_lj_fluid_dense_bit_exact(cuda):
    """The plain LJ workload at N=4000: Dense idx identical to the oracle's, order included."""
    R, P, L = fcc_system(10)
    box = np.full(3, L, np.float32)
    fns, nb, Rt = _gpu_list(R, box, 2.5, 0.3, 0, cuda)
    onl = O.NeighborListOracle(box, np.float32(2.5), np.float32(0.3), fmt=O.DENSE)
    onb = onl.allocate(R)
    skip = near_cutoff_pairs(R, box, float(np.float32(2.8)))
    assert nb.max_occupancy == onb.max_occupancy
    assert nb.cell_list_capacity == onb.cell_list_capacity
    got = nb.idx.cpu().numpy()
    assert _strict_equal_rows(got, onb.idx, len(R), skip) == []
    cnt = nb.nbr_count.cpu().numpy()
    np.testing.assert_array_equal(cnt, (onb.idx < len(R)).sum(1))


def test_update_skin_semantics(cuda):
    """Small moves keep the list; a move beyond skin/2 rebuilds (partition.py:1146-1154)."""
    R, P, L = fcc_system(6)
    box = np.full(3, L, np.float32)
    fns, nb, Rt = _gpu_list(R, box, 2.5, 0.3, 0, cuda)
    before = nb.idx.clone()
    ref_before = nb.reference_position.clone()
    R2 = Rt.clone()
    R2[:, 0] = torch.remainder(R2[:, 0] + 0.1, float(L))      # 0.1 < 0.15: no rebuild
    nb2 = fns.update(R2, nb)
    torch.cuda.synchronize()
    assert torch.equal(nb2.idx, before)
    assert torch.equal(nb2.reference_position, ref_before)
    R3 = Rt.clone()
    R3[7] = torch.remainder(R3[7] + 1.0, float(L))             # one atom moves 1.0: rebuild
    nb3 = fns.update(R3, nb2)
    onl = O.NeighborListOracle(box, np.float32(2.5), np.float32(0.3))
    ob = onl.build(R3.cpu().numpy(), nb.max_occupancy, 0, nb.cell_list_capacity)
    skip = near_cutoff_pairs(R3.cpu().numpy(), box, float(np.float32(2.8)))
    assert _strict_equal_rows(nb3.idx.cpu().numpy(), ob.idx, len(R), skip) == []
    assert torch.equal(nb3.reference_position, R3)


@pytest.mark.parametrize('r_cut,dc,cm', [(0.12, True, 1.5), (0.25, False, 1.5),
                                         (0.31, False, 1.5), (0.31, False, 1.0)])
@pytest.mark.parametrize('mask_self', [False, True])
@pytest.mark.parametrize('fmt', [0, 1, 2])
def test_capacity_shapes(cuda, r_cut, dc, cm, mask_self, fmt):
    """tests/partition_test.py:489-546 on the GPU."""
    if fmt == 0:
        want = (20, 19) if mask_self else (20, 20)
    elif fmt == 1:
        want = (2, 380) if mask_self else (2, 400)
    else:
        want = (2, 190)
    R = np.full((20, 3), 0.5, np.float32)
    fns, nb, Rt = _gpu_list(R, np.ones(3, np.float32), r_cut, 0.1 * r_cut, fmt, cuda,
                            capacity_multiplier=cm, disable_cell_list=dc, mask_self=mask_self)
    assert not bool(nb.did_buffer_overflow)
    assert tuple(nb.idx.shape) == want
    nb2 = fns.update(Rt + 0.1, nb)
    assert not bool(nb2.did_buffer_overflow)
    assert tuple(nb2.idx.shape) == want


def test_overflow_is_sticky(cuda):
    """tests/partition_test.py:363-401 (free space, collapse) and stickiness."""
    from jax_md_gb300 import partition, space
    disp, _ = space.free()
    fns = partition.neighbor_list(disp, 100.0, 3.0, 0.0)
    R = torch.tensor([[20.0, 20.0], [30.0, 30.0], [40.0, 40.0], [50.0, 50.0]], device=cuda)
    nb = fns.allocate(R)
    assert not bool(nb.did_buffer_overflow)
    assert nb.idx.dtype == torch.int32
    R2 = R.clone()
    R2[1] = R2[0]
    nb = fns.update(R2, nb)
    assert bool(nb.did_buffer_overflow)
    nb = fns.update(R, nb)
    assert bool(nb.did_buffer_overflow)      # sticky


def test_cell_list_buffers_match_oracle(cuda):
    from jax_md_gb300 import partition
    box = np.array([8.65, 8.0], np.float32)
    R = np.array([[0.25, 0.25], [8.5, 1.95], [8.1, 1.5], [3.7, 7.9]], np.float32)
    cl = partition.cell_list(box, 1.0).allocate(torch.tensor(R, device=cuda))
    assert cl.id_buffer.dtype == torch.int32
    ids = cl.id_buffer[..., 0].cpu().numpy()
    assert ids[0, 0, 0] == 0 and ids[1, 7, 1] == 1 and ids[1, 7, 0] == 2 and ids[7, 3, 1] == 3
    pos = cl.position_buffer.cpu().numpy()
    np.testing.assert_array_equal(pos[1, 7, 1], R[1])
    rng = np.random.default_rng(1)
    for dim, bx in ((2, [9.0, 3.25]), (3, [9.0, 3.0, 7.25])):
        bx = np.array(bx, np.float32)
        R = (rng.uniform(size=(1000, dim)) * bx).astype(np.float32)
        cl = partition.cell_list(bx, 1.0).allocate(torch.tensor(R, device=cuda))
        cap = O.estimate_cell_capacity(R, bx, 1.0, 1.25, dim)
        ocl = O.cell_list(R, bx, 1.0, cap)
        assert cl.cell_capacity == cap
        np.testing.assert_array_equal(cl.id_buffer.reshape(-1).cpu().numpy(),
                                      ocl.id_buffer.reshape(-1))
        np.testing.assert_array_equal(cl.particle_cell_id.cpu().numpy(), ocl.particle_cell_id)
        # emplace round trip (partition_test.py:102-128)
        idf = cl.id_buffer.reshape(-1).long().cpu()
        pf = cl.position_buffer.reshape(-1, dim).cpu()
        out = torch.zeros(1001, dim)
        out[idf] = pf
        np.testing.assert_array_equal(out[:-1].numpy(), R)


def test_crowded_cells_exceed_shared_stage(cuda):
    """~110 atoms per cell: each cell's candidate stream (>2048) is read from global memory."""
    box = np.full(3, 9.0, np.float32)
    R = random_box(3000, 3, box, seed=11)
    fns, nb, Rt = _gpu_list(R, box, 2.9, 0.05, 0, cuda)
    onl = O.NeighborListOracle(box, np.float32(2.9), np.float32(0.05), fmt=O.DENSE)
    onb = onl.allocate(R)
    assert onb.use_cell_list and nb.cell_list_capacity == onb.cell_list_capacity
    skip = near_cutoff_pairs(R, box, float(np.float32(np.float32(2.9) + np.float32(0.05))))
    assert _strict_equal_rows(nb.idx.cpu().numpy(), onb.idx, len(R), skip) == []
