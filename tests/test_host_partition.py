"""Host-side logic of partition (no GPU): the float32 cell grid
(partition.py:146-188) against the oracle's, the sticky PartitionError bits
and messages (partition.py:494-561), format predicates, Dense row strides and
box parsing."""
import numpy as np
import pytest
import torch

from jax_md_gb300 import partition
from oracle import md_oracle as O


@pytest.mark.parametrize('box,cut,dim', [(10.0, 2.8, 3), ([9.0, 4.0, 7.25], 0.615, 3),
                                         ([8.65, 8.0], 1.0, 2), (100.776, 2.8, 3),
                                         (16.796, 2.8, 3)])
def test_cell_dimensions_match_oracle(box, cut, dim):
    cps, cs, count = partition.cell_dimensions(dim, box, cut)
    ref = O.cell_dimensions(np.broadcast_to(np.asarray(box, np.float64), (dim,)), cut, dim)
    ref_cps, ref_cs = np.asarray(ref[0]).reshape(-1)[:dim], np.asarray(ref[1]).reshape(-1)[:dim]
    assert cps.tolist() == [int(v) for v in ref_cps]
    np.testing.assert_array_equal(cs, ref_cs.astype(np.float32))
    assert count == int(np.prod(cps))


def test_benchmark_grid():
    """The LJ benchmark's grid: 35 cells of 2.879 per side at N = 864,000."""
    cps, cs, count = partition.cell_dimensions(3, 100.776, np.float32(2.5) + np.float32(0.3))
    assert cps.tolist() == [35, 35, 35] and count == 42875
    assert abs(float(cs[0]) - 2.879) < 1e-3


def test_partition_error_bits_are_sticky():
    e = partition.PartitionError(torch.zeros((), dtype=torch.uint8))
    assert str(e) == ''
    e = e.update(partition.PEC.CELL_SIZE_TOO_SMALL, True)
    e = e.update(partition.PEC.NEIGHBOR_LIST_OVERFLOW, False)
    assert int(e.code) == 4 and 'Cell size too small' in str(e)
    e = e.update(partition.PEC.NEIGHBOR_LIST_OVERFLOW, True)
    assert int(e.code) == 5 and 'Neighbor list buffer overflow' in str(e)
    e = e.update(partition.PEC.NEIGHBOR_LIST_OVERFLOW, False)
    assert int(e.code) == 5
    assert [int(b) for b in partition.PEC] == [0, 1, 2, 4, 8]


def test_formats_row_stride_and_boxes():
    assert partition.is_sparse(partition.Sparse) and partition.is_sparse(partition.OrderedSparse)
    assert not partition.is_sparse(partition.Dense)
    for w, ld in ((1, 8), (8, 8), (9, 16), (98, 104)):
        assert partition._row_ld(w) == ld
    assert partition._box_list(5.0, 3) == [5.0] * 3
    assert partition._box_list(np.diag([3.0, 4.0]), 2) == [3.0, 4.0]
    assert partition._box_list(torch.tensor([2.0, 3.0, 4.0]), 3) == [2.0, 3.0, 4.0]
    with pytest.raises(NotImplementedError, match='periodic_general'):
        partition._box_list(np.array([[3.0, 0.5], [0.0, 4.0]]), 2)


def _nl(cps, cap, dim=3):
    from jax_md_gb300 import _native as N
    nl = N.NList()
    nl.space.dim = dim
    nl.use_cell_list = 1
    for d in range(dim):
        nl.cells_per_side[d] = cps
        nl.cell_size[d] = 2.9
    nl.cell_capacity = cap
    nl.format = N.DENSE
    nl.max_occupancy = 100
    return nl


@pytest.mark.parametrize('cps,cap,K,dim,want', [
    (35, 40, 5, 3, (8575, 2520, 5)),     # the LJ benchmark grid: 7 segments per row
    (12, 40, 5, 3, (432, 2520, 5)),      # 5 + 5 + 2 cells per row
    (5, 52, 5, 3, (50, 2340, 3)),        # K clipped to cells - 2
    (3, 46, 5, 3, (27, 1242, 1)),
    (12, 10, 8, 2, (24, 300, 8)),        # 2D: 3 staged rows
])
def test_segment_plan(cps, cap, K, dim, want):
    """jmd_segment_plan (host arithmetic, no device needed): segments =
    ceil(cells_x / K) x cells_y (x cells_z), capacity 3^(d-1) (K + 2) x cell
    capacity atoms of 16 bytes, K at most cells_x - 2."""
    from jax_md_gb300 import simulate
    plan = simulate.segment_plan(_nl(cps, cap, dim), K)
    assert plan is not None
    nseg, capa, smem, used, list_bytes = plan
    assert (nseg, capa, used) == want
    assert smem == (capa + 1) * 16   # + the far slot
    # list buffer: the chunk-count table, a 256-byte staging record per
    # segment, one block per segment (header, 16-bit counts, chunks of 8
    # slots for K x cell capacity own atoms)
    P = (used * cap + 7) // 8 * 8
    nch = 13
    assert list_bytes == ((4 * nseg + 15) // 16 * 16 + nseg * 256
                          + nseg * (16 + 2 * P + nch * P * 16))


@pytest.mark.parametrize('cps,cap,K', [(2, 40, 5), (35, 40, 0), (35, 40, 15), (35, 800, 5)])
def test_segment_plan_rejects(cps, cap, K):
    """Fewer than 3 cells per side, K outside 1..14, or a staging block beyond
    a CTA's shared memory: the segment layout does not apply."""
    from jax_md_gb300 import simulate
    assert simulate.segment_plan(_nl(cps, cap), K) is None


def test_segment_threads_default():
    from jax_md_gb300 import simulate
    assert simulate.segment_threads_default(5, 40) == 160
    assert simulate.segment_threads_default(1, 46) == 64
    assert simulate.segment_threads_default(14, 60) == 256


def test_segment_autotuner_candidates_and_cache_keys():
    """The autotuner's candidates on the benchmark's grid: every admitted K
    with full lists (staged or global), half lists (also at 256 threads),
    and the tiled list; a tiled choice survives the cache's JSON round trip
    as a name, a segment choice as a tuple."""
    import json
    from jax_md_gb300 import tune
    cands = tune.segment_candidates(_nl(35, 40, 3))
    assert 'tiled' in cands
    shapes = [c for c in cands if c != 'tiled']
    assert {c[0] for c in shapes} == {2, 3, 4, 5, 6, 8}
    assert (5, 160, 1, 0) in shapes and (5, 160, 0, 0) in shapes and (5, 160, 0, 1) in shapes
    assert (5, 256, 0, 1) in shapes
    assert all(64 <= c[1] <= 256 and c[1] % 32 == 0 for c in shapes)
    for c in ('tiled', (5, 160, 0, 1)):
        k = json.dumps(c if isinstance(c, str) else list(c))
        assert tune._unkey(json.loads(k)) == c
