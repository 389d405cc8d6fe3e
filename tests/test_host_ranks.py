"""Ensembles split across ranks (CPU, gloo): the batched forms' independent
systems are partitioned over processes with no exchange during the run, and
the ensemble mean and its shared-parameter gradients are combined by one
all-reduce.  World size 2 runs as two spawned processes on 127.0.0.1."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from jax_md_gb300 import batch


def _sizes(n=128, seed=0):
    rng = np.random.default_rng(seed)
    return [int(round(rng.uniform(500, 20000) ** (1 / 3))) ** 3 for _ in range(n)]


@pytest.mark.parametrize('ranks', [1, 2, 3, 8])
def test_partition_systems_covers_and_balances(ranks):
    sizes = _sizes()
    parts = batch.partition_systems(sizes, ranks)
    assert len(parts) == ranks
    flat = sorted(b for p in parts for b in p)
    assert flat == list(range(len(sizes)))
    assert all(p == sorted(p) for p in parts)
    loads = [sum(sizes[b] for b in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)
    assert parts == batch.partition_systems(sizes, ranks)   # same split on every rank


def test_partition_systems_edge_cases():
    assert batch.partition_systems([], 2) == [[], []]
    assert batch.partition_systems([7], 3) == [[0], [], []]
    with pytest.raises(ValueError):
        batch.partition_systems([1, 2], 0)
    with pytest.raises(ValueError):
        batch.partition_systems([1, -2], 2)


def _per_system(b):
    """A stand-in per-system loss and its gradient wrt 3 shared parameters."""
    return float(np.sin(b) + b * 0.01), np.array([np.cos(b), b * 1e-3, 1.0])


def test_reduce_ensemble_single_process():
    vals = [_per_system(b) for b in range(10)]
    s = torch.tensor(sum(v for v, g in vals), dtype=torch.float64)
    g = torch.tensor(sum(g for v, g in vals), dtype=torch.float32)
    mean, (gm,) = batch.reduce_ensemble(s, 10, [g])
    assert abs(float(mean) - np.mean([v for v, _ in vals])) < 1e-12
    assert gm.dtype == torch.float32
    assert np.allclose(gm.numpy(), np.mean([g for _, g in vals], axis=0))
    with pytest.raises(ValueError):
        batch.reduce_ensemble(torch.tensor(0.0), 0)


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, out_dir):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        mine = batch.partition_systems(sizes, world)[rank]
        s = torch.tensor(sum(_per_system(b)[0] for b in mine), dtype=torch.float64)
        g = torch.tensor(sum((_per_system(b)[1] for b in mine), np.zeros(3)),
                         dtype=torch.float64)
        mean, (gm,) = batch.reduce_ensemble(s, len(mine), [g])
        np.save(os.path.join(out_dir, f'r{rank}.npy'),
                np.concatenate([[float(mean)], gm.numpy(), [len(mine)]]))
    finally:
        dist.destroy_process_group()


def test_reduce_ensemble_two_ranks_gloo(tmp_path):
    sizes = _sizes(37, seed=3)
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), sizes, str(tmp_path)), nprocs=world, join=True)
    res = [np.load(tmp_path / f'r{r}.npy') for r in range(world)]
    ref_v = np.mean([_per_system(b)[0] for b in range(len(sizes))])
    ref_g = np.mean([_per_system(b)[1] for b in range(len(sizes))], axis=0)
    for r in res:
        assert abs(r[0] - ref_v) < 1e-12
        assert np.allclose(r[1:4], ref_g, rtol=0, atol=1e-12)
    assert res[0][4] + res[1][4] == len(sizes) and res[0][4] > 0 and res[1][4] > 0
