"""Launch-shape autotuner for the Dense pair kernels.

Times the fused NVE step kernel for each threads-per-atom choice (4, 8, 16) on
the caller's own system, keeps the fastest, and caches the choice on disk keyed
by (device name, atom-count bucket, row width, dimension, potential, species).
The kernels read the choice from a library-wide setting
(jmd_set_dense_threads_per_atom).
"""
from __future__ import annotations

import ctypes
import json
import math
import os
from pathlib import Path

import torch

from . import _native as N

CACHE = Path(os.environ.get('JAX_MD_GB300_TUNE_CACHE',
                            Path.home() / '.cache' / 'jax_md_gb300' / 'tune.json'))
CHOICES = (4, 8, 16)


def _key(n, width, dim, pair) -> str:
    dev = torch.cuda.get_device_name()
    bucket = 2 ** int(math.log2(max(n, 1)))
    return f'{dev}|n~{bucket}|w{width}|d{dim}|k{pair.kind}|s{pair.n_species}'


def _load():
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def _save(d):
    try:
        CACHE.parent.mkdir(parents=True, exist_ok=True)
        CACHE.write_text(json.dumps(d, indent=1, sort_keys=True))
    except OSError:
        pass


def set_threads_per_atom(tpa: int):
    N.check(N.lib().jmd_set_dense_threads_per_atom(int(tpa)), 'set threads per atom')


def autotune_dense(energy_fn, state, neighbor, shift_fn, dt, reps: int = 20, use_cache=True):
    """Picks threads-per-atom for the fused step of this system; returns (tpa, timings ms)."""
    from . import simulate
    R = state.position
    n, dim = R.shape
    species, pair = energy_fn._resolve(R, {})
    key = _key(n, neighbor.max_occupancy, dim, pair)
    cache = _load() if use_cache else {}
    if key in cache:
        set_threads_per_atom(cache[key]['tpa'])
        return cache[key]['tpa'], cache[key]['ms']
    sp = simulate._shift_space(shift_fn, dim)
    xb = torch.empty((n, 4), dtype=torch.float32, device=R.device)
    pm = state.momentum.clone()
    flag = torch.zeros((), dtype=torch.int32, device=R.device)
    L = N.lib()
    plan = neighbor.plan

    def launch():
        N.check(L.jmd_nve_fused_step(ctypes.byref(pair), ctypes.byref(sp), R.data_ptr(),
                                     xb.data_ptr(), pm.data_ptr(), None, 1.0, N.ptr(species), n,
                                     neighbor.idx.data_ptr(), plan.ld, neighbor.max_occupancy,
                                     plan.count.data_ptr(), float(dt),
                                     neighbor.reference_position.data_ptr(), plan.threshold_sq,
                                     flag.data_ptr(), N.stream_ptr()), 'fused step')
    timings = {}
    for tpa in CHOICES:
        set_threads_per_atom(tpa)
        for _ in range(3):
            launch()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            launch()
        e1.record()
        torch.cuda.synchronize()
        timings[tpa] = e0.elapsed_time(e1) / reps
    best = min(timings, key=timings.get)
    set_threads_per_atom(best)
    if use_cache:
        cache[key] = {'tpa': best, 'ms': timings}
        _save(cache)
    return best, timings
