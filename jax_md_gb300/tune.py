"""Launch-shape autotuners.

autotune_segment: the device engine's segment-local list (simulate.run with a
cell-sorted state): cells per segment K and threads per segment CTA, timed as
whole engine runs (rebuilds included) on a copy of the caller's own state;
the choice is recorded for the cell grid (simulate.run picks it up) and cached
on disk keyed by (device name, grid, cell capacity, potential, species).

autotune_dense: threads per atom (4, 8, 16) of the row-major Dense fused
step kernel (the caller's-list path, jmd_nve_fused_step), read by the kernels
from a library-wide setting (jmd_set_dense_threads_per_atom).
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


def _seg_key(nl, pair) -> str:
    dev = torch.cuda.get_device_name()
    d = nl.space.dim
    cps = 'x'.join(str(c) for c in nl.cells_per_side[:d])
    return f'seg|{dev}|c{cps}|cap{nl.cell_capacity}|k{pair.kind}|s{pair.n_species}'


def segment_candidates(nl):
    """(cells, threads, stage_lists, half) to try: K in 2..8 (those the
    grid admits) with the default thread count and the neighbouring multiples
    of 32, each with full lists (block staged in shared memory or read from
    global memory) or half lists (Newton's third law); and 'tiled', the
    engine's tiled int32 list."""
    from . import simulate
    out = []
    for K in (2, 3, 4, 5, 6, 8):
        plan = simulate.segment_plan(nl, K)
        if plan is None or plan[3] != K:
            continue
        t0 = simulate.segment_threads_default(K, nl.cell_capacity)
        for t in sorted({t0 - 32, t0, t0 + 32}):
            if 64 <= t <= 256:
                out.append((K, t, 1, 0))
                out.append((K, t, 0, 0))
                out.append((K, t, 0, 1))   # half lists (Newton's third law)
        # the half-list kernel spreads list chunks over the threads, so it
        # can use more threads than a segment has atoms
        if t0 + 32 < 256:
            out.append((K, 256, 0, 1))
    out.append('tiled')   # the tiled int32 list, thread per atom
    return out


def _unkey(k):
    return k if isinstance(k, str) else tuple(k)


def autotune_segment(apply_fn, state, neighbor, steps: int = 20, reps: int = 2,
                     use_cache: bool = True, candidates=None):
    """Picks (cells per segment, threads per CTA) for simulate.run on this
    system by timing `steps`-step engine runs (CUDA graph, rebuilds included)
    from copies of `state`; records the choice for the cell grid and returns
    ((cells, threads), {choice: ms per step}).  Returns (None, {}) when the
    segment layout does not apply."""
    from . import simulate
    nl = neighbor.plan.nl
    species, pair = apply_fn.stepper.energy_fn._resolve(state.position, {})
    key = _seg_key(nl, pair)
    gk = simulate._grid_key(nl)
    cache = _load() if use_cache else {}
    if key in cache:
        c = cache[key]['choice']
        choice = c if isinstance(c, str) else tuple(c)
        simulate._segment_choice[gk] = choice
        return choice, {_unkey(json.loads(k)): v for k, v in cache[key]['ms'].items()}
    cands = list(candidates) if candidates is not None else segment_candidates(nl)
    if not cands:
        return None, {}
    timings = {}
    for c in cands:
        st = state.copy()
        simulate.run(apply_fn, st, neighbor, steps, layout=c)   # captures the graph
        best = float('inf')
        for _ in range(reps):
            st = state.copy()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            simulate.run(apply_fn, st, neighbor, steps, layout=c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / steps)
        timings[c] = best
        del st
    choice = min(timings, key=timings.get)
    simulate._segment_choice[gk] = choice
    if use_cache:
        cache[key] = {'choice': choice if isinstance(choice, str) else list(choice),
                      'ms': {json.dumps(k if isinstance(k, str) else list(k)): v
                             for k, v in timings.items()}}
        _save(cache)
    return choice, timings
