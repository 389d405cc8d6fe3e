"""Benchmark: LJ fluid, N = 864,000 (FCC 60^3 x 4), NVE, fp32, Dense neighbour list.

One step = the reference's loop body (jax_md/partition.py:841-854):
    nbrs = nbrs.update(state.position); state = apply_fn(state, neighbor=nbrs)
i.e. the device-side skin test, the (conditional) cell-list + neighbour rebuild,
the velocity-Verlet step with the LJ pair-force kernel.

  value : atom-steps/s, state resident in HBM, steps replayed from a CUDA graph;
  e2e   : the same through the public API with host (pinned) buffers: every
          step copies positions and momenta host->device, runs the step, and
          copies them back device->host;
  roofline: the pair-force kernel timed alone (CUDA events), algorithmic bytes
          per launch / duration vs the measured HBM copy bandwidth;
  cpu_baseline: the oracle's float32 OpenMP restatement (kind "port") on a
          bounded sample of the same workload.

--impl reference runs only the CPU arm (the reference is JAX, absent here; the
oracle port stands in for it) and prints its own line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = 'atom-steps/s LJ N=864k NVE fp32'
N_CELLS = 60
DENSITY, KT, DT, SKIN = 0.8442, 0.722, 0.005, 0.3
# DRAM bytes per atom of the timed fused step of each engine list, from ncu
# captures at N=864,000 (dram__bytes_read.sum + dram__bytes_write.sum of the
# launches of one step, divided by N): the half-list step k_seg_half +
# k_seg_integrate, the tiled step k_tiled; None where not captured
DRAM_BYTES_PER_ATOM = {'half': 230.4, 'full': None, 'tiled': 378.4}


def workload(cells: int, n: int) -> str:
    """The workload string both arms print (same physics, same inputs)."""
    return (f'LJ fluid FCC {cells}^3x4 N={n} rho=0.8442 rc=2.5 r_onset=2.0 skin=0.3 '
            'dt=0.005 NVE Dense')


def peaks():
    p = ROOT / 'MEASURED_PEAKS.json'
    if p.exists():
        d = json.loads(p.read_text())
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ('clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', os.environ.get('CUDA_VISIBLE_DEVICES', '0').split(',')[0],
                                          f'--query-gpu={q}', '--format=csv,noheader,nounits',
                                          '-lms', '20'], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # let the sampler start before the timed region; keep only what follows
            t0 = time.perf_counter()
            while not self.samples and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        self.mark = len(self.samples)
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [s.strip() for s in line.split(',')]
            if len(parts) == 6:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if len(self.samples) > self.mark:
            self.samples = self.samples[self.mark:]
        if not self.samples:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unavailable']}
        sm = [float(s[0]) for s in self.samples if s[0].replace('.', '').isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if s[2 + k].lower() == 'active'})
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': max(mx) if mx else None, 'reasons': reasons, 'samples': len(self.samples)}


def cpu_port_run(R, P, L, steps, threads=0):
    from oracle import build as ob
    lib = ctypes.CDLL(str(ob.build()))
    fp = ctypes.POINTER(ctypes.c_float)
    lib.md_cpu_run.argtypes = [fp, fp, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                               ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    x = np.ascontiguousarray(R, np.float32).copy()
    p = np.ascontiguousarray(P, np.float32).copy()
    t0 = time.perf_counter()
    rb = lib.md_cpu_run(x.ctypes.data_as(fp), p.ctypes.data_as(fp), len(x), float(L), 2.0, 2.5,
                        SKIN, DT, 128, steps, threads)
    dt = time.perf_counter() - t0
    return dt, rb, lib.md_cpu_max_threads()


def _events(dev):
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def nvt_section(dev, efn, nfn, shift, R, P, steps, warmup):
    """The NVT half of the large workload: Nose-Hoover (chain 5, tau = 100 dt,
    kT = 0.722) on the same N = 864,000 system, K steps as one graph launch."""
    import torch
    from jax_md_gb300 import simulate
    Rt = torch.tensor(R, device=dev)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nvt_nose_hoover(efn, shift, DT, KT)
    st = init(0, Rt, momenta=torch.tensor(P, device=dev), neighbor=nb)
    simulate.run(apply, st, nb, max(3, warmup))
    simulate.run(apply, st, nb, steps)          # records the graph of K steps
    H0 = float(simulate.nvt_nose_hoover_invariant(efn, st, KT, neighbor=nb.update(st.position)))
    cur = torch.cuda.current_stream(dev)
    e0, e1 = _events(dev)
    torch.cuda.synchronize()
    e0.record(cur)
    simulate.run(apply, st, nb, steps)
    e1.record(cur)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    n = len(R)
    H1 = float(simulate.nvt_nose_hoover_invariant(efn, st, KT, neighbor=nb.update(st.position)))
    T = float((st.momentum.double() ** 2).sum() / (3 * n))
    return {'workload': f'Nose-Hoover NVT, same system, chain 5, tau=100 dt, kT={KT}',
            'steps': steps, 'atom_steps_per_s': n * steps / (ms / 1e3),
            'ms_per_step': ms / steps, 'invariant_drift_per_atom': (H1 - H0) / n,
            'temperature': T, 'overflow': bool(nb.did_buffer_overflow)}


def morse_section(dev, R, P, L, steps, warmup):
    """Morse pairs (energy.morse x the multiplicative cutoff: eps 5, alpha 5,
    radii 2.0 / 2.5) on the same N = 864,000 FCC positions, sigma at the
    lattice's nearest-neighbour distance (the crystal sits at the minimum),
    momenta at half the LJ run's: NVE, K steps as one graph launch.  The
    list (cutoff 2.5 + skin 0.3) matches the LJ run's, so the rates compare
    directly; a Morse pair costs two exponentials."""
    import torch
    from jax_md_gb300 import energy, partition, quantity, simulate, space
    sigma = float(np.float32((4 / DENSITY) ** (1 / 3) / np.sqrt(2)))
    disp, shift = space.periodic(float(L))
    nfn, efn = energy.morse_neighbor_list(disp, float(L), sigma=sigma, dr_threshold=SKIN,
                                          format=partition.Dense)
    Rt = torch.tensor(R, device=dev)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nve(efn, shift, DT)
    st = init(0, Rt, momenta=torch.tensor(P, device=dev) * 0.5, neighbor=nb)
    st, nb = simulate.run(apply, st, nb, max(3, warmup), neighbor_fn=nfn)
    st, nb = simulate.run(apply, st, nb, steps, neighbor_fn=nfn)   # records the graph
    E0 = float(efn.energy_f64(st.position, nb) + quantity._ke_f64(st.momentum))
    cur = torch.cuda.current_stream(dev)
    e0, e1 = _events(dev)
    torch.cuda.synchronize()
    e0.record(cur)
    simulate.run(apply, st, nb, steps)
    e1.record(cur)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    n = len(R)
    E1 = float(efn.energy_f64(st.position, nb) + quantity._ke_f64(st.momentum))
    return {'workload': f'Morse NVE (eps 5, alpha 5, sigma {sigma:.4f}, radii 2.0/2.5), same '
                        f'N={n} FCC positions, momenta x0.5',
            'steps': steps, 'atom_steps_per_s': n * steps / (ms / 1e3), 'ms_per_step': ms / steps,
            'energy_drift_per_atom': (E1 - E0) / n, 'overflow': bool(nb.did_buffer_overflow)}


def batched_section(dev, n_sys=512, fire_steps=200, nve_steps=200, seed=0, use_graph=True,
                    with_plain=True, f_tol=1e-6, fire_max=100000, nve_run=2000):
    """512 uneven 2D bidisperse soft-sphere systems (N ~ U[64, 4096], phi
    0.84, sigma_ij = (d_i + d_j) / 2 with d in {1.0, 1.4}).  The run as
    stated: FIRE from the random start until every system has max |F_i| <
    f_tol (a system that gets there stops; the ones that stall at the
    float32 floor run to fire_max, and the floor is reported), then nve_run
    NVE steps at kT = 1e-4 -- all systems in one graph launch per chunk.
    Throughput against the single-system API, system by system on the same
    GPU, over the same number of steps (fire_steps FIRE steps, nve_steps NVE
    steps; one CUDA graph per system on both)."""
    import torch
    from jax_md_gb300 import batch, energy, minimize, partition, simulate, space
    from oracle import md_oracle as O
    rng = np.random.default_rng(seed)
    sizes = rng.integers(64, 4097, n_sys)
    systems = [O.bidisperse_2d(int(n), 0.84, seed + 1 + k) for k, n in enumerate(sizes)]
    sigma = np.array([[1.0, 1.2], [1.2, 1.4]])
    n_tot = int(sizes.sum())
    Rs = [torch.tensor(R, device=dev) for R, L, sp in systems]
    bt = batch.pack(Rs, [float(L) for R, L, sp in systems], species=[sp for R, L, sp in systems])
    disp, _ = space.periodic(float(systems[0][1]))
    _, efn = energy.soft_sphere_neighbor_list(disp, float(systems[0][1]),
                                              torch.tensor(systems[0][2], device=dev), sigma=sigma)
    fns = batch.neighbor_list(1.4, 0.2)
    nb = fns.allocate(bt, extra_capacity=4)
    run = batch.BatchRunner(bt, fns, nb, batch.BatchPairEnergy(efn), dt=0.01)
    run.fire_init(0.0)
    tuned = batch.autotune(run, steps=20)      # launch shapes of the batched kernels
    x0, f0 = bt.position.clone(), run.force.clone()
    cur = torch.cuda.current_stream(dev)

    def timed(fn):
        e0, e1 = _events(dev)
        torch.cuda.synchronize()
        e0.record(cur)
        out = fn()
        e1.record(cur)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, out

    def restore():
        bt.position.copy_(x0)
        run.force.copy_(f0)
        fns._build(nb, bt.position)
        run.fire_init(0.0)

    def max_force_per_system():
        f = run.force[:, :2].double().norm(dim=1)
        out = torch.zeros(n_sys, dtype=torch.float64, device=dev)
        return out.scatter_reduce(0, bt.atom_sys.long(), f, reduce='amax', include_self=True)

    # throughput legs: fixed step counts, graph-replayed
    restore()
    run.fire(fire_steps, use_graph)          # records the graph
    restore()
    t_bfire, _ = timed(lambda: run.fire(fire_steps, use_graph))
    # the stated run: FIRE to f_tol, then NVE; the per-system max force is
    # read back between chunks (a system under f_tol stops)
    chunk = 10000
    restore()
    run.fire_init(f_tol)
    run.fire(chunk, use_graph)                # records the chunk's graph
    restore()
    run.fire_init(f_tol)
    progress, fire_taken, t_min = [], 0, 0.0
    while fire_taken < fire_max:
        dt_chunk, _ = timed(lambda: run.fire(chunk, use_graph))
        t_min += dt_chunk
        fire_taken += chunk
        fm = max_force_per_system()
        progress.append([fire_taken, int(run.n_done.item()), float(fm.max()), float(fm.median())])
        if progress[-1][1] == n_sys:
            break
    fmax = max_force_per_system()
    converged = int((fmax < f_tol).sum())
    # float32 resolution of the positions: one ulp of the box side L
    boxes = torch.as_tensor([float(L) for R, L, sp in systems], dtype=torch.float64, device=dev)
    ulp = torch.pow(2.0, torch.floor(torch.log2(boxes)) - 23)
    floor_ratio = fmax / ulp
    run.set_momenta(1e-4, seed=7)
    p0 = run.momentum.clone()
    run.nve(nve_steps, use_graph)            # records the graph
    run.momentum.copy_(p0)
    t_bnve, _ = timed(lambda: run.nve(nve_steps, use_graph))
    t_run_nve, _ = timed(lambda: run.nve(nve_run, use_graph))
    overflow = bool(nb.did_buffer_overflow)
    stated = {'fire_f_tol': f_tol, 'fire_steps_run': int(fire_taken), 'fire_s': t_min,
              'systems_converged': converged, 'systems': n_sys,
              'max_force_after_fire': float(fmax.max()),
              'median_max_force_after_fire': float(fmax.median()),
              'progress_steps_done_maxF_medianF': progress,
              'max_force_over_position_ulp': {'median': float(floor_ratio.median()),
                                              'max': float(floor_ratio.max())},
              'nve_steps': nve_run, 'nve_s': t_run_nve,
              'note': 'the float32 floor: a position carries one ulp of the box side, so with '
                      'unit contact stiffness the residual force of a packing cannot fall much '
                      'below a few ulp(L); the systems that reach the tolerance are the small '
                      'boxes, the others stall at max_force_over_position_ulp ulps'}
    if not with_plain:
        return {'workload': f'{n_sys} 2D bidisperse soft-sphere systems (total {n_tot})',
                'autotune': tuned, 'stated_run': stated,
                'batched_fire_atom_steps_per_s': n_tot * fire_steps / t_bfire,
                'batched_nve_atom_steps_per_s': n_tot * nve_steps / t_bnve,
                'launch': 'cuda graph' if use_graph else 'direct', 'overflow': overflow}

    # plain: the same systems one at a time through the single-system API,
    # each system's FIRE steps captured in its own CUDA graph
    plain = []
    for k, (R, L, sp) in enumerate(systems):
        d_k, s_k = space.periodic(float(L))
        nfn_k, efn_k = energy.soft_sphere_neighbor_list(d_k, float(L), torch.tensor(sp, device=dev),
                                                        sigma=sigma, format=partition.Dense)
        Rk = torch.tensor(R, device=dev)
        plain.append((nfn_k, efn_k, s_k, Rk, nfn_k.allocate(Rk, extra_capacity=4)))
    chunk = 50
    graphs = []
    for nfn_k, efn_k, s_k, Rk, nb_k in plain:
        init, apply = minimize.fire_descent(efn_k, s_k)
        st = init(Rk.clone(), neighbor=nb_k)
        apply(st, neighbor=nb_k.update(st.position))    # allocates the kernels' scratch
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(chunk):
                apply(st, neighbor=nb_k.update(st.position))
        graphs.append(g)

    def plain_fire():
        for g in graphs:
            for _ in range(fire_steps // chunk):
                g.replay()
    t_pfire, _ = timed(plain_fire)
    del graphs
    states = []
    for k, (nfn_k, efn_k, s_k, Rk, nb_k) in enumerate(plain):
        init, apply = simulate.nve(efn_k, s_k, 0.01)
        pk = p0[bt.rows(k), :2]
        st = init(0, Rk, momenta=pk, neighbor=nb_k)
        # records each system's graph (every run re-sorts at its start: one
        # graph per system, which the timed pass replays)
        simulate.run(apply, st, nb_k, nve_steps, warm_start=False)
        states.append((apply, st, nb_k))

    def plain_nve():
        for apply, st, nb_k in states:
            simulate.run(apply, st, nb_k, nve_steps, warm_start=False)
    t_pnve, _ = timed(plain_nve)
    fire_plain_steps = (fire_steps // chunk) * chunk
    return {
        'workload': f'{n_sys} 2D bidisperse soft-sphere systems, N~U[64,4096] (total {n_tot}), '
                    f'phi=0.84, skin 0.2, FIRE to max|F|<{f_tol:g} then {nve_run} NVE steps '
                    'kT=1e-4 dt=0.01',
        'stated_run': stated,
        'fire_steps': fire_steps, 'nve_steps': nve_steps, 'autotune': tuned,
        'batched_fire_atom_steps_per_s': n_tot * fire_steps / t_bfire,
        'plain_fire_atom_steps_per_s': n_tot * fire_plain_steps / t_pfire,
        'fire_speedup': (n_tot * fire_steps / t_bfire) / (n_tot * fire_plain_steps / t_pfire),
        'batched_nve_atom_steps_per_s': n_tot * nve_steps / t_bnve,
        'plain_nve_atom_steps_per_s': n_tot * nve_steps / t_pnve,
        'nve_speedup': t_pnve / t_bnve,
        'plain': 'per-system calls of the single-system API on the same GPU (FIRE: each '
                 f'system\'s {chunk} steps captured in its own CUDA graph; NVE: simulate.run, '
                 'one engine graph per system)',
        'overflow': overflow,
    }


def _ka_replica(rng, n):
    """A seeded Kob-Andersen replica of exactly n atoms at rho = 1.2: n
    distinct sites drawn from the smallest cubic lattice that has n, jittered
    by +-0.05 of the spacing; 20% B; momenta Gaussian at kT = 0.6."""
    L = float(np.float32((n / 1.2) ** (1 / 3)))
    m = int(np.ceil(n ** (1 / 3) - 1e-9))
    while m ** 3 < n:
        m += 1
    g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing='ij'), -1).reshape(-1, 3)
    g = g[np.sort(rng.choice(len(g), n, replace=False))]
    a = L / m
    R = np.mod((g + 0.5) * a + rng.uniform(-0.05, 0.05, g.shape) * a, L).astype(np.float32)
    sp = np.zeros(n, np.int32)
    sp[rng.permutation(n)[: n // 5]] = 1
    P = (rng.standard_normal(R.shape) * np.sqrt(0.6)).astype(np.float32)
    P -= P.mean(0, keepdims=True)
    return R, P, L, sp


def batched_adjoint_section(dev, n_sys=128, steps=500, seed=0):
    """128 Kob-Andersen replicas (80:20, rho = 1.2, N drawn uniformly from
    [500, 20000], seeded random lattice-site states, momenta at kT = 0.6):
    gradient of the ensemble-mean PE/N after 500 Nose-Hoover steps (chain 5,
    tau = 100 dt, kT = 0.6) with respect to the shared sigma / epsilon
    matrices, by the batched adjoint (record length chosen to fit HBM),
    against the cost of finite differences with plain per-replica forward
    runs (one CUDA graph per replica; central differences of the two AB
    parameters need five ensemble passes, one is timed).  The NVE adjoint of
    the same replicas is reported beside it."""
    import torch
    from jax_md_gb300 import batch, energy, partition, simulate, space
    rng = np.random.default_rng(seed)
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sizes_n = rng.integers(500, 20001, n_sys)
    systems = [_ka_replica(rng, int(n)) for n in sizes_n]
    n_tot = sum(len(x[0]) for x in systems)
    bt = batch.pack([torch.tensor(R, device=dev) for R, P, L, sp in systems],
                    [L for R, P, L, sp in systems], species=[sp for R, P, L, sp in systems])
    disp, shift = space.periodic(systems[0][2])
    _, efn = energy.lennard_jones_neighbor_list(disp, systems[0][2],
                                                torch.tensor(systems[0][3], device=dev),
                                                sigma=sig, epsilon=eps, dr_threshold=0.3)
    fns = batch.neighbor_list(2.5, 0.3)
    nb = fns.allocate(bt, extra_capacity=12)
    ef = batch.BatchPairEnergy(efn)
    R0 = bt.R.clone()
    P0 = torch.tensor(np.concatenate([P for R, P, L, sp in systems]), device=dev)
    sizes = torch.tensor(bt.sizes, dtype=torch.float64, device=dev)
    sig_t = torch.tensor(sig, dtype=torch.float32, device=dev, requires_grad=True)
    eps_t = torch.tensor(eps, dtype=torch.float32, device=dev, requires_grad=True)

    def timed(fn):
        e0, e1 = _events(dev)
        torch.cuda.synchronize()
        e0.record(torch.cuda.current_stream(dev))
        out = fn()
        e1.record(torch.cuda.current_stream(dev))
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3, out

    def adjoint_leg(traj):
        def forward():
            with torch.no_grad():
                return traj(R0, P0, sigma=sig_t.detach(), epsilon=eps_t.detach())

        def forward_backward():
            sig_t.grad = None
            eps_t.grad = None
            xn, pn = traj(R0, P0, sigma=sig_t, epsilon=eps_t)
            fns.update(torch.nn.functional.pad(xn.detach(), (0, 1)).contiguous(), nb)
            E = ef.energy_fn_autograd(bt, nb)(xn, sigma=sig_t, epsilon=eps_t)
            loss = (E / sizes).mean()
            loss.backward()
            return loss
        forward()
        forward_backward()
        t_f, _ = timed(forward)
        t_fb, loss = timed(forward_backward)
        return {'forward_s': t_f, 'forward_backward_s': t_fb,
                'gradient_cost_ratio': t_fb / t_f,
                'batched_forward_atom_steps_per_s': n_tot * steps / t_f,
                'dloss_dsigma_AB': float((sig_t.grad[0, 1] + sig_t.grad[1, 0]).detach()),
                'dloss_depsilon_AB': float((eps_t.grad[0, 1] + eps_t.grad[1, 0]).detach()),
                'loss': float(loss.detach()), 'overflow': bool(nb.did_buffer_overflow)}

    def plain_leg(nvt):
        runs = []
        for R, P, L, sp in systems:
            d_k, s_k = space.periodic(L)
            nfn_k, efn_k = energy.lennard_jones_neighbor_list(
                d_k, L, torch.tensor(sp, device=dev), sigma=sig, epsilon=eps, dr_threshold=0.3,
                format=partition.Dense)
            Rk = torch.tensor(R, device=dev)
            nb_k = nfn_k.allocate(Rk, extra_capacity=12)
            if nvt:
                init, apply = simulate.nvt_nose_hoover(efn_k, s_k, 0.005, 0.6)
            else:
                init, apply = simulate.nve(efn_k, s_k, 0.005)
            st = init(0, Rk, momenta=torch.tensor(P, device=dev), neighbor=nb_k)
            # captures this replica's graph (every run re-sorts at its start:
            # one graph per replica, which the timed pass replays)
            simulate.run(apply, st, nb_k, steps, warm_start=False)
            runs.append((apply, st, nb_k))

        def plain():
            for apply, st, nb_k in runs:
                simulate.run(apply, st, nb_k, steps, warm_start=False)
        t, _ = timed(plain)
        return t

    trn = batch.BatchNvtTrajectory(bt, fns, nb, ef, 0.005, 0.6, steps)
    seg = trn.segment_length(bt.n, 3)
    out = {
        'workload': f'{n_sys} Kob-Andersen replicas, N from U[500,20000] (total {n_tot}), '
                    f'rho=1.2, {steps} Nose-Hoover steps (chain 5, tau=100 dt, kT=0.6) dt=0.005, '
                    'loss mean_b PE_b/N_b, grad wrt shared sigma[2x2], epsilon[2x2]',
        'record': {'steps_per_segment': seg, 'checkpointed': seg < steps,
                   'bytes_per_step': 3 * bt.n * 3 * 4 + 2 * n_sys * 66 * 8},
    }
    try:
        out.update(adjoint_leg(trn))
        t_plain = plain_leg(True)
        out.update({'plain_forward_ensemble_s': t_plain,
                    'plain_finite_difference_s': 5 * t_plain,
                    'speedup_vs_finite_differences': 5 * t_plain / out['forward_backward_s'],
                    'plain': 'per-replica simulate.run of nvt_nose_hoover, one CUDA graph per '
                             'replica; central differences of the two AB parameters = 5 ensemble '
                             'passes (one timed)'})
    except (RuntimeError, MemoryError) as ex:
        out['error'] = str(ex)[:300]
    # the NVE adjoint of the same replicas (graph-replayed segments)
    try:
        nve = adjoint_leg(batch.BatchTrajectory(bt, fns, nb, ef, 0.005, steps))
        t_plain_nve = plain_leg(False)
        nve.update({'workload': f'same replicas, {steps} NVE steps',
                    'plain_forward_ensemble_s': t_plain_nve,
                    'speedup_vs_finite_differences': 5 * t_plain_nve / nve['forward_backward_s']})
    except (RuntimeError, MemoryError) as ex:
        nve = {'error': str(ex)[:300]}
    out['nve'] = nve
    out['note'] = ('over 500 steps the gradient of a chaotic trajectory is large; the FP64 '
                   'finite-difference checks run 12-20 steps (tests)')
    return out


def adjoint_section(dev, steps=2000, checkpoint_every=100, seed=0):
    """Kob-Andersen 80:20 binary LJ, N = 8000 at rho = 1.2: 200 FIRE steps,
    momenta at kT = 0.8, then the gradient of PE/N + 0.1 MSD after 2000 NVE
    steps (dt 0.005) with respect to the species sigma / epsilon matrices and
    the initial positions, checkpointed every 100 steps; reports the forward
    time and the forward + backward time."""
    import torch
    from jax_md_gb300 import adjoint, energy, minimize, partition, space
    from oracle import md_oracle as O
    n_side = 20
    L = float(np.float32((n_side ** 3 / 1.2) ** (1 / 3)))
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(n_side)] * 3, indexing='ij'), -1).reshape(-1, 3)
    R = np.mod((g + 0.5) * (L / n_side) + rng.uniform(-0.05, 0.05, g.shape), L).astype(np.float32)
    n = len(R)
    species = np.zeros(n, np.int32)
    species[rng.permutation(n)[: n // 5]] = 1
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    disp, shift = space.periodic(L)
    sp_t = torch.tensor(species, device=dev)
    nfn, efn = energy.lennard_jones_neighbor_list(disp, L, sp_t, sigma=sig, epsilon=eps,
                                                  dr_threshold=0.3, format=partition.Dense)
    Rt = torch.tensor(R, device=dev)
    nb = nfn.allocate(Rt, extra_capacity=8)
    init, apply = minimize.fire_descent(efn, shift)
    st = init(Rt, neighbor=nb)
    for _ in range(200):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    R0 = st.position.contiguous().clone()
    # the relaxed structure has another occupancy than the lattice start
    nb = nfn.allocate(R0, extra_capacity=8)
    P0 = torch.tensor(O.maxwell_boltzmann(n, 3, 0.8, seed + 1), device=dev)
    traj = adjoint.nve_trajectory(efn, nfn, shift, 0.005, steps, checkpoint_every=checkpoint_every)
    sig_t = torch.tensor(sig, dtype=torch.float32, device=dev, requires_grad=True)
    eps_t = torch.tensor(eps, dtype=torch.float32, device=dev, requires_grad=True)

    def forward():
        with torch.no_grad():
            return traj(R0, P0, nb, sigma=sig_t.detach(), epsilon=eps_t.detach())

    def forward_backward():
        Rg = R0.clone().requires_grad_(True)
        xn, pn = traj(Rg, P0, nb, sigma=sig_t, epsilon=eps_t)
        nb2 = nb.update(xn.detach())
        E = efn(xn, nb2, sigma=sig_t, epsilon=eps_t)
        d = disp(xn, Rg)
        loss = E / n + 0.1 * (d * d).sum(-1).mean()
        loss.backward()
        return loss

    forward()
    forward_backward()
    cur = torch.cuda.current_stream(dev)
    out = {}
    for name, fn in (('forward_s', forward), ('forward_backward_s', forward_backward)):
        e0, e1 = _events(dev)
        torch.cuda.synchronize()
        e0.record(cur)
        fn()
        e1.record(cur)
        torch.cuda.synchronize()
        out[name] = e0.elapsed_time(e1) / 1e3
    out.update({
        'workload': f'Kob-Andersen N={n} rho=1.2, 200 FIRE steps, kT=0.8, {steps} NVE steps '
                    f'dt=0.005, checkpoints every {checkpoint_every}, loss PE/N + 0.1 MSD, '
                    'grad wrt sigma[2x2], epsilon[2x2], R0',
        'gradient_cost_ratio': out['forward_backward_s'] / out['forward_s'],
        'forward_atom_steps_per_s': n * steps / out['forward_s'],
    })
    return out


def cpu_nvt_baseline(R, P, L, budget_s=8.0):
    """The float32 OpenMP port's Nose-Hoover run (chain 5, tau = 100 dt, chain
    in f64) on a bounded number of steps of the same system."""
    from oracle import build as ob
    lib = ctypes.CDLL(str(ob.build()))
    fp = ctypes.POINTER(ctypes.c_float)
    lib.md_cpu_run_nvt.argtypes = [fp, fp, ctypes.c_int] + [ctypes.c_float] * 5 + \
        [ctypes.c_int] * 3 + [ctypes.c_double] * 2 + [ctypes.c_int] * 3 + [ctypes.c_void_p]

    def run(steps):
        x = np.ascontiguousarray(R, np.float32).copy()
        p = np.ascontiguousarray(P, np.float32).copy()
        t0 = time.perf_counter()
        rb = lib.md_cpu_run_nvt(x.ctypes.data_as(fp), p.ctypes.data_as(fp), len(x), float(L), 2.0,
                                2.5, SKIN, DT, 128, steps, 0, KT, 100 * DT, 5, 2, 3, None)
        return time.perf_counter() - t0, rb
    dt1, _ = run(2)
    steps = min(200, max(2, int(budget_s / max(dt1 / 2, 1e-3))))
    dt, rb = run(steps)
    threads = ctypes.CDLL(str(ob.build())).md_cpu_max_threads()
    return {'value': len(R) * steps / dt, 'unit': 'atom-steps/s', 'cores': threads, 'kind': 'port',
            'sample': f'{steps} Nose-Hoover steps of the N={len(R)} LJ system ({rb} rebuilds), '
                      f'float32 OpenMP restatement, {threads} threads'}


def cpu_baseline(R, P, L, budget_s=15.0):
    """Times the float32 OpenMP port on a bounded number of steps of the same system."""
    dt1, _, threads = cpu_port_run(R, P, L, 2)
    steps = max(2, int(budget_s / max(dt1 / 2, 1e-3)))
    steps = min(steps, 200)
    dt, rb, threads = cpu_port_run(R, P, L, steps)
    return {'value': len(R) * steps / dt, 'unit': 'atom-steps/s', 'cores': threads, 'kind': 'port',
            'sample': f'{steps} NVE steps of the N={len(R)} LJ system (full size, '
                      f'{rb} rebuilds), float32 OpenMP restatement, {threads} threads'}


def run_reference(args):
    import torch.distributed as dist  # noqa: F401
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    from oracle import md_oracle as O
    R, L = O.fcc_lattice(N_CELLS, DENSITY, 0.05, 0)
    P = O.maxwell_boltzmann(len(R), 3, KT, 1)
    # warmup + timed, each step a bounded sample (the whole run stays within minutes)
    sample_steps = 5
    for _ in range(args.warmup):
        cpu_port_run(R, P, L, 1)
    times = []
    threads = 0
    for _ in range(args.steps):
        dt, rb, threads = cpu_port_run(R, P, L, sample_steps)
        times.append(dt / sample_steps)
    per = float(np.median(times))
    v = len(R) / per
    line = {'metric': METRIC, 'value': v, 'unit': 'atom-steps/s', 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': per * 1e3,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic', 'impl': 'reference',
            'config': {'workload': workload(N_CELLS, len(R)), 'inputs': 'host memory (CPU run)'},
            'cpu_baseline': {'value': v, 'unit': 'atom-steps/s', 'cores': threads, 'kind': 'port',
                             'sample': f'{sample_steps} NVE steps per timed step incl. cell list, '
                                       'neighbour list and forces (float32 OpenMP restatement; '
                                       'JAX is not installed on this box)'},
            'e2e': {'value': v, 'unit': 'atom-steps/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=1000)
    ap.add_argument('--warmup', type=int, default=20)
    ap.add_argument('--impl', default='native')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-extras', action='store_true',
                    help='skip the batched and adjoint measurements')
    ap.add_argument('--cells', type=int, default=N_CELLS)
    ap.add_argument('--workload', default='lj864k', choices=['lj864k', 'batched'],
                    help='batched: only the batched soft-sphere workload (FIRE + NVE)')
    ap.add_argument('--no-tune', action='store_true',
                    help='skip the segment autotuner (default cells per segment and threads)')
    ap.add_argument('--segment', default=None,
                    help='cells,threads,stage_lists,half: use this segment launch shape '
                         'instead of autotuning (for profiling a chosen shape)')
    ap.add_argument('--direct', action='store_true',
                    help='launch the engine kernels directly instead of replaying its CUDA '
                         'graph (profilers list every kernel of the timed region this way)')
    args = ap.parse_args()
    if args.impl == 'reference':
        return run_reference(args)

    import torch
    from jax_md_gb300 import _build
    _build.build()
    from jax_md_gb300 import energy, partition, quantity, simulate, space
    from jax_md_gb300 import _native as NAT
    from oracle import md_oracle as O

    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    dev = torch.device(f'cuda:{local}')
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')

    if args.workload == 'batched':
        r = batched_section(dev, fire_steps=args.steps, nve_steps=args.steps,
                            use_graph=not args.direct, with_plain=False)
        if rank == 0:
            print(json.dumps({'metric': 'atom-steps/s batched 2D soft spheres (FIRE, NVE)',
                              'value': r['batched_nve_atom_steps_per_s'], 'unit': 'atom-steps/s',
                              'n_gpus': world, 'steps': args.steps, 'higher_is_better': True,
                              'config': r}))
        return
    R, L = O.fcc_lattice(args.cells, DENSITY, 0.05, 0)
    P = O.maxwell_boltzmann(len(R), 3, KT, 1)
    n = len(R)
    disp, shift = space.periodic(float(L))
    nfn, efn = energy.lennard_jones_neighbor_list(disp, float(L), dr_threshold=SKIN,
                                                  format=partition.Dense)
    Rt = torch.tensor(R, device=dev)
    nb = nfn.allocate(Rt)
    init, apply = simulate.nve(efn, shift, DT)
    st = init(0, Rt, momenta=torch.tensor(P, device=dev), neighbor=nb)

    # launch shape: project autotuner (cells per segment, threads per CTA of
    # the engine's segment-local list), timed on copies of this state
    from jax_md_gb300 import tune
    if args.segment:
        seg_choice = ('tiled' if args.segment == 'tiled' else
                      tuple(int(v) for v in args.segment.split(',')))
        simulate._segment_choice[simulate._grid_key(nb.plan.nl)] = seg_choice
        seg_ms = {}
    elif args.no_tune:
        seg_choice, seg_ms = None, {}
    else:
        seg_choice, seg_ms = tune.autotune_segment(apply, st, nb, steps=20, use_cache=False)
    # warm-up: the engine run (also builds and caches its CUDA graph)
    graphed = not args.direct
    simulate.run(apply, st, nb, max(3, args.warmup), use_graph=graphed)
    torch.cuda.synchronize()
    simulate.run(apply, st, nb, args.steps, use_graph=graphed)  # records the graph for K steps
    torch.cuda.synchronize()
    E0 = float(efn.energy_f64(st.position, nb) + quantity._ke_f64(st.momentum))
    rebuilds0 = 0
    cur = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks() as clk:
        torch.cuda.nvtx.range_push('timed')
        ev0.record(cur)
        simulate.run(apply, st, nb, args.steps, use_graph=graphed)  # exactly K steps
        ev1.record(cur)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t)
    ms_per_step = ms / args.steps
    value = n * world * args.steps / (ms / 1e3)
    E1 = float(efn.energy_f64(st.position, nb) + quantity._ke_f64(st.momentum))
    overflow = bool(nb.did_buffer_overflow)

    # dominant kernel alone: the segment fused step on the engine's
    # cell-ordered state (force + both half kicks + drift + skin test)
    import ctypes as _C
    sb = st._sorted
    nbar = float(sb.cnt.float().mean())
    # list bytes per atom a perfect kernel reads: two-byte entries (half of
    # them with half lists) + count
    chunk_bytes = (2.0 * float(sb.cnt.clamp(max=nb.max_occupancy).double().mean())
                   / (2.0 if getattr(sb, 'seg_half', 0) else 1.0) + 2.0)
    species, pair = efn._resolve(st.position, {})
    sp = simulate._shift_space(shift, 3)
    xo = torch.empty((n, 4), dtype=torch.float32, device=dev)
    pm = sb.p.clone()
    flag = torch.zeros((), dtype=torch.int32, device=dev)
    L_ = NAT.lib()
    seg_on = sb.seg is not None
    facc = torch.zeros((n, 4), dtype=torch.float32, device=dev)  # half lists' force accumulator

    def fused():
        if seg_on:
            NAT.check(L_.jmd_nve_fused_step_segment(
                _C.byref(pair), _C.byref(sp), _C.byref(nb.plan.nl), sb.seg_cells, sb.seg_threads,
                sb.seg_list_smem, sb.seg_half, sb.xa.data_ptr(), xo.data_ptr(), pm.data_ptr(),
                facc.data_ptr(), 1.0, n, 0, sb.seg.data_ptr(), sb.seg.numel(), DT,
                sb.ref.data_ptr(), nb.plan.threshold_sq, flag.data_ptr(), sb.ws.data_ptr(),
                sb.ws.numel(), sb.seg_status.data_ptr(), NAT.stream_ptr()), 'segment fused step')
        else:
            NAT.check(L_.jmd_nve_fused_step_tiled(_C.byref(pair), _C.byref(sp), sb.xa.data_ptr(),
                                                  xo.data_ptr(), pm.data_ptr(), 1.0, None, n,
                                                  sb.idx.data_ptr(), sb.ld, nb.max_occupancy,
                                                  sb.cnt.data_ptr(), DT, sb.ref.data_ptr(),
                                                  nb.plan.threshold_sq, flag.data_ptr(),
                                                  NAT.stream_ptr()), 'fused step')
    for _ in range(3):
        fused()
    torch.cuda.synchronize()
    reps = 50
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(cur)
    for r in range(reps):
        fused()            # same input each time: identical work per launch
    e1.record(cur)
    torch.cuda.synchronize()
    kern_ms = e0.elapsed_time(e1) / reps
    assert int(sb.seg_status) == 0, 'segment staging reported a problem'
    # algorithmic bytes of one atom-step of the path (plain Dense LJ NVE,
    # fp32): 4 n-bar (the Dense list entries) + 96 (position, momentum and
    # force rows read and written, 16 B each), n-bar the mean stored
    # neighbour count -- the path's figure, independent of the layout that
    # runs it.  The timed layout itself needs fewer: `layout_bytes_per_atom`
    # (the list as read -- 16-byte chunks of 8 two-byte staged slots, or int32
    # entries on the tiled list -- with the count, position read + write,
    # momentum read + write, reference read, and for half lists the force
    # accumulator reduced into, read and cleared), and the ncu DRAM bytes in
    # `traffic`.
    path_bytes = 4.0 * nbar + 96.0
    list_bytes = chunk_bytes if seg_on else 4 * nbar + 4
    half = bool(getattr(sb, 'seg_half', 0)) and seg_on
    layout_name = 'half' if half else ('full' if seg_on else 'tiled')
    layout_bytes = list_bytes + 80 + (48 if half else 0)
    kern_bytes = n * path_bytes
    hbm, src = peaks()
    achieved = kern_bytes / (kern_ms / 1e3) / 1e9
    step_bytes = kern_bytes

    # e2e: host pinned buffers through the public API (simulate.run, default
    # path), every step: positions and momenta copied in, one step, copied out
    xh = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    ph = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    xh.copy_(st.position)
    ph.copy_(st.momentum)
    e2e_steps = max(5, min(args.steps, 50))
    # two public-API variants of a one-step call: the default (the atoms are
    # sorted into cell order and the private list built on every call) and
    # sort=False (the caller's Dense list, rebuilt only when the skin test
    # fires); the faster is reported, with its name
    e2e_variants = {}
    for name, sort in (('simulate.run(apply, state, nbrs, 1)', None),
                       ('simulate.run(apply, state, nbrs, 1, sort=False)', False)):
        simulate.run(apply, st, nb, 1, sort=sort)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            st.position.copy_(xh, non_blocking=True)
            st.momentum.copy_(ph, non_blocking=True)
            simulate.run(apply, st, nb, 1, sort=sort)
            xh.copy_(st.position, non_blocking=True)
            ph.copy_(st.momentum, non_blocking=True)
        torch.cuda.synchronize()
        e2e_variants[name] = n * world * e2e_steps / (time.perf_counter() - t0)
    e2e_call = max(e2e_variants, key=e2e_variants.get)
    e2e_value = e2e_variants[e2e_call]

    # per step: the fused step kernel + the conditional-set kernel; the rebuild
    # chain (6 kernels) runs only on rebuild steps
    launches_per_step = 2
    line = {
        'metric': METRIC, 'value': value, 'unit': 'atom-steps/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_per_step,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic',
        'config': {'workload': workload(args.cells, n),
                   'multi_gpu': 'replicas only (one independent system per GPU)',
                   'l2': 'inputs larger than L2 (neighbour list ~%d MB)' % int(n * list_bytes / 1e6),
                   'mean_neighbors': nbar, 'max_occupancy': nb.max_occupancy,
                   'launch': 'cuda graph' if graphed else 'direct',
                   'private_list': 'segment-local (16-bit staged slots)' if seg_on else 'tiled int32',
                   'segment': {'cells': sb.seg_cells, 'threads': sb.seg_threads,
                               'list_smem_bytes': sb.seg_list_smem,
                               'half_lists': bool(getattr(sb, 'seg_half', 0)),
                               'autotuned': seg_choice is not None and not args.segment,
                               'autotune_ms_per_step': {(k if isinstance(k, str) else
                                                         'x'.join(str(int(v)) for v in k)): t
                                                        for k, t in seg_ms.items()}},
                   'energy_drift_per_atom': (E1 - E0) / n, 'overflow': overflow},
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': hbm, 'unit': 'GB/s',
                     'frac': achieved / hbm,
                     'traffic': (DRAM_BYTES_PER_ATOM[layout_name] * n
                                 if DRAM_BYTES_PER_ATOM.get(layout_name) else None),
                     'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of the '
                                       'timed step\'s launches at N=864000, per atom x N',
                     'layout': layout_name,
                     'peak_source': src,
                     'kernel': (('k_seg_half + k_seg_integrate (LJ, segment-local half lists, '
                                 'Newton\'s third law, FP32x2)') if half else
                                ('k_seg_step fused NVE step (LJ, segment-local list, FP32x2)'
                                 if seg_on else 'k_tiled fused NVE step (LJ, Dense tiled, FP32x2)')),
                     'kernel_ms': kern_ms,
                     'bytes_per_atom': path_bytes,
                     'bytes_per_atom_rule': '4 n_bar + 96 (Dense list entries + position, '
                                            'momentum and force rows read and written)',
                     'layout_bytes_per_atom': layout_bytes,
                     'step_algorithmic_GBps': step_bytes * args.steps / (ms / 1e3) / 1e9},
        'e2e': {'value': e2e_value, 'unit': 'atom-steps/s', 'h2d_bytes_per_step': 2 * n * 12,
                'd2h_bytes_per_step': 2 * n * 12, 'call': e2e_call,
                'variants': e2e_variants,
                'per_step': 'pinned host positions and momenta copied in, one step, copied out'},
        'gpu_launches': launches_per_step * args.steps,
        'clocks': clk.summary(),
    }
    if rank == 0 and not args.no_extras:
        line['nvt'] = nvt_section(dev, efn, nfn, shift, R, P, args.steps, args.warmup)
        line['batched'] = batched_section(dev)
        line['adjoint'] = adjoint_section(dev)
        line['batched_adjoint'] = batched_adjoint_section(dev)
    if rank == 0 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline(R, P, L)
        if 'nvt' in line:
            line['nvt']['cpu_baseline'] = cpu_nvt_baseline(R, P, L)
    if rank == 0 and not args.no_extras:
        # last, and guarded: the newest kernels, so that nothing they do can
        # cost the line above
        try:
            line['morse'] = morse_section(dev, R, P, L, args.steps, args.warmup)
        except (RuntimeError, MemoryError) as ex:
            line['morse'] = {'error': str(ex)[:300]}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
