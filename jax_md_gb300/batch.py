"""Batches of independent periodic systems of uneven size on one GPU.

JAX MD batches systems with ``jax.vmap``, which needs every system to have
the same number of atoms.  Here systems of any sizes are packed end to end
(``pack``); every per-atom array of the batch is the concatenation of the
systems' arrays, ``sys_offset[b]:sys_offset[b+1]`` are system b's rows, and
each system keeps its own periodic box and its own cell grid.  Each phase of
a step (binning, neighbour search, forces, integration, the FIRE update) is a
single launch over all systems, and ``BatchRunner`` replays whole runs of NVE
(simulate.py:227-243) or FIRE (minimize.py:124-226) from one CUDA graph.

Per system the results are those of the single-system API: the neighbour
sets of ``partition.neighbor_list`` (partition.py:1034-1121, cell grid from
``_cell_dimensions`` with the list cutoff), the forces and energies of the
``smap.pair_neighbor_list`` energy it is given (smap.py:922-979), and the
updates of ``simulate.nve`` / ``minimize.fire_descent``.  Row order inside a
neighbour row may differ from the reference's (the sets are equal).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as N
from . import smap
from .smap import _bins_to_grads, _param_tensor


class Batch:
    """Systems packed end to end: positions ``[N, 4]`` float4 rows (the
    ``[N, dim]`` view is ``R``), ``sys_offset`` / ``atom_sys`` / ``box`` on the
    device, ``species`` (int32 ``[N]``) when given."""

    def __init__(self, positions: Sequence[torch.Tensor], boxes: Sequence, species=None,
                 device=None):
        if len(positions) == 0:
            raise ValueError('a batch needs at least one system')
        dims = {int(p.shape[1]) for p in positions}
        if len(dims) != 1 or dims.pop() not in (2, 3):
            raise ValueError('every system must have the same dimension, 2 or 3')
        self.dim = int(positions[0].shape[1])
        dev = torch.device(device) if device is not None else positions[0].device
        self.device = dev
        self.sizes = [int(p.shape[0]) for p in positions]
        self.n_systems = len(positions)
        off = np.zeros(self.n_systems + 1, np.int64)
        off[1:] = np.cumsum(self.sizes)
        if off[-1] >= 2 ** 31 - 1:
            raise ValueError('a batch holds fewer than 2^31 atoms')
        self.offsets = off
        self.n = int(off[-1])
        box = np.ones((self.n_systems, 3), np.float32)
        for b, L in enumerate(boxes):
            Lv = np.broadcast_to(np.asarray(L, np.float32), (self.dim,))
            if np.any(Lv <= 0):
                raise ValueError(f'system {b}: box sides must be positive')
            box[b, :self.dim] = Lv
        self.box_host = box
        self.box = torch.tensor(box, device=dev)
        self.position = torch.zeros((self.n, 4), dtype=torch.float32, device=dev)
        for b, p in enumerate(positions):
            pb = torch.as_tensor(p, dtype=torch.float32, device=dev)
            Lt = self.box[b, :self.dim]
            self.position[off[b]:off[b + 1], :self.dim] = torch.remainder(pb, Lt)
        self.sys_offset = torch.tensor(off.astype(np.int32), device=dev)
        self.atom_sys = torch.repeat_interleave(
            torch.arange(self.n_systems, dtype=torch.int32, device=dev),
            torch.tensor(self.sizes, device=dev)).to(torch.int32)
        self.species = None
        if species is not None:
            self.species = torch.cat([torch.as_tensor(s, device=dev).to(torch.int32).reshape(-1)
                                      for s in species]).contiguous()
            if self.species.numel() != self.n:
                raise ValueError('species must give one entry per atom of every system')

    @property
    def R(self) -> torch.Tensor:
        return self.position[:, :self.dim]

    def rows(self, b: int) -> slice:
        return slice(int(self.offsets[b]), int(self.offsets[b + 1]))

    def split(self, t: torch.Tensor) -> List[torch.Tensor]:
        """Per-system views of a per-atom array."""
        return [t[self.rows(b)] for b in range(self.n_systems)]


def pack(positions, boxes, species=None, device=None) -> Batch:
    """Packs systems (``[N_b, dim]`` positions, box side(s) per system,
    optional per-atom species) into one Batch."""
    return Batch(positions, boxes, species, device)


class _Grid:
    """Per-system cell grids for a list cutoff (partition.py:146-188 per
    system: cells_per_side = floor(L / cutoff), cell_size = L / cells_per_side)."""

    def __init__(self, batch: Batch, cutoff: float):
        L = batch.box_host[:, :batch.dim]
        # a box shorter than three cutoffs gets one or two cells along that axis,
        # where the search visits each distinct cell once (the pair set of the
        # reference's all-pairs candidates, partition.py:893-898)
        cps = np.maximum(np.floor(L / np.float32(cutoff)).astype(np.int64), 1)
        cs = (L / cps.astype(np.float32)).astype(np.float32)
        ncell = np.prod(cps, axis=1)
        if int(ncell.max()) > 24576:
            raise ValueError('a system has more than 24576 cells (the batched binning works in '
                             'shared memory); raise the cutoff or split the system')
        coff = np.zeros(batch.n_systems + 1, np.int64)
        coff[1:] = np.cumsum(ncell)
        cps3 = np.ones((batch.n_systems, 3), np.int32)
        cps3[:, :batch.dim] = cps
        cs3 = np.ones((batch.n_systems, 3), np.float32)
        cs3[:, :batch.dim] = cs
        dev = batch.device
        self.cps = torch.tensor(cps3, device=dev)
        self.cs = torch.tensor(cs3, device=dev)
        self.cell_offset = torch.tensor(coff.astype(np.int32), device=dev)
        self.total_cells = int(coff[-1])
        self.max_cells = int(ncell.max())
        s = N.Batch()
        s.dim = batch.dim
        s.n_systems = batch.n_systems
        s.n_atoms = batch.n
        s.total_cells = self.total_cells
        s.max_cells = self.max_cells
        s.sys_offset = batch.sys_offset.data_ptr()
        s.atom_sys = batch.atom_sys.data_ptr()
        s.box = batch.box.data_ptr()
        s.cell_offset = self.cell_offset.data_ptr()
        s.cells_per_side = self.cps.data_ptr()
        s.cell_size = self.cs.data_ptr()
        self.struct = s


@dataclasses.dataclass
class BatchNeighborList:
    """Dense lists of every system in the engine's tiled layout (see
    jmd_batch_nlist): entries of atom i (global row) are
    ``idx[(i//32)*ld*32 + k*32 + i%32]`` for ``k < count[i]``, global ids."""
    idx: torch.Tensor
    count: torch.Tensor
    reference_position: torch.Tensor
    error: torch.Tensor           # uint8 [1], PartitionErrorCode bits
    occupancy: torch.Tensor       # int32 [1], largest row found by the last build
    max_occupancy: int
    ld: int
    flag: torch.Tensor
    workspace: torch.Tensor
    batch: Batch
    grid: _Grid
    cutoff: float
    threshold_sq: float
    mask_self: bool

    def struct(self) -> N.BatchNList:
        s = N.BatchNList()
        s.cutoff_sq = float(np.float32(np.float32(self.cutoff) * np.float32(self.cutoff)))
        s.max_occupancy = self.max_occupancy
        s.ld = self.ld
        s.mask_self = 1 if self.mask_self else 0
        s.idx = self.idx.data_ptr()
        s.count = self.count.data_ptr()
        s.reference_position = self.reference_position.data_ptr()
        s.occupancy = self.occupancy.data_ptr()
        s.error_code = self.error.data_ptr()
        s.rebuild_flag = self.flag.data_ptr()
        s.workspace = self.workspace.data_ptr()
        s.workspace_bytes = self.workspace.numel()
        return s

    @property
    def did_buffer_overflow(self) -> bool:
        return bool(int(self.error.item()) & 3)

    def dense(self, b: int) -> np.ndarray:
        """System b's list as the reference's Dense ``[N_b, max_occupancy]``
        array of system-local ids padded with N_b (rows sorted; host copy)."""
        rows = self.batch.rows(b)
        n_b = rows.stop - rows.start
        i = torch.arange(rows.start, rows.stop, device=self.idx.device)
        k = torch.arange(self.max_occupancy, device=self.idx.device)
        pos = (i[:, None] // 32) * self.ld * 32 + k[None, :] * 32 + (i[:, None] % 32)
        ent = self.idx[pos.reshape(-1)].reshape(n_b, self.max_occupancy).long() - rows.start
        cnt = self.count[rows].long()
        ent = torch.where(k[None, :] < cnt[:, None], ent, torch.full_like(ent, n_b))
        out = ent.cpu().numpy()
        out.sort(axis=1)
        return out


class BatchNeighborListFns:
    """``allocate(batch)`` / ``update(position, nbrs)`` over a batch, the
    batched form of partition.neighbor_list (partition.py:801-1164): the list
    cutoff is r_cutoff + dr_threshold, capacity int(max_occupancy *
    capacity_multiplier + extra_capacity) (partition.py:1090-1104) shared by
    all systems, and update rebuilds (every system) when any atom moved more
    than dr_threshold / 2 since the last build."""

    def __init__(self, r_cutoff, dr_threshold=0.0, capacity_multiplier=1.25, mask_self=True):
        self.r_cutoff = float(r_cutoff)
        self.dr_threshold = float(dr_threshold)
        f32 = np.float32
        # float32 arithmetic of the reference's run (partition.py:880-884)
        self.cutoff = float(f32(f32(self.r_cutoff) + f32(self.dr_threshold)))
        self.capacity_multiplier = float(capacity_multiplier)
        self.mask_self = bool(mask_self)
        self.threshold_sq = float(f32((f32(self.dr_threshold) / f32(2)) ** 2)) \
            if self.dr_threshold > 0 else -1.0

    def _make(self, batch, grid, max_occ):
        dev = batch.device
        ld = ((max_occ + 7) // 8) * 8
        n_pad = ((batch.n + 31) // 32) * 32
        ws = N.lib().jmd_batch_nlist_workspace_bytes(ctypes.byref(grid.struct))
        return BatchNeighborList(
            idx=torch.empty(max(n_pad * ld, 1), dtype=torch.int32, device=dev),
            count=torch.zeros(max(batch.n, 1), dtype=torch.int32, device=dev),
            reference_position=torch.zeros((max(batch.n, 1), 4), dtype=torch.float32, device=dev),
            error=torch.zeros(1, dtype=torch.uint8, device=dev),
            occupancy=torch.zeros(1, dtype=torch.int32, device=dev),
            max_occupancy=int(max_occ), ld=int(ld),
            flag=torch.zeros(1, dtype=torch.int32, device=dev),
            workspace=torch.empty(ws, dtype=torch.uint8, device=dev),
            batch=batch, grid=grid, cutoff=self.cutoff, threshold_sq=self.threshold_sq,
            mask_self=self.mask_self)

    def _build(self, nb, position, gated=False):
        N.check(N.lib().jmd_batch_neighbor_list_build(ctypes.byref(nb.grid.struct),
                                                      ctypes.byref(nb.struct()),
                                                      position.data_ptr(), 1 if gated else 0,
                                                      N.stream_ptr()), 'batch_neighbor_list_build')

    def allocate(self, batch: Batch, extra_capacity: int = 0) -> BatchNeighborList:
        N.require_cuda(batch.position)
        grid = _Grid(batch, self.cutoff)
        # count pass: a first build at a generous width reports the largest row
        probe = self._make(batch, grid, 64)
        self._build(probe, batch.position)
        occ = int(probe.occupancy.item())
        if occ > probe.max_occupancy:
            probe = self._make(batch, grid, occ)
            self._build(probe, batch.position)
            occ = int(probe.occupancy.item())
        cap = int(np.float32(occ) * np.float32(self.capacity_multiplier) + extra_capacity)
        cap = max(1, min(cap, max(batch.sizes) - (1 if self.mask_self else 0)))
        nb = self._make(batch, grid, max(cap, 1))
        self._build(nb, batch.position)
        return nb

    def update(self, position: torch.Tensor, nbrs: BatchNeighborList) -> BatchNeighborList:
        L = N.lib()
        if self.threshold_sq < 0:
            self._build(nbrs, position)
            return nbrs
        N.check(L.jmd_batch_skin_check(ctypes.byref(nbrs.grid.struct), ctypes.byref(nbrs.struct()),
                                       position.data_ptr(), self.threshold_sq, N.stream_ptr()),
                'batch_skin_check')
        self._build(nbrs, position, gated=True)
        return nbrs


def neighbor_list(r_cutoff, dr_threshold=0.0, capacity_multiplier=1.25,
                  mask_self=True) -> BatchNeighborListFns:
    return BatchNeighborListFns(r_cutoff, dr_threshold, capacity_multiplier, mask_self)


class BatchPairEnergy:
    """The pair energy of a single-system ``energy.*_neighbor_list`` energy
    function (smap.PairNeighborListEnergy: its potential and parameters),
    evaluated on every system of a batch with the batch's species."""

    def __init__(self, energy_fn: smap.PairNeighborListEnergy):
        if not isinstance(energy_fn, smap.PairNeighborListEnergy):
            raise NotImplementedError('batched energies come from jax_md_gb300.energy '
                                      '*_neighbor_list energy functions')
        self.energy_fn = energy_fn

    def pair(self, batch: Batch, **dyn):
        """(species, jmd_pair) with the batch's species and any sigma /
        epsilon / alpha given as keywords (scalars or species matrices)."""
        dyn = dict(dyn)
        if batch.species is not None:
            dyn['species'] = batch.species
        species, pair = self.energy_fn._resolve(batch.R, dyn)
        return species, pair

    def forces(self, batch: Batch, nbrs: BatchNeighborList, out=None, energies=None,
               position=None, **dyn):
        """Forces of every system (``[N, 4]`` float4 rows) and, with
        ``energies`` (f64 ``[B]``), the per-system potential energies, at
        ``position`` (float4 rows; default the batch's)."""
        species, pair = self.pair(batch, **dyn)
        x = batch.position if position is None else position
        if out is None:
            out = torch.empty((batch.n, 4), dtype=torch.float32, device=batch.device)
        N.check(N.lib().jmd_batch_pair_forces(ctypes.byref(pair), ctypes.byref(nbrs.grid.struct),
                                              ctypes.byref(nbrs.struct()), x.data_ptr(),
                                              N.ptr(species), out.data_ptr(), N.ptr(energies),
                                              N.stream_ptr()), 'batch_pair_forces')
        return out

    def energy_fn_autograd(self, batch: Batch, nbrs: BatchNeighborList):
        """``E(R, sigma=None, epsilon=None) -> [B]`` per-system potential
        energies, differentiable with respect to R (``[N, dim]``) and to sigma /
        epsilon tensors that require grad (shared by every system)."""
        def fn(R, sigma=None, epsilon=None):
            dyn = {}
            if sigma is not None:
                dyn['sigma'] = sigma
            if epsilon is not None:
                dyn['epsilon'] = epsilon
            return _BatchEnergy.apply(R, _param_tensor(sigma), _param_tensor(epsilon),
                                      (self, batch, nbrs, dyn))
        return fn

    def energies(self, batch: Batch, nbrs: BatchNeighborList) -> torch.Tensor:
        e = torch.empty(batch.n_systems, dtype=torch.float64, device=batch.device)
        scratch = torch.empty((batch.n, 4), dtype=torch.float32, device=batch.device)
        self.forces(batch, nbrs, out=scratch, energies=e)
        return e


FIRE_DEFAULTS = dict(dt_start=0.1, dt_max=0.4, n_min=5, f_inc=1.1, f_dec=0.5, alpha_start=0.1,
                     f_alpha=0.99)


class BatchRunner:
    """Device state of a batch (momenta, forces, FIRE scalars per system) and
    the graph-replayed runners.  Unit mass unless ``mass`` is given (scalar).

    ``fire(n)`` / ``nve(n)`` run n steps of every system as one CUDA graph
    launch (recorded on first use of each n); ``minimize`` repeats FIRE
    chunks until every system's largest atom force norm is below f_tol."""

    def __init__(self, batch: Batch, neighbor_fns: BatchNeighborListFns, nbrs: BatchNeighborList,
                 energy: BatchPairEnergy, dt: float = 1e-3, mass: float = 1.0, **fire):
        self.batch, self.neighbor_fns, self.nbrs, self.energy = batch, neighbor_fns, nbrs, energy
        dev = batch.device
        n = max(batch.n, 1)
        self.momentum = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        self.force = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        self.fire_state = torch.zeros(8 * batch.n_systems, dtype=torch.float32, device=dev)
        self.done = torch.zeros(batch.n_systems, dtype=torch.int32, device=dev)
        self.n_done = torch.zeros(1, dtype=torch.int32, device=dev)
        self.dt = float(np.float32(dt))
        self.mass = float(mass)
        params = dict(FIRE_DEFAULTS)
        params.update({k: v for k, v in fire.items() if k in FIRE_DEFAULTS})
        self.fire_params = N.FireParams(*[float(np.float32(params[k])) for k in (
            'dt_start', 'dt_max', 'n_min', 'f_inc', 'f_dec', 'alpha_start', 'f_alpha')], 0.0)
        self.species, self.pair = energy.pair(batch)
        self.compute_forces()

    def struct(self) -> N.BatchSystem:
        s = N.BatchSystem()
        s.batch = self.nbrs.grid.struct
        s.nlist = self.nbrs.struct()
        s.pair = self.pair
        s.species = N.ptr(self.species)
        s.position = self.batch.position.data_ptr()
        s.momentum = self.momentum.data_ptr()
        s.force = self.force.data_ptr()
        s.mass = None
        s.mass_scalar = self.mass
        s.dt = self.dt
        s.threshold_sq = self.neighbor_fns.threshold_sq
        s.fire_state = self.fire_state.data_ptr()
        s.done = self.done.data_ptr()
        s.n_done = self.n_done.data_ptr()
        return s

    def compute_forces(self):
        self.neighbor_fns.update(self.batch.position, self.nbrs)
        self.energy.forces(self.batch, self.nbrs, out=self.force)
        return self.force

    def set_momenta(self, kT: float, seed: int = 0):
        """Gaussian momenta at temperature kT with each system's net momentum
        removed (simulate.py:141-165, per system)."""
        g = torch.Generator(device=self.batch.device).manual_seed(seed)
        d = self.batch.dim
        p = torch.randn((self.batch.n, d), generator=g, device=self.batch.device) * math.sqrt(
            kT * self.mass)
        for b in range(self.batch.n_systems):
            r = self.batch.rows(b)
            p[r] -= p[r].mean(0, keepdim=True)
        self.momentum.zero_()
        self.momentum[:, :d] = p

    def fire_init(self, f_tol: float = 0.0):
        self.fire_params.f_tol = float(np.float32(f_tol))
        N.check(N.lib().jmd_batch_fire_init(ctypes.byref(self.struct()),
                                            ctypes.byref(self.fire_params), N.stream_ptr()),
                'batch_fire_init')
        self.momentum.zero_()

    def fire(self, n_steps: int, use_graph: bool = True) -> int:
        N.check(N.lib().jmd_batch_fire_run(ctypes.byref(self.struct()),
                                           ctypes.byref(self.fire_params), int(n_steps),
                                           1 if use_graph else 0, N.stream_ptr()), 'batch_fire_run')
        return int(n_steps)

    def minimize(self, f_tol: float, max_steps: int, chunk: int = 200, use_graph=True) -> int:
        """FIRE from rest until every system has max |F_i| < f_tol (or
        max_steps); returns the number of steps run."""
        self.fire_init(f_tol)
        steps = 0
        while steps < max_steps:
            k = min(chunk, max_steps - steps)
            self.fire(k, use_graph)
            steps += k
            if int(self.n_done.item()) == self.batch.n_systems:
                break
        return steps

    def nve(self, n_steps: int, use_graph: bool = True):
        N.check(N.lib().jmd_batch_nve_run(ctypes.byref(self.struct()), int(n_steps),
                                          1 if use_graph else 0, N.stream_ptr()), 'batch_nve_run')

    def kinetic(self):
        """(kinetic energy [B] f64, largest atom force norm [B])."""
        ke = torch.empty(self.batch.n_systems, dtype=torch.float64, device=self.batch.device)
        fm = torch.empty(self.batch.n_systems, dtype=torch.float32, device=self.batch.device)
        N.check(N.lib().jmd_batch_kinetic_energy(ctypes.byref(self.nbrs.grid.struct),
                                                 self.momentum.data_ptr(), self.force.data_ptr(),
                                                 None, self.mass, ke.data_ptr(), fm.data_ptr(),
                                                 N.stream_ptr()), 'batch_kinetic_energy')
        return ke, fm

    def potential(self):
        return self.energy.energies(self.batch, self.nbrs)

    # ---------------------------------------------------------- Nose-Hoover
    def nvt_init(self, kT, chain_length: int = 5, chain_steps: int = 2, sy_steps: int = 3,
                 tau=None):
        """One Nose-Hoover chain per system at temperature kT (a scalar or one
        value per system), as simulate.nvt_nose_hoover's init_fn
        (simulate.py:625-637) for each system: chain masses kT tau^2, the first
        times the system's degrees of freedom, zero chain positions and
        momenta, the system's kinetic energy.  tau defaults to 100 dt."""
        self.nhc = _nhc_constants(self.dt, chain_length, chain_steps, sy_steps, tau)
        ke, _ = self.kinetic()
        self.chain = _chain_init(self.batch, ke, kT, self.nhc)
        self.p_scale = torch.ones(2 * self.batch.n_systems, dtype=torch.float64,
                                  device=self.batch.device)

    def nvt_struct(self) -> N.BatchNvt:
        if getattr(self, 'chain', None) is None:
            raise RuntimeError('call nvt_init first')
        v = N.BatchNvt()
        v.chain = self.nhc
        v.chain_state = self.chain.data_ptr()
        v.p_scale = self.p_scale.data_ptr()
        return v

    def nvt(self, n_steps: int, use_graph: bool = True):
        """n_steps of Nose-Hoover NVT of every system (simulate.py:649-667)."""
        N.check(N.lib().jmd_batch_nvt_run(ctypes.byref(self.struct()),
                                          ctypes.byref(self.nvt_struct()), int(n_steps),
                                          1 if use_graph else 0, N.stream_ptr()), 'batch_nvt_run')

    def nvt_invariant(self) -> torch.Tensor:
        """Per-system conserved quantity of the NVT run
        (simulate.nvt_nose_hoover_invariant, simulate.py:672-701), f64 [B]."""
        self.compute_forces()
        ke, _ = self.kinetic()
        c = self.chain
        M1 = self.nhc.chain_length
        dof = torch.tensor(self.batch.sizes, dtype=torch.float64,
                           device=c.device) * self.batch.dim
        kT = c[:, 65]
        xi, pxi, Q = c[:, :M1], c[:, 16:16 + M1], c[:, 32:32 + M1]
        E = self.potential() + ke
        E = E + pxi[:, 0] ** 2 / (2 * Q[:, 0]) + dof * kT * xi[:, 0]
        E = E + (pxi[:, 1:] ** 2 / (2 * Q[:, 1:])).sum(1) + kT * xi[:, 1:].sum(1)
        return E


def _nhc_constants(dt, chain_length, chain_steps, sy_steps, tau) -> N.Nhc:
    if not 2 <= int(chain_length) <= 16:
        raise ValueError('chain_length must be between 2 and 16')
    if int(sy_steps) not in (1, 3, 5, 7):
        raise ValueError('sy_steps must be 1, 3, 5 or 7')
    if int(chain_steps) < 1:
        raise ValueError('chain_steps must be >= 1')
    dt32 = float(np.float32(dt))
    c = N.Nhc()
    c.chain_length, c.chain_steps, c.sy_steps = int(chain_length), int(chain_steps), int(sy_steps)
    c.dof = 0
    c.dt = dt32
    c.tau = float(np.float32(dt32 * 100 if tau is None else tau))
    return c


def _chain_init(batch: 'Batch', ke: torch.Tensor, kT, nhc: N.Nhc) -> torch.Tensor:
    """[B, 66] f64 chain states (the layout of jmd_nhc_half_step) of a batch."""
    B, dev = batch.n_systems, batch.device
    kTs = torch.as_tensor(kT, dtype=torch.float64, device=dev).reshape(-1).expand(B)
    dof = torch.tensor(batch.sizes, dtype=torch.float64, device=dev) * batch.dim
    chain = torch.zeros((B, 66), dtype=torch.float64, device=dev)
    chain[:, 32:32 + nhc.chain_length] = (kTs * nhc.tau ** 2)[:, None]
    chain[:, 32] *= dof
    chain[:, 64] = ke
    chain[:, 65] = kTs
    return chain


def _system_struct(nbrs: BatchNeighborList, pair, species, x, p, f, mass, dt, threshold_sq):
    s = N.BatchSystem()
    s.batch = nbrs.grid.struct
    s.nlist = nbrs.struct()
    s.pair = pair
    s.species = N.ptr(species)
    s.position, s.momentum, s.force = x.data_ptr(), p.data_ptr(), f.data_ptr()
    s.mass = None
    s.mass_scalar = float(mass)
    s.dt = float(np.float32(dt))
    s.threshold_sq = threshold_sq
    return s


class _BatchEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, R, sigma, epsilon, cfg):
        energy, batch, nbrs, dyn = cfg
        dim = batch.dim
        x = torch.zeros((batch.n, 4), dtype=torch.float32, device=R.device)
        x[:, :dim] = R.detach()
        e = torch.empty(batch.n_systems, dtype=torch.float64, device=R.device)
        F = energy.forces(batch, nbrs, energies=e, position=x, **dyn)
        ctx.save_for_backward(sigma if sigma is not None else torch.empty(0),
                              epsilon if epsilon is not None else torch.empty(0))
        ctx.has = (sigma is not None, epsilon is not None)
        ctx.cfg, ctx.x, ctx.F = cfg, x, F
        return e

    @staticmethod
    def backward(ctx, gE):
        energy, batch, nbrs, dyn = ctx.cfg
        sigma, epsilon = ctx.saved_tensors
        sigma = sigma if ctx.has[0] else None
        epsilon = epsilon if ctx.has[1] else None
        w = gE.to(torch.float64).contiguous()
        gR = -ctx.F[:, :batch.dim] * w[batch.atom_sys.long()].to(torch.float32)[:, None]
        gs = ge = None
        if sigma is not None or epsilon is not None:
            species, pair = energy.pair(batch, **dyn)
            bins = torch.zeros(130, dtype=torch.float64, device=gE.device)
            N.check(N.lib().jmd_batch_energy_param_grad(
                ctypes.byref(pair), ctypes.byref(nbrs.grid.struct), ctypes.byref(nbrs.struct()),
                ctx.x.data_ptr(), N.ptr(species), w.data_ptr(), bins.data_ptr(), N.stream_ptr()),
                'batch_energy_param_grad')
            gs, ge = _bins_to_grads(bins, None, sigma, epsilon)
        return gR, gs, ge, None


class _Busy:
    """Marks a BatchTrajectory's buffers as holding a run awaiting backward."""

    def __init__(self, tr):
        self.tr = tr
        tr.busy = True

    def __del__(self):
        self.tr.busy = False


class _BatchTrajectoryFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, R0, P0, sigma, epsilon, cfg):
        tr, dyn = cfg
        if tr.busy:
            raise RuntimeError('this BatchTrajectory holds a recorded run whose backward has not '
                               'run yet (one buffer set per BatchTrajectory): call backward first '
                               'or use a second BatchTrajectory')
        bt, nb, dim = tr.batch, tr.nbrs, tr.batch.dim
        buf = tr.buffers()
        buf['x'].zero_()
        buf['p'].zero_()
        buf['x'][:, :dim] = torch.remainder(R0.detach(), bt.box[bt.atom_sys.long(), :dim])
        buf['p'][:, :dim] = P0.detach()
        tr.neighbor_fns._build(nb, buf['x'])
        species, pair = tr.energy.pair(bt, **dyn)
        tr.energy.forces(bt, nb, out=buf['f'], position=buf['x'], **dyn)
        sysd = _system_struct(nb, pair, species, buf['x'], buf['p'], buf['f'], tr.mass, tr.dt,
                              tr.neighbor_fns.threshold_sq)
        L = N.lib()
        segs = tr.segments
        for c, (s0, s1) in enumerate(segs):
            last = c == len(segs) - 1
            if not last:
                buf['ck_x'][c].copy_(buf['x'])
                buf['ck_p'][c].copy_(buf['p'])
                buf['ck_f'][c].copy_(buf['f'])
            N.check(L.jmd_batch_nve_run_recorded(ctypes.byref(sysd),
                                                 buf['traj'].data_ptr() if last else None,
                                                 s1 - s0, 1, 1, N.stream_ptr()),
                    'batch_nve_run_recorded')
        if nb.did_buffer_overflow:
            raise RuntimeError('a batched neighbour list overflowed during the trajectory; '
                               'allocate it with more capacity')
        if any(ctx.needs_input_grad[:4]):
            # the recorded trajectory must survive until backward; the lease is
            # released by backward or when the autograd graph is freed
            ctx.lease = _Busy(tr)
        ctx.cfg = (tr, sysd, species, buf)
        ctx.has = (sigma is not None, epsilon is not None)
        ctx.save_for_backward(sigma if sigma is not None else torch.empty(0),
                              epsilon if epsilon is not None else torch.empty(0))
        return buf['x'][:, :dim].clone(), buf['p'][:, :dim].clone()

    @staticmethod
    def backward(ctx, gx, gp):
        tr, sysd, species, buf = ctx.cfg
        sigma, epsilon = ctx.saved_tensors
        sigma = sigma if ctx.has[0] else None
        epsilon = epsilon if ctx.has[1] else None
        dim = tr.batch.dim
        buf['xbar'].zero_()
        buf['pbar'].zero_()
        if gx is not None:
            buf['xbar'][:, :dim] = gx
        if gp is not None:
            buf['pbar'][:, :dim] = gp
        want = sigma is not None or epsilon is not None
        bins = torch.zeros(130, dtype=torch.float64, device=buf['x'].device)
        L = N.lib()
        segs = tr.segments
        for c in reversed(range(len(segs))):
            s0, s1 = segs[c]
            last = c == len(segs) - 1
            if not last:
                buf['x'].copy_(buf['ck_x'][c])
                buf['p'].copy_(buf['ck_p'][c])
                buf['f'].copy_(buf['ck_f'][c])
                N.check(L.jmd_batch_nve_run_recorded(ctypes.byref(sysd), buf['traj'].data_ptr(),
                                                     s1 - s0, 1, 1, N.stream_ptr()),
                        'batch_nve_run_recorded')
            N.check(L.jmd_batch_nve_adjoint_segment(
                ctypes.byref(sysd), buf['traj'].data_ptr(), s1 - s0, 1 if last else 0,
                1 if c == 0 else 0, buf['xbar'].data_ptr(), buf['pbar'].data_ptr(),
                buf['rec'].data_ptr(), bins.data_ptr() if want else None, 1, N.stream_ptr()),
                'batch_nve_adjoint_segment')
        gs, ge = _bins_to_grads(bins, None, sigma, epsilon) if want else (None, None)
        ctx.lease = None
        return buf['xbar'][:, :dim].clone(), buf['pbar'][:, :dim].clone(), gs, ge, None


class BatchTrajectory:
    """``traj(R0, P0, sigma=None, epsilon=None) -> (x_n, p_n)``: n_steps of NVE
    of every system of a batch (``[N, dim]`` packed arrays), differentiable with
    respect to R0, P0 and sigma / epsilon shared by all systems, through the
    batched reverse Verlet pass (checkpointed every ``checkpoint_every`` steps;
    None keeps the whole trajectory when it fits a quarter of free memory).
    ``nbrs`` is rebuilt in place.  Unit mass unless ``mass`` is given.  One
    set of device buffers: a forward pass that records for backward must be
    followed by its backward before the next one (a second call raises)."""

    def __init__(self, batch: Batch, neighbor_fns: BatchNeighborListFns, nbrs: BatchNeighborList,
                 energy: BatchPairEnergy, dt: float, n_steps: int, checkpoint_every=None,
                 mass: float = 1.0):
        if int(n_steps) < 1:
            raise ValueError('n_steps must be >= 1')
        self.batch, self.neighbor_fns, self.nbrs, self.energy = batch, neighbor_fns, nbrs, energy
        self.dt, self.n_steps, self.mass = float(dt), int(n_steps), float(mass)
        n = max(batch.n, 1)
        if checkpoint_every is None:
            free, _ = torch.cuda.mem_get_info()
            k = int(free // 4 // (16 * n)) - 1
        else:
            k = int(checkpoint_every)
        k = max(1, min(k, self.n_steps))
        self.segments = [(s0, min(s0 + k, self.n_steps)) for s0 in range(0, self.n_steps, k)]
        self.k = k
        self._buf = None
        self.busy = False

    def buffers(self):
        if self._buf is None:
            n, dev = max(self.batch.n, 1), self.batch.device
            f4 = lambda *s: torch.zeros(s + (n, 4), dtype=torch.float32, device=dev)
            ns = len(self.segments)
            self._buf = dict(x=f4(), p=f4(), f=f4(), traj=f4(self.k + 1), ck_x=f4(ns), ck_p=f4(ns),
                             ck_f=f4(ns), xbar=f4(), pbar=f4(),
                             rec=torch.zeros((2 * n, 4), dtype=torch.float32, device=dev))
        return self._buf

    def __call__(self, R0, P0, sigma=None, epsilon=None):
        dyn = {}
        if sigma is not None:
            dyn['sigma'] = sigma
        if epsilon is not None:
            dyn['epsilon'] = epsilon
        return _BatchTrajectoryFn.apply(R0, P0, _param_tensor(sigma), _param_tensor(epsilon),
                                        (self, dyn))


# Reverse pass of batched Nose-Hoover NVT: the single-system recurrence
# (adjoint._NvtTrajectoryFn) with every scalar of it per system.  Step k
# records x_k, p_k, the chain before each half step, the scales s1, s2 and
# r = p after the Verlet step; backward, with p-bar, chain-momentum and KE
# cotangents per system:
#     sbar2_b = sum_{i in b} pbar_i . r_i;  rbar = s2 pbar;
#     (pxibar', kebar) = J_H^T(pxibar, sbar2);  rbar += kebar r / m
#     xbar += VJP(x_{k+1}, h (rbar + qbar_{k+1}))
#     qbar = rbar + (dt/m) xbar;  sbar1_b = sum qbar . p_k;  pbar = s1 qbar
#     (pxibar, kebar) = J_H^T(pxibar', sbar1);  pbar += kebar p_k / m
# and finally xbar += VJP(x_0, h qbar_0).
class _BatchNvtTrajectoryFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, R0, P0, sigma, epsilon, cfg):
        tr, dyn = cfg
        bt, nb, dim = tr.batch, tr.nbrs, tr.batch.dim
        n, dev, B = max(bt.n, 1), bt.device, bt.n_systems
        f4 = lambda: torch.zeros((n, 4), dtype=torch.float32, device=dev)
        x, p, f = f4(), f4(), f4()
        x[:, :dim] = torch.remainder(R0.detach(), bt.box[bt.atom_sys.long(), :dim])
        p[:, :dim] = P0.detach()
        tr.neighbor_fns._build(nb, x)
        species, pair = tr.energy.pair(bt, **dyn)
        tr.energy.forces(bt, nb, out=f, position=x, **dyn)
        sysd = _system_struct(nb, pair, species, x, p, f, tr.mass, tr.dt,
                              tr.neighbor_fns.threshold_sq)
        L = N.lib()
        ke = torch.empty(B, dtype=torch.float64, device=dev)
        N.check(L.jmd_batch_kinetic_energy(ctypes.byref(nb.grid.struct), p.data_ptr(), None, None,
                                           tr.mass, ke.data_ptr(), None, N.stream_ptr()),
                'batch_kinetic_energy')
        chain = _chain_init(bt, ke, tr.kT, tr.nhc)
        nvt = N.BatchNvt()
        nvt.chain, nvt.chain_state, nvt.p_scale = tr.nhc, chain.data_ptr(), None
        steps = tr.n_steps
        s1 = torch.empty((steps, B), dtype=torch.float64, device=dev)
        s2 = torch.empty_like(s1)
        ke2 = torch.empty_like(s1)

        def half(update_mass, measure, scale, ke_out):
            N.check(L.jmd_batch_nhc_half_step(ctypes.byref(nb.grid.struct), ctypes.byref(nvt),
                                              p.data_ptr(), None, tr.mass, update_mass, measure,
                                              scale.data_ptr(), N.ptr(ke_out), N.stream_ptr()),
                    'batch_nhc_half_step')

        def run_steps(k0, count, tape):
            """Steps k0 .. k0 + count - 1 on (x, p, f, chain); with ``tape``
            each step's (x_k, p_k, chain_a, r, chain_b) is appended."""
            for k in range(k0, k0 + count):
                if tape is not None:
                    x_k, p_k, chain_a = x[:, :dim].clone(), p[:, :dim].clone(), chain.clone()
                half(1, 0, s1[k], None)
                N.check(L.jmd_batch_nve_run(ctypes.byref(sysd), 1, 0, N.stream_ptr()),
                        'batch_nve_run')
                if tape is not None:
                    r, chain_b = p[:, :dim].clone(), chain.clone()
                half(0, 1, s2[k], ke2[k])
                if tape is not None:
                    tape.append((x_k, p_k, chain_a, r, chain_b))

        seg = tr.segment_length(n, dim)
        tape, checkpoints = [], []
        if seg >= steps:
            run_steps(0, steps, tape)
        else:
            for k0 in range(0, steps, seg):
                # a segment starts from a fresh list, so its replay in the
                # reverse pass repeats it bit for bit
                tr.neighbor_fns._build(nb, x)
                checkpoints.append((x.clone(), p.clone(), f.clone(), chain.clone()))
                run_steps(k0, min(seg, steps - k0), None)
        if nb.did_buffer_overflow:
            raise RuntimeError('a batched neighbour list overflowed during the trajectory; '
                               'allocate it with more capacity')

        def replay(si, k0, count):
            ck = checkpoints[si]
            for buf, v in zip((x, p, f, chain), ck):
                buf.copy_(v)
            tr.neighbor_fns._build(nb, x)
            out = []
            run_steps(k0, count, out)
            return out
        ctx.cfg = (tr, species, pair, tape, x[:, :dim].clone(), s1, s2, ke2,
                   (seg, checkpoints, replay, (sysd, x, p, f, chain)))
        ctx.has = (sigma is not None, epsilon is not None)
        ctx.save_for_backward(sigma if sigma is not None else torch.empty(0),
                              epsilon if epsilon is not None else torch.empty(0))
        return x[:, :dim].clone(), p[:, :dim].clone()

    @staticmethod
    def backward(ctx, gx, gp):
        tr, species, pair, full_tape, x_n, s1, s2, ke2, (seg, checkpoints, replay, _) = ctx.cfg
        sigma, epsilon = ctx.saved_tensors
        sigma = sigma if ctx.has[0] else None
        epsilon = epsilon if ctx.has[1] else None
        bt, nb, dim = tr.batch, tr.nbrs, tr.batch.dim
        n, dev, B = max(bt.n, 1), bt.device, bt.n_systems
        sys_of = bt.atom_sys.long()
        dt = float(np.float32(tr.dt))
        h = float(np.float32(dt / 2))
        inv_m = 1.0 / tr.mass
        xbar = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        if gx is not None:
            xbar[:, :dim] += gx
        pbar = torch.zeros((n, dim), dtype=torch.float32, device=dev)
        if gp is not None:
            pbar += gp
        want = sigma is not None or epsilon is not None
        bins = torch.zeros(130, dtype=torch.float64, device=dev)
        pxi = torch.zeros((B, 16), dtype=torch.float64, device=dev)
        pxi1 = torch.zeros_like(pxi)
        kebar = torch.zeros(B, dtype=torch.float64, device=dev)
        x4 = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        lam4 = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        rec = torch.zeros((2 * n, 4), dtype=torch.float32, device=dev)
        L = N.lib()
        g = ctypes.byref(nb.grid.struct)
        rbar = torch.empty((n, dim), dtype=torch.float32, device=dev)
        qbar = torch.empty((n, dim), dtype=torch.float32, device=dev)
        pend = torch.empty((n, dim), dtype=torch.float32, device=dev)
        sbar1 = torch.empty(B, dtype=torch.float64, device=dev)
        sbar2 = torch.empty(B, dtype=torch.float64, device=dev)
        pbar = pbar.contiguous()
        s_ptr = lambda t, k: t.data_ptr() + k * t.stride(0) * t.element_size()  # row k of [steps, B]

        def chain_vjp(chain_in, ke, update_mass, cot_p, cot_s, out_p):
            N.check(L.jmd_batch_nhc_half_step_vjp(
                ctypes.byref(nb.grid.struct), ctypes.byref(tr.nhc), chain_in.data_ptr(),
                ke.data_ptr(), update_mass, cot_p.data_ptr(), cot_s.data_ptr(), out_p.data_ptr(),
                kebar.data_ptr(), N.stream_ptr()), 'batch_nhc_half_step_vjp')

        def vjp_at(x):  # the cotangent is in lam4
            x4[:, :dim] = x
            tr.neighbor_fns.update(x4, nb)
            N.check(L.jmd_batch_pair_force_vjp(
                ctypes.byref(pair), ctypes.byref(nb.grid.struct), ctypes.byref(nb.struct()),
                x4.data_ptr(), lam4.data_ptr(), N.ptr(species), 1.0, xbar.data_ptr(),
                bins.data_ptr() if want else None, rec.data_ptr(), N.stream_ptr()),
                'batch_pair_force_vjp')

        # one reverse step: fused per-system reductions and cotangent updates
        # (jmd_batch_dot_per_system, jmd_batch_nvt_adjoint_update) around the
        # chain VJPs and the force VJP
        pending = None
        upd = L.jmd_batch_nvt_adjoint_update

        def reverse_step(k, entry, x1, pending):
            x_k, p_k, chain_a, r, chain_b = entry
            N.check(L.jmd_batch_dot_per_system(g, pbar.data_ptr(), dim, r.data_ptr(), r.stride(0),
                                               sbar2.data_ptr(), N.stream_ptr()), 'dot')
            chain_vjp(chain_b, ke2[k], 0, pxi, sbar2, pxi1)
            # rbar = pbar s2 + kebar r / m ; lam4 = h (rbar + pending)
            N.check(upd(g, 0, pbar.data_ptr(), r.data_ptr(), r.stride(0), s_ptr(s2, k),
                        kebar.data_ptr(), inv_m, h, N.ptr(pending), rbar.data_ptr(),
                        lam4.data_ptr(), None, N.stream_ptr()), 'nvt adjoint pre')
            vjp_at(x1)
            # qbar = rbar + (dt / m) xbar ; sbar1 = sum qbar . p_k
            N.check(upd(g, 1, rbar.data_ptr(), p_k.data_ptr(), p_k.stride(0), None, None, inv_m,
                        dt * inv_m, xbar.data_ptr(), qbar.data_ptr(), None, sbar1.data_ptr(),
                        N.stream_ptr()), 'nvt adjoint post')
            chain_vjp(chain_a, chain_a[:, 64].contiguous(), 1, pxi1, sbar1, pxi)
            # pbar = qbar s1 + kebar p_k / m
            N.check(upd(g, 2, qbar.data_ptr(), p_k.data_ptr(), p_k.stride(0), s_ptr(s1, k),
                        kebar.data_ptr(), inv_m, 0.0, None, pbar.data_ptr(), None, None,
                        N.stream_ptr()), 'nvt adjoint pbar')
            pend.copy_(qbar)
            return pend

        # segments in reverse; a checkpointed segment is replayed from its
        # checkpoint to rebuild its tape
        steps = tr.n_steps
        segs = ([(k0, min(seg, steps - k0)) for k0 in range(0, steps, seg)] if checkpoints
                else [(0, steps)])
        x_end = x_n
        for si in range(len(segs) - 1, -1, -1):
            k0, count = segs[si]
            tape = replay(si, k0, count) if checkpoints else full_tape
            for kk in range(len(tape) - 1, -1, -1):
                x1 = tape[kk + 1][0] if kk + 1 < len(tape) else x_end
                pending = reverse_step(k0 + kk, tape[kk], x1, pending)
            x_end = tape[0][0]
            del tape
        lam4[:, :dim] = h * pending
        vjp_at(x_end)
        gs, ge = _bins_to_grads(bins, None, sigma, epsilon) if want else (None, None)
        return xbar[:, :dim].clone(), pbar.contiguous(), gs, ge, None


class BatchNvtTrajectory:
    """``traj(R0, P0, sigma=None, epsilon=None) -> (x_n, p_n)``: n_steps of
    Nose-Hoover NVT of every system of a batch (a fresh chain per system at
    kT, simulate.nvt_nose_hoover), differentiable with respect to R0, P0 and
    sigma / epsilon shared by all systems.  Every step is recorded (positions,
    momenta and the chains) while that fits a quarter of the free device
    memory (``checkpoint_every=None``); otherwise, or with
    ``checkpoint_every=k``, (x, p, F, chains) are kept every k steps and each
    segment is replayed from its checkpoint (and a fresh list) before its
    reverse pass.  ``nbrs`` is rebuilt in place.  Unit mass unless ``mass``
    is given."""

    def __init__(self, batch: Batch, neighbor_fns: BatchNeighborListFns, nbrs: BatchNeighborList,
                 energy: BatchPairEnergy, dt: float, kT, n_steps: int, chain_length: int = 5,
                 chain_steps: int = 2, sy_steps: int = 3, tau=None, mass: float = 1.0,
                 checkpoint_every=None):
        if int(n_steps) < 1:
            raise ValueError('n_steps must be >= 1')
        if not 2 <= int(chain_length) <= 7:
            raise NotImplementedError('the chain adjoint supports chain_length 2..7')
        self.batch, self.neighbor_fns, self.nbrs, self.energy = batch, neighbor_fns, nbrs, energy
        self.dt, self.kT, self.n_steps, self.mass = float(dt), kT, int(n_steps), float(mass)
        self.nhc = _nhc_constants(dt, chain_length, chain_steps, sy_steps, tau)
        self.checkpoint_every = checkpoint_every

    def segment_length(self, n: int, dim: int) -> int:
        """Steps per recorded segment: ``checkpoint_every``, or all steps when
        their record (x, p, r per atom and two chains per system per step)
        fits a quarter of the free device memory."""
        if self.checkpoint_every is not None:
            return max(1, min(int(self.checkpoint_every), self.n_steps))
        per_step = 3 * n * dim * 4 + 2 * self.batch.n_systems * 66 * 8
        free = torch.cuda.mem_get_info(self.batch.device)[0] if self.batch.device.type == 'cuda' \
            else 1 << 34
        fit = max(1, int((free // 4) // max(per_step, 1)))
        return self.n_steps if fit >= self.n_steps else fit

    def __call__(self, R0, P0, sigma=None, epsilon=None):
        dyn = {}
        if sigma is not None:
            dyn['sigma'] = sigma
        if epsilon is not None:
            dyn['epsilon'] = epsilon
        return _BatchNvtTrajectoryFn.apply(R0, P0, _param_tensor(sigma), _param_tensor(epsilon),
                                           (self, dyn))


FORCE_BLOCKS = (64, 128, 256)
FIRE_THREADS = (256, 512, 1024)


def set_launch(force_block: int = 128, fire_threads: int = 1024):
    """Launch shapes of the batched kernels (jmd_batch_set_launch)."""
    N.check(N.lib().jmd_batch_set_launch(int(force_block), int(fire_threads)), 'batch_set_launch')


def autotune(runner: BatchRunner, steps: int = 20) -> dict:
    """Times ``steps`` graph-replayed FIRE steps of the runner's batch for every
    launch shape (force CTA size x FIRE-update threads per system), each from
    the same starting state, keeps the fastest and returns the timings (ms).
    The runner's state is restored afterwards."""
    bt, nb = runner.batch, runner.nbrs
    saved = [t.clone() for t in (bt.position, runner.momentum, runner.force, runner.fire_state,
                                 runner.done, runner.n_done)]

    def restore():
        for t, v in zip((bt.position, runner.momentum, runner.force, runner.fire_state,
                         runner.done, runner.n_done), saved):
            t.copy_(v)
        runner.neighbor_fns._build(nb, bt.position)

    times = {}
    stream = torch.cuda.current_stream(bt.device)
    for fb in FORCE_BLOCKS:
        for ft in FIRE_THREADS:
            set_launch(fb, ft)
            restore()
            runner.fire(steps)                      # records this shape's graph
            restore()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            runner.fire(steps)
            e1.record(stream)
            torch.cuda.synchronize()
            times[(fb, ft)] = e0.elapsed_time(e1)
    best = min(times, key=times.get)
    set_launch(*best)
    restore()
    return {'best': best, 'ms': {f'{k[0]}x{k[1]}': v for k, v in times.items()}}


# ------------------------------------------------------------------ ranks --
def partition_systems(sizes: Sequence[int], n_ranks: int) -> List[List[int]]:
    """Systems of an ensemble split across ``n_ranks`` processes, one GPU
    each.  The systems are independent units: each rank packs and runs its
    own share with no exchange during the run (weak scaling).  Largest
    system first onto the least-loaded rank (load = atoms; ties to the lower
    rank); each rank's list is in ascending system order.  Deterministic, so
    every rank computes the same split from the same sizes."""
    if int(n_ranks) < 1:
        raise ValueError('n_ranks must be >= 1')
    sizes = [int(s) for s in sizes]
    if any(s < 0 for s in sizes):
        raise ValueError('system sizes must be >= 0')
    load = [0] * int(n_ranks)
    out: List[List[int]] = [[] for _ in range(int(n_ranks))]
    for b in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(len(load)), key=lambda k: (load[k], k))
        out[r].append(b)
        load[r] += sizes[b]
    return [sorted(x) for x in out]


def reduce_ensemble(local_sum: torch.Tensor, n_local: int, grads: Sequence[torch.Tensor] = (),
                    group=None):
    """Mean over every rank's systems of a per-system quantity, and of its
    gradients with respect to parameters shared by all systems.  Each rank
    passes the sum over its own systems (a scalar tensor), how many systems
    that is, and the gradients of that sum; one all-reduce (SUM) of
    [sum, count, grads...] in f64 gives (mean, [gradient of the mean]) on
    every rank.  Without an initialised process group it is the
    single-process mean."""
    dev = local_sum.device
    parts = [local_sum.detach().reshape(1).to(torch.float64),
             torch.tensor([float(n_local)], dtype=torch.float64, device=dev)]
    parts += [g.detach().reshape(-1).to(device=dev, dtype=torch.float64) for g in grads]
    buf = torch.cat(parts)
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    count = buf[1]
    if float(count) <= 0:
        raise ValueError('the ensemble has no systems')
    out, off = [], 2
    for g in grads:
        k = g.numel()
        out.append((buf[off:off + k] / count).reshape(g.shape).to(g.dtype))
        off += k
    return buf[0] / count, out
