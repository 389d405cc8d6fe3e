"""Pair maps over neighbour lists (jax_md/smap.py) backed by the CUDA kernels.

``pair_neighbor_list(fn, displacement, species=None, reduce_axis=None,
ignore_unused_parameters=False, **kwargs)`` keeps the reference signature
(smap.py:856-979) and returns ``fn_mapped(R, neighbor, **dynamic_kwargs)``.
``fn`` must be one of the potentials in ``jax_md_gb300.energy`` (there is
no kernel for an arbitrary Python function, and no CPU fallback).
Parameters are scalars or, with ``species``, [S, S] matrices (smap.py:778-823).

The returned energy is float32 like the reference (an f64 sum cast back,
util.high_precision_sum); it is differentiable with respect to ``R`` (the
backward pass returns -F from the same kernel launch).  The object also
exposes ``forces``, ``energy_f64`` and ``compute`` for the integrators.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np
import torch

from . import _native as N
from . import partition
from . import space as _space


def _param_matrix(v, n_species: int, name: str):
    """Scalar or [S, S] species matrix -> nested list [8][8] of floats."""
    if isinstance(v, torch.Tensor):
        v = v.detach().cpu().double().numpy()
    a = np.asarray(v, np.float64)
    out = np.zeros((N.MAX_SPECIES, N.MAX_SPECIES))
    if a.ndim == 0:
        out[:, :] = float(a)
        return out
    if a.ndim == 1:
        raise NotImplementedError(f'per-particle parameter arrays ({name}) are not supported by the '
                                  'pair kernels; use scalars or species matrices')
    if a.ndim == 2:
        if n_species == 0:
            raise NotImplementedError(f'an [N, N] parameter matrix ({name}) needs species; per-pair '
                                      'matrices are not supported by the pair kernels')
        S = a.shape[0]
        if S > N.MAX_SPECIES:
            raise ValueError(f'at most {N.MAX_SPECIES} species are supported')
        out[:S, :S] = a
        return out
    raise ValueError(f'Parameter array must be either a scalar, a vector, or a matrix. '
                     f'Found ndim={a.ndim}.')


def _host(v):
    return v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)


def _per_particle_table(params: dict):
    """Per-particle [N] parameter arrays as a species table.

    The reference combines a per-particle array as 0.5 (p_i + p_j)
    (smap.py:833-838 with :704-713).  Atoms whose per-particle values are all
    equal share a species, and the species matrices hold the pairwise means
    (in float32, as the reference computes them), so the species kernels give
    exactly the reference's pair parameters.  Returns (params with the
    matrices, species [N] int32, number of species), or None when no
    parameter is per-particle.  At most 8 distinct value combinations."""
    keys = [k for k in ('sigma', 'epsilon', 'alpha')
            if params.get(k) is not None and np.ndim(_host(params[k])) == 1]
    if not keys:
        return None
    if any(params.get(k) is not None and np.ndim(_host(params[k])) == 2
           for k in ('sigma', 'epsilon', 'alpha')):
        raise NotImplementedError('per-particle parameter arrays together with species matrices '
                                  'are not supported by the pair kernels')
    cols = [_host(params[k]).astype(np.float32) for k in keys]
    n = cols[0].shape[0]
    if any(c.shape[0] != n for c in cols):
        raise ValueError('per-particle parameter arrays must have one entry per atom')
    uniq, inv = np.unique(np.stack(cols, 1), axis=0, return_inverse=True)
    if len(uniq) > N.MAX_SPECIES:
        # continuous per-particle values: the generic pair kernels combine
        # them per pair (jmd_pair.particle_sigma / particle_epsilon)
        if 'alpha' in keys:
            raise NotImplementedError('per-particle alpha arrays with more than '
                                      f'{N.MAX_SPECIES} distinct values are not supported by the '
                                      'pair kernels')
        return _Continuous({k: c for k, c in zip(keys, cols)})
    out = dict(params)
    for c, k in enumerate(keys):
        v = uniq[:, c]
        out[k] = (np.float32(0.5) * (v[:, None] + v[None, :])).astype(np.float64)
    return out, np.asarray(inv).reshape(-1).astype(np.int32), len(uniq)


class _Continuous:
    """Per-particle sigma / epsilon arrays with more distinct values than the
    species table holds: passed to the kernels as per-atom arrays."""

    def __init__(self, host: dict):
        self.host = host          # name -> float32 [N]
        self.device = {}          # (name, device) -> tensor

    @property
    def n(self):
        return next(iter(self.host.values())).shape[0]

    def tensor(self, name, device):
        key = (name, str(device))
        t = self.device.get(key)
        if t is None:
            t = torch.as_tensor(self.host[name]).to(device=device, dtype=torch.float32).contiguous()
            self.device[key] = t
        return t


def make_pair_struct(fn, params: dict, n_species: int) -> N.Pair:
    p = N.Pair()
    p.kind = fn.kind
    p.n_species = n_species
    p.per_pair_cutoff = 1 if params.get('per_pair_cutoff', False) else 0
    rc = fn.r_cutoff
    p.r_cutoff = float(np.float32(rc)) if np.isfinite(rc) else 3.0e38
    ro = fn.r_onset
    p.r_onset = float(np.float32(ro)) if np.isfinite(ro) else p.r_cutoff
    # the elementwise functions' own defaults (energy.py:125-131, 246-250, 346-352)
    defaults = {'sigma': 1.0, 'epsilon': 5.0, 'alpha': 5.0} if fn.kind == N.MORSE else \
        {'sigma': 1.0, 'epsilon': 1.0, 'alpha': 2.0}
    for key, default in defaults.items():
        m = _param_matrix(params.get(key, default), n_species, key)
        arr = getattr(p, key)
        for a in range(N.MAX_SPECIES):
            for b in range(N.MAX_SPECIES):
                arr[a][b] = float(m[a, b])
    return p


def _param_tensor(v):
    if isinstance(v, torch.Tensor) and v.requires_grad and v.dim() == 1:
        raise NotImplementedError('gradients with respect to per-particle parameter arrays are not '
                                  'available (the kernels accumulate them per species pair)')
    return v if isinstance(v, torch.Tensor) and v.requires_grad else None


def _bins_to_grads(bins, pair, sigma, epsilon):
    """Maps the kernel's gradient bins onto the shapes of sigma / epsilon.

    bins: [130] f64 = d/d sigma[a][b] (0..63), d/d epsilon[a][b] (64..127) and
    the global cutoff scale max(sigma) (128), credited to the largest sigma
    entry as jax.grad does through jnp.max (energy.py:319-320)."""
    out = []
    for v, off in ((sigma, 0), (epsilon, 64)):
        if v is None:
            out.append(None)
            continue
        if v.dim() == 0:
            g = bins[off:off + 1].sum()
            if off == 0:
                g = g + bins[128]
        else:
            S = v.shape[0]
            g = bins[off:off + 64].reshape(8, 8)[:S, :S].clone()
            if off == 0:
                flat = torch.argmax(v.detach().reshape(-1))
                g.reshape(-1)[flat] += bins[128]
        out.append(g.to(v.dtype))
    return out


class _ForceFn(torch.autograd.Function):
    """F(R; sigma, epsilon) with a backward pass through the VJP kernel."""

    @staticmethod
    def forward(ctx, R, sigma, epsilon, owner, neighbor, dynamic):
        F = owner.forces(R.detach(), neighbor, **dynamic)
        ctx.save_for_backward(R, sigma if sigma is not None else torch.empty(0),
                              epsilon if epsilon is not None else torch.empty(0))
        ctx.owner, ctx.neighbor, ctx.dynamic = owner, neighbor, dynamic
        ctx.has = (sigma is not None, epsilon is not None)
        return F

    @staticmethod
    def backward(ctx, lam):
        R, sigma, epsilon = ctx.saved_tensors
        sigma = sigma if ctx.has[0] else None
        epsilon = epsilon if ctx.has[1] else None
        gR, bins, _ = ctx.owner.force_vjp(R.detach(), ctx.neighbor, lam.contiguous(), **ctx.dynamic)
        gs, ge = _bins_to_grads(bins, None, sigma, epsilon)
        return gR.to(R.dtype), gs, ge, None, None, None


class _EnergyFn(torch.autograd.Function):
    """E(R; sigma, epsilon); dE/dR = -F is itself differentiable (through _ForceFn)."""

    @staticmethod
    def forward(ctx, R, sigma, epsilon, owner, neighbor, dynamic):
        E = owner.energy_f64(R.detach(), neighbor, **dynamic)
        ctx.save_for_backward(R, sigma if sigma is not None else torch.empty(0),
                              epsilon if epsilon is not None else torch.empty(0))
        ctx.owner, ctx.neighbor, ctx.dynamic = owner, neighbor, dynamic
        ctx.has = (sigma is not None, epsilon is not None)
        return E.to(R.dtype)

    @staticmethod
    def backward(ctx, gE):
        R, sigma, epsilon = ctx.saved_tensors
        sigma = sigma if ctx.has[0] else None
        epsilon = epsilon if ctx.has[1] else None
        F = _ForceFn.apply(R, sigma, epsilon, ctx.owner, ctx.neighbor, ctx.dynamic)
        gR = -F * gE.to(F.dtype)
        gs = ge = None
        if sigma is not None or epsilon is not None:
            bins = ctx.owner.energy_param_grad(R.detach(), ctx.neighbor, **ctx.dynamic)
            gs, ge = _bins_to_grads(bins, None, sigma, epsilon)
            gs = gs * gE if gs is not None else None
            ge = ge * gE if ge is not None else None
        return gR, gs, ge, None, None, None


class PairNeighborListEnergy:
    """fn_mapped of smap.pair_neighbor_list, bound to the CUDA kernels."""

    def __init__(self, fn, displacement_or_metric, species, reduce_axis, ignore_unused_parameters,
                 params):
        if not hasattr(fn, 'kind'):
            raise NotImplementedError('pair_neighbor_list needs a potential from '
                                      'jax_md_gb300.energy (lennard_jones, soft_sphere, morse or '
                                      'their multiplicative_isotropic_cutoff); there is no kernel for '
                                      f'{fn!r}')
        self.fn = fn
        self.geometry = _space.geometry_of(displacement_or_metric)
        self.species = species
        self.reduce_axis = reduce_axis
        self.ignore_unused_parameters = ignore_unused_parameters
        self.params = dict(params)
        # per-particle arrays given here are read once, as the reference's
        # closure captures them
        self._pp_static = _per_particle_table(self.params)
        self._pp_species = {}
        if reduce_axis is not None and tuple(reduce_axis) not in ((1,), (0, 1)):
            raise NotImplementedError('reduce_axis must be None, (1,) or (0, 1) for the pair kernels')

    # -- plumbing ---------------------------------------------------------
    def has_particle_arrays(self) -> bool:
        """Per-particle parameter arrays too varied for the species table:
        only the generic pair kernels take them (not the device engine)."""
        return isinstance(self._pp_static, _Continuous)

    def _resolve(self, R, dynamic):
        species = dynamic.get('species', self.species)
        params = dict(self.params)
        overridden = False
        for k in ('sigma', 'epsilon', 'alpha'):
            if k in dynamic:
                params[k] = dynamic[k]
                overridden = True
        pp = _per_particle_table(params) if overridden else self._pp_static
        if isinstance(pp, _Continuous):
            if species is not None and not isinstance(species, int):
                raise NotImplementedError('per-particle parameter arrays together with a species '
                                          'array are not supported by the pair kernels')
            if pp.n != R.shape[0]:
                raise ValueError('per-particle parameter arrays must have one entry per atom')
            scal = dict(params)
            for k, v in pp.host.items():
                # the table's scalar entry: max sigma (the cutoff scale), or
                # any epsilon (replaced per pair)
                scal[k] = float(np.max(v)) if k == 'sigma' else 1.0
            pair = make_pair_struct(self.fn, scal, 0)
            if 'sigma' in pp.host:
                pair.particle_sigma = pp.tensor('sigma', R.device).data_ptr()
            if 'epsilon' in pp.host:
                pair.particle_epsilon = pp.tensor('epsilon', R.device).data_ptr()
            # keep the device arrays alive past the asynchronous launch
            self._pp_live = pp
            return None, pair
        if pp is not None:
            if species is not None and not isinstance(species, int):
                raise NotImplementedError('per-particle parameter arrays together with a species '
                                          'array are not supported by the pair kernels')
            params, sp_host, S = pp
            if len(sp_host) != R.shape[0]:
                raise ValueError('per-particle parameter arrays must have one entry per atom')
            species = self._pp_species.get(R.device) if not overridden else None
            if species is None:
                species = torch.as_tensor(sp_host).to(device=R.device, dtype=torch.int32)
                if not overridden:
                    self._pp_species = {R.device: species}
            return species, make_pair_struct(self.fn, params, S)
        S = 0
        for k in ('sigma', 'epsilon', 'alpha'):
            v = params.get(k)
            if v is not None and np.ndim(v.detach().cpu() if isinstance(v, torch.Tensor) else v) == 2:
                S = max(S, int(v.shape[0]) if hasattr(v, 'shape') else len(v))
        if S:
            if species is None or isinstance(species, int):
                raise NotImplementedError('species matrices need a per-atom species array')
            if not isinstance(species, torch.Tensor):
                species = torch.as_tensor(np.asarray(species))
            species = species.to(device=R.device, dtype=torch.int32).contiguous()
        else:
            species = None
        return species, make_pair_struct(self.fn, params, S)

    def launch(self, R, neighbor, force=None, energy=None, per_atom=None, virial=None, **dynamic):
        R, rs = partition._rows(R)
        n, dim = R.shape
        species, pair = self._resolve(R, dynamic)
        sp = self.geometry.space(dim, dynamic.get('box'), dynamic.get('new_box'))
        fmt = {partition.Dense: N.DENSE, partition.Sparse: N.SPARSE,
               partition.OrderedSparse: N.ORDERED_SPARSE}[neighbor.format]
        idx = neighbor.idx
        if idx.dtype != torch.int32:
            idx = idx.to(torch.int32)
        if idx.dim() != 2 or idx.stride(1) != 1:
            idx = idx.contiguous()
        if fmt == N.DENSE and idx.shape[0] != n:
            raise ValueError('neighbor list has a different number of atoms than R')
        width = idx.shape[1]
        ld = idx.stride(0) if idx.shape[0] > 1 else max(width, 1)
        cnt = neighbor.nbr_count if (fmt == N.DENSE and hasattr(neighbor, 'nbr_count')
                                      and neighbor.nbr_count is not None
                                      and neighbor.idx is idx) else None
        L = N.lib()
        ws = N.workspace(L.jmd_pair_workspace_bytes(n), R.device, 'pair')
        fs = force.stride(0) if force is not None else 0
        N.check(L.jmd_pair_forces(ctypes.byref(pair), ctypes.byref(sp), fmt, R.data_ptr(), rs,
                                  N.ptr(species), n, idx.data_ptr(), ld, width, N.ptr(cnt),
                                  N.ptr(force), fs, N.ptr(energy), N.ptr(per_atom), N.ptr(virial),
                                  ws.data_ptr(), ws.numel(), N.stream_ptr()), 'pair_forces')

    def forces(self, R, neighbor, out: Optional[torch.Tensor] = None, **dynamic):
        """-dE/dR as [N, d] (rows of stride 4 when R has them)."""
        if out is None:
            out = torch.empty((R.shape[0], 4), dtype=torch.float32, device=R.device)[:, :R.shape[1]]
        self.launch(R, neighbor, force=out, **dynamic)
        return out

    def compute(self, R, neighbor, force=True, per_atom=False, virial=False, **dynamic):
        """(energy f64 0-d, forces or None, per-atom energy or None, virial[6|3] or None)."""
        dev = R.device
        e = torch.empty((), dtype=torch.float64, device=dev)
        f = torch.empty((R.shape[0], 4), dtype=torch.float32, device=dev)[:, :R.shape[1]] if force else None
        pa = torch.empty(R.shape[0], dtype=torch.float32, device=dev) if per_atom else None
        dim = R.shape[1]
        w = torch.empty(6 if dim == 3 else 3, dtype=torch.float64, device=dev) if virial else None
        self.launch(R, neighbor, force=f, energy=e, per_atom=pa, virial=w, **dynamic)
        return e, f, pa, w

    def energy_f64(self, R, neighbor, **dynamic):
        return self.compute(R, neighbor, force=False, **dynamic)[0]

    def __call__(self, R, neighbor, **dynamic):
        per_particle = self.reduce_axis is not None and tuple(self.reduce_axis) == (1,)
        if per_particle:
            if neighbor.format is partition.OrderedSparse:
                raise ValueError('Cannot report per-particle values with a neighbor list whose '
                                 'format is `OrderedSparse`. Please use either `Dense` or `Sparse`.')
            _, _, pa, _ = self.compute(R.detach(), neighbor, force=False, per_atom=True, **dynamic)
            return pa

        sigma = _param_tensor(dynamic.get('sigma'))
        epsilon = _param_tensor(dynamic.get('epsilon'))
        if R.requires_grad or sigma is not None or epsilon is not None:
            return _EnergyFn.apply(R, sigma, epsilon, self, neighbor, dynamic)
        return self.energy_f64(R, neighbor, **dynamic).to(R.dtype)

    # -- adjoint ------------------------------------------------------------
    def force_fn_autograd(self, R, neighbor, **dynamic):
        """-dE/dR as a differentiable function of R and of sigma / epsilon
        tensors passed in ``dynamic`` (backward through the VJP kernel)."""
        return _ForceFn.apply(R, _param_tensor(dynamic.get('sigma')),
                              _param_tensor(dynamic.get('epsilon')), self, neighbor, dynamic)

    def _vjp_launch(self, R, neighbor, lam, weight, gR, gp, ge, **dynamic):
        R, rs = partition._rows(R)
        n, dim = R.shape
        species, pair = self._resolve(R, dynamic)
        sp = self.geometry.space(dim, dynamic.get('box'), dynamic.get('new_box'))
        idx = neighbor.idx
        if lam.stride(-1) != 1:
            lam = lam.contiguous()
        if neighbor.format is not partition.Dense:
            fmt = N.SPARSE if neighbor.format is partition.Sparse else N.ORDERED_SPARSE
            if idx.dtype != torch.int32 or idx.stride(1) != 1:
                idx = idx.to(torch.int32).contiguous()
            N.check(N.lib().jmd_pair_force_vjp_sparse(
                ctypes.byref(pair), ctypes.byref(sp), fmt, R.data_ptr(), rs, N.ptr(species), n,
                idx.data_ptr(), idx.stride(0), idx.shape[1], lam.data_ptr(), lam.stride(0),
                float(weight), N.ptr(gR), gR.stride(0) if gR is not None else 0, N.ptr(gp),
                N.ptr(ge), N.stream_ptr()), 'pair_force_vjp_sparse')
            return
        cnt = getattr(neighbor, 'nbr_count', None)
        N.check(N.lib().jmd_pair_force_vjp(
            ctypes.byref(pair), ctypes.byref(sp), R.data_ptr(), rs, N.ptr(species), n,
            idx.data_ptr(), idx.stride(0), idx.shape[1], N.ptr(cnt), lam.data_ptr(), lam.stride(0),
            float(weight), N.ptr(gR), gR.stride(0) if gR is not None else 0, N.ptr(gp), N.ptr(ge),
            N.stream_ptr()), 'pair_force_vjp')

    def force_vjp(self, R, neighbor, lam, weight=1.0, grad_R=None, grad_params=None, **dynamic):
        """(dF/dR)^T lam and d(lam . F)/d(sigma, epsilon) bins (accumulated into
        grad_R / grad_params when given).  Returns (grad_R, grad_params, None)."""
        dev = R.device
        n, dim = R.shape
        if grad_R is None:
            grad_R = torch.zeros((n, 4), dtype=torch.float32, device=dev)[:, :dim]
        if grad_params is None:
            grad_params = torch.zeros(130, dtype=torch.float64, device=dev)
        self._vjp_launch(R, neighbor, lam, weight, grad_R, grad_params, None, **dynamic)
        return grad_R, grad_params, None

    def energy_param_grad(self, R, neighbor, out=None, **dynamic):
        """dE/d(sigma, epsilon) bins [130] (f64)."""
        dev = R.device
        if out is None:
            out = torch.zeros(130, dtype=torch.float64, device=dev)
        lam = torch.zeros_like(R, dtype=torch.float32)
        self._vjp_launch(R, neighbor, lam, 0.0, None, None, out, **dynamic)
        return out


def pair_neighbor_list(fn, displacement_or_metric, species=None, reduce_axis=None,
                       ignore_unused_parameters: bool = False, **kwargs):
    """smap.pair_neighbor_list (smap.py:856-979)."""
    kwargs.pop('fractional_coordinates', None)
    return PairNeighborListEnergy(fn, displacement_or_metric, species, reduce_axis,
                                  ignore_unused_parameters, kwargs)


class PairAllEnergy:
    """smap.pair (smap.py:548-691): every pair i != j, through an all-pairs list."""

    def __init__(self, fn, displacement_or_metric, species, reduce_axis, params):
        self.inner = PairNeighborListEnergy(fn, displacement_or_metric, species, reduce_axis,
                                            True, params)
        self.fn = fn
        self.geometry = self.inner.geometry
        self._cache = {}

    def _neighbors(self, R, box=None):
        """The all-pairs list at R (pruned at the cutoff, rebuilt every call);
        ``box`` is a general cell's ``box`` keyword.  A list that overflows
        (pairs came closer) is re-allocated, so every pair is always kept."""
        n, dim = R.shape
        key = (n, dim, R.device)
        geo = self.geometry
        frac = isinstance(geo, _space.GeneralDisplacement) and geo.fractional_coordinates
        kw = {'box': box} if (box is not None and frac) else {}
        nb = self._cache.get(key)
        if nb is None:
            lbox = geo.box if geo.periodic else 1.0e30
            rc = self.fn.r_cutoff
            if self.fn.kind == N.SOFT_SPHERE:
                sig = self.inner.params.get('sigma', 1.0)
                rc = float(np.max(np.asarray(sig.detach().cpu() if isinstance(sig, torch.Tensor) else sig)))
            if not np.isfinite(rc):
                rc = 1.0e18
            fns = partition.neighbor_list(geo, lbox, rc, 0.0, capacity_multiplier=1.0,
                                          disable_cell_list=True, fractional_coordinates=frac)
            nb = (fns, fns.allocate(R, **kw))
            self._cache = {key: nb}
            return nb[1]
        lst = nb[0].update(R, nb[1], **kw)
        if kw and bool(lst.did_buffer_overflow):
            lst = nb[0].allocate(R, extra_capacity=max(8, lst.max_occupancy // 4), **kw)
            self._cache = {key: (nb[0], lst)}
        return lst

    def __call__(self, R, **dynamic):
        return self.inner(R, self._neighbors(R.detach(), dynamic.get('box')), **dynamic)

    def compute(self, R, **kw):
        return self.inner.compute(R, self._neighbors(R, kw.get('box')), **kw)

    def forces(self, R, **kw):
        return self.inner.forces(R, self._neighbors(R, kw.get('box')), **kw)


def pair(fn, displacement_or_metric, species=None, reduce_axis=None, **kwargs):
    """smap.pair (smap.py:548-691) for the kernel potentials."""
    kwargs.pop('ignore_unused_parameters', None)
    return PairAllEnergy(fn, displacement_or_metric, species, reduce_axis, kwargs)
