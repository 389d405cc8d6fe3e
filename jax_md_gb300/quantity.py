"""Physical quantities (jax_md/quantity.py) on device tensors.

``force`` / ``canonicalize_force`` return the kernel force function for the
CUDA-backed energies (one launch, no autograd tape) and fall back to
``torch.autograd`` only for user-written energy functions of tensors.
``pressure`` / ``stress`` take the virial dU/d(strain) from the pair kernel
instead of differentiating through a box perturbation (quantity.py:202-282).
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional

import numpy as np
import torch

from . import _native as N
from . import smap
from . import space as _space


def _kernel_energy(fn):
    return isinstance(fn, (smap.PairNeighborListEnergy, smap.PairAllEnergy))


def force(energy_fn):
    """quantity.py:58-60: -dE/dR."""
    if _kernel_energy(energy_fn):
        def force_fn(R, neighbor=None, **kwargs):
            if isinstance(energy_fn, smap.PairAllEnergy):
                return energy_fn.forces(R, **kwargs)
            return energy_fn.forces(R, neighbor, **kwargs)
        force_fn.energy_fn = energy_fn
        return force_fn

    def force_fn(R, **kwargs):
        Rg = R.detach().requires_grad_(True)
        with torch.enable_grad():
            E = energy_fn(Rg, **kwargs)
            (g,) = torch.autograd.grad(E, Rg)
        return -g
    force_fn.energy_fn = energy_fn
    return force_fn


def canonicalize_force(energy_or_force_fn):
    """quantity.py:76-102: accepts an energy or a force function."""
    if _kernel_energy(energy_or_force_fn):
        return force(energy_or_force_fn)
    if getattr(energy_or_force_fn, 'energy_fn', None) is not None:
        return energy_or_force_fn
    cache = {}

    def force_fn(R, **kwargs):
        f = cache.get('fn')
        if f is None:
            out = energy_or_force_fn(R, **kwargs)
            if isinstance(out, torch.Tensor) and out.dim() == 0:
                f = force(energy_or_force_fn)
            elif isinstance(out, torch.Tensor) and out.shape == R.shape:
                f = energy_or_force_fn
            else:
                raise ValueError('Provided function should be compatible with either an energy or '
                                 f'a force. Found a function whose output has shape {getattr(out, "shape", None)}.')
            cache['fn'] = f
        return f(R, **kwargs)
    return force_fn


def count_dof(position) -> int:
    """quantity.py:105-108."""
    return int(position.numel())


def volume(dimension: int, box) -> float:
    """quantity.py:111-121."""
    b = np.asarray(box.detach().cpu() if isinstance(box, torch.Tensor) else box, np.float64)
    if b.ndim == 0:
        return float(b) ** dimension
    if b.ndim == 1:
        return float(np.prod(b))
    return float(np.linalg.det(b))


def _mass_arg(mass):
    if isinstance(mass, torch.Tensor) and mass.numel() > 1:
        return mass.reshape(-1).contiguous().float(), 1.0
    return None, float(mass)


def kinetic_energy(*unused_args, momentum=None, velocity=None, mass=1.0):
    """quantity.py:124-159 (f64 reduction on the device)."""
    if unused_args:
        raise ValueError('To use the kinetic energy function, you must explicitly pass either '
                         'momentum or velocity as a keyword argument.')
    if momentum is not None and velocity is not None:
        raise ValueError('To use the kinetic energy function, you must pass either a momentum or '
                         'a velocity.')
    if momentum is None:
        m = mass.reshape(-1, 1) if isinstance(mass, torch.Tensor) and mass.numel() > 1 else mass
        momentum = velocity * m
    return _ke_f64(momentum, mass).to(momentum.dtype)


def _ke_f64(momentum, mass=1.0, out=None):
    N.require_cuda(momentum)
    if momentum.stride(-1) != 1:
        momentum = momentum.contiguous()
    n, dim = momentum.shape
    mptr, m0 = _mass_arg(mass)
    out = torch.empty((), dtype=torch.float64, device=momentum.device) if out is None else out
    L = N.lib()
    ws = N.workspace(L.jmd_reduce_workspace_bytes(n), momentum.device, 'reduce')
    N.check(L.jmd_kinetic_energy(momentum.data_ptr(), momentum.stride(0), N.ptr(mptr), m0, n, dim,
                                 out.data_ptr(), ws.data_ptr(), ws.numel(), N.stream_ptr()),
            'kinetic_energy')
    return out


def temperature(*unused_args, momentum=None, velocity=None, mass=1.0):
    """quantity.py:162-199: sum p^2/m / dof."""
    if momentum is None:
        m = mass.reshape(-1, 1) if isinstance(mass, torch.Tensor) and mass.numel() > 1 else mass
        momentum = velocity * m
    ke = _ke_f64(momentum, mass)
    return (2.0 * ke / momentum.numel()).to(momentum.dtype)


def _virial(energy_fn, position, box=None, **kwargs):
    """dU/d(strain) as a [d, d] f64 matrix; ``box`` reaches the energy as its
    keyword (a general cell's current cell), and is dropped for a space that
    refuses it, as quantity.py:225-229 does."""
    if not _kernel_energy(energy_fn):
        raise NotImplementedError('pressure/stress need a CUDA-backed energy function')
    nb = kwargs.pop('neighbor', None)

    def run(**kw):
        if isinstance(energy_fn, smap.PairAllEnergy):
            return energy_fn.compute(position, force=False, virial=True, **kw)[3]
        return energy_fn.compute(position, nb, force=False, virial=True, **kw)[3]
    if box is not None:
        try:
            W = run(box=box, **kwargs)
        except _space.UnexpectedBoxException:
            W = run(**kwargs)
    else:
        W = run(**kwargs)
    dim = position.shape[1]
    if dim == 3:
        xx, yy, zz, xy, xz, yz = W
        return torch.stack([torch.stack([xx, xy, xz]), torch.stack([xy, yy, yz]),
                            torch.stack([xz, yz, zz])])
    xx, yy, xy = W
    return torch.stack([torch.stack([xx, xy]), torch.stack([xy, yy])])


def pressure(energy_fn, position, box, kinetic_energy=0.0, **kwargs):
    """quantity.py:202-235: (2 KE - tr dU/d(strain)) / (d V)."""
    dim = position.shape[1]
    W = _virial(energy_fn, position, box=box, **kwargs)
    V = volume(dim, box)
    ke = kinetic_energy if isinstance(kinetic_energy, torch.Tensor) else torch.tensor(
        float(kinetic_energy), dtype=torch.float64, device=position.device)
    return ((2.0 * ke.double() - torch.trace(W)) / (dim * V)).to(position.dtype)


def stress(energy_fn, position, box, mass=1.0, velocity=None, **kwargs):
    """quantity.py:238-282: (sum m v v^T - dU/d(strain)) / V."""
    dim = position.shape[1]
    W = _virial(energy_fn, position, box=box, **kwargs)
    V = volume(dim, box)
    VxV = torch.zeros((dim, dim), dtype=torch.float64, device=position.device)
    if velocity is not None:
        v = velocity.double()
        m = mass.double().reshape(-1, 1) if isinstance(mass, torch.Tensor) else float(mass)
        VxV = torch.einsum('na,nb->ab', m * v, v)
    return ((VxV - W) / V).to(position.dtype)


def clipped_force(energy_fn, max_force: float):
    """quantity.py:63-73: the force with each atom's vector clipped to norm
    max_force."""
    force_fn = force(energy_fn)

    def wrapped(R, *args, **kwargs):
        f = force_fn(R, *args, **kwargs)
        n = torch.linalg.norm(f, dim=-1, keepdim=True)
        return torch.where(n > max_force, f / n * max_force, f)
    return wrapped


def nball_unit_volume(spatial_dimension: int) -> float:
    """quantity.py:592-596: volume of the unit ball in d dimensions."""
    return math.pi ** (spatial_dimension / 2) / math.gamma(spatial_dimension / 2 + 1)


def particle_volume(radii, spatial_dimension: int, particle_count=1, species=None):
    """quantity.py:599-624: total volume of balls of the given radii (per
    particle, per species with `species`, or with counts)."""
    r = np.asarray(radii.detach().cpu() if isinstance(radii, torch.Tensor) else radii, np.float64)
    v = nball_unit_volume(spatial_dimension) * r ** spatial_dimension
    if species is not None:
        sp = np.asarray(species.detach().cpu() if isinstance(species, torch.Tensor) else species)
        particle_count = np.bincount(sp.reshape(-1))
    return float(np.sum(np.asarray(particle_count) * v))


def volume_fraction(box, radii, spatial_dimension: int, particle_count=1, species=None) -> float:
    """quantity.py:627-639."""
    return particle_volume(radii, spatial_dimension, particle_count, species) / \
        volume(spatial_dimension, box)


def box_size_at_volume_fraction(volume_fraction: float, radii, spatial_dimension: int,
                                particle_count=1, species=None) -> float:
    """quantity.py:642-654."""
    v = particle_volume(radii, spatial_dimension, particle_count, species)
    return (v / volume_fraction) ** (1.0 / spatial_dimension)


def box_size_at_number_density(particle_count: int, number_density: float,
                               spatial_dimension: int) -> float:
    """quantity.py:657-660."""
    return (particle_count / number_density) ** (1.0 / spatial_dimension)

