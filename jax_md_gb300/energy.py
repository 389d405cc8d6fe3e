"""Pair potentials and their neighbour-list builders (jax_md/energy.py).

The elementwise functions (``lennard_jones``, ``soft_sphere``, ``morse``,
``multiplicative_isotropic_cutoff``) evaluate the reference formulas on
tensors and are tagged so that ``smap.pair_neighbor_list`` can map them onto
the fused CUDA pair kernels.  ``lennard_jones_neighbor_list``,
``soft_sphere_neighbor_list`` and ``morse_neighbor_list`` keep the reference
signatures and plug-in points (``neighbor_list_fn=``,
``pair_neighbor_list_fn=``).
"""
from __future__ import annotations

import math
from typing import Callable, Optional

import numpy as np
import torch

from . import _native as N
from . import partition, smap, space


class PairFunction:
    """A pair potential the CUDA kernels implement.

    kind: N.LJ (with the multiplicative cutoff), N.LJ_TRUNCATED, N.SOFT_SPHERE,
    N.MORSE (smoothed between r_onset and r_cutoff when r_onset < r_cutoff).
    r_onset / r_cutoff: absolute radii of the smoothing or truncation."""

    def __init__(self, kind: int, elementwise: Callable, r_onset: float = math.inf,
                 r_cutoff: float = math.inf, name: str = ''):
        self.kind = kind
        self.elementwise = elementwise
        self.r_onset = r_onset
        self.r_cutoff = r_cutoff
        self.__name__ = name or getattr(elementwise, '__name__', 'pair')

    def __call__(self, dr, *args, **kwargs):
        return self.elementwise(dr, *args, **kwargs)


def _lj(dr, sigma=1.0, epsilon=1.0, **unused):
    """energy.py:246-272."""
    idr = sigma / dr
    idr = idr * idr
    idr6 = idr * idr * idr
    idr12 = idr6 * idr6
    return torch.nan_to_num(4.0 * epsilon * (idr12 - idr6))


def _ss(dr, sigma=1.0, epsilon=1.0, alpha=2.0, **unused):
    """energy.py:125-173."""
    x = dr / sigma
    inside = x < 1.0
    base = torch.where(inside, 1.0 - x, torch.zeros_like(x))
    return torch.where(inside, epsilon / alpha * base ** alpha, torch.zeros_like(x))


def _morse(dr, sigma=1.0, epsilon=5.0, alpha=5.0, **unused):
    """energy.py:346-371."""
    U = epsilon * (1.0 - torch.exp(-alpha * (dr - sigma))) ** 2 - epsilon
    return torch.nan_to_num(U)


lennard_jones = PairFunction(N.LJ_TRUNCATED, _lj, name='lennard_jones')
soft_sphere = PairFunction(N.SOFT_SPHERE, _ss, name='soft_sphere')
morse = PairFunction(N.MORSE, _morse, name='morse')


def multiplicative_isotropic_cutoff(fn, r_onset, r_cutoff):
    """energy.py:534-580: S(r) f(r) with the C1 switch of HOOMD-blue."""
    r_onset = float(r_onset)
    r_cutoff = float(r_cutoff)
    rc, ro = r_cutoff ** 2, r_onset ** 2

    def smooth(dr):
        r = dr ** 2
        inner = torch.where(dr < r_cutoff, (rc - r) ** 2 * (rc + 2 * r - 3 * ro) / (rc - ro) ** 3,
                            torch.zeros_like(dr))
        return torch.where(dr < r_onset, torch.ones_like(dr), inner)

    def cutoff_fn(dr, *args, **kwargs):
        return smooth(dr) * fn(dr, *args, **kwargs)

    base = fn.kind if isinstance(fn, PairFunction) else None
    if base == N.LJ_TRUNCATED:
        return PairFunction(N.LJ, cutoff_fn, r_onset, r_cutoff, name='lennard_jones_smoothed')
    if base == N.MORSE and not np.isfinite(fn.r_cutoff):
        return PairFunction(N.MORSE, cutoff_fn, r_onset, r_cutoff, name='morse_smoothed')
    return cutoff_fn


def truncated(fn: PairFunction, r_cutoff: float) -> PairFunction:
    """fn(r) for r < r_cutoff, else 0 (the LJ truncation of quantity_test.py:441-446)."""
    if fn.kind != N.LJ_TRUNCATED:
        raise NotImplementedError('truncation is provided for lennard_jones')

    def t(dr, *args, **kwargs):
        return torch.where(dr < r_cutoff, fn(dr, *args, **kwargs), torch.zeros_like(dr))

    return PairFunction(N.LJ_TRUNCATED, t, r_cutoff, float(r_cutoff), name='lennard_jones_truncated')


def _max(x) -> float:
    if isinstance(x, torch.Tensor):
        return float(x.max())
    return float(np.max(np.asarray(x)))


def lennard_jones_neighbor_list(displacement_or_metric, box_size, species=None, sigma=1.0,
                                epsilon=1.0, r_onset: float = 2.0, r_cutoff: float = 2.5,
                                dr_threshold: float = 0.5, per_particle: bool = False,
                                fractional_coordinates: bool = False,
                                format=partition.OrderedSparse,
                                neighbor_list_fn: Callable = partition.neighbor_list,
                                pair_neighbor_list_fn: Callable = smap.pair_neighbor_list,
                                **neighbor_kwargs):
    """energy.py:300-343."""
    ms = _max(sigma)
    r_onset = np.float32(r_onset) * np.float32(ms)
    r_cutoff = np.float32(r_cutoff) * np.float32(ms)
    neighbor_fn = neighbor_list_fn(displacement_or_metric, box_size, float(r_cutoff),
                                   float(np.float32(dr_threshold)),
                                   fractional_coordinates=fractional_coordinates, format=format,
                                   **neighbor_kwargs)
    energy_fn = pair_neighbor_list_fn(
        multiplicative_isotropic_cutoff(lennard_jones, float(r_onset), float(r_cutoff)),
        space.canonicalize_displacement_or_metric(displacement_or_metric),
        ignore_unused_parameters=True, species=species, sigma=sigma, epsilon=epsilon,
        reduce_axis=(1,) if per_particle else None)
    return neighbor_fn, energy_fn


def soft_sphere_neighbor_list(displacement_or_metric, box_size, species=None, sigma=1.0,
                              epsilon=1.0, alpha=2.0, dr_threshold: float = 0.2,
                              per_particle: bool = False, fractional_coordinates: bool = False,
                              format=partition.OrderedSparse,
                              neighbor_list_fn: Callable = partition.neighbor_list,
                              pair_neighbor_list_fn: Callable = smap.pair_neighbor_list,
                              **neighbor_kwargs):
    """energy.py:200-243."""
    list_cutoff = _max(sigma)
    neighbor_fn = neighbor_list_fn(displacement_or_metric, box_size, float(np.float32(list_cutoff)),
                                   float(np.float32(dr_threshold)),
                                   fractional_coordinates=fractional_coordinates, format=format,
                                   **neighbor_kwargs)
    energy_fn = pair_neighbor_list_fn(
        soft_sphere, space.canonicalize_displacement_or_metric(displacement_or_metric),
        ignore_unused_parameters=True, species=species, sigma=sigma, epsilon=epsilon, alpha=alpha,
        reduce_axis=(1,) if per_particle else None)
    return neighbor_fn, energy_fn


def lennard_jones_pair(displacement_or_metric, species=None, sigma=1.0, epsilon=1.0,
                       r_onset: float = 2.0, r_cutoff: float = 2.5, per_particle: bool = False):
    """energy.py:275-297: all-pairs LJ, evaluated through an all-pairs list."""
    ms = _max(sigma)
    fn = multiplicative_isotropic_cutoff(lennard_jones, float(np.float32(r_onset) * ms),
                                         float(np.float32(r_cutoff) * ms))
    return smap.pair(fn, displacement_or_metric, species=species, sigma=sigma, epsilon=epsilon,
                     reduce_axis=(1,) if per_particle else None)


def soft_sphere_pair(displacement_or_metric, species=None, sigma=1.0, epsilon=1.0, alpha=2.0,
                     per_particle: bool = False):
    """energy.py:176-197."""
    return smap.pair(soft_sphere, displacement_or_metric, species=species, sigma=sigma,
                     epsilon=epsilon, alpha=alpha, reduce_axis=(1,) if per_particle else None)


def morse_pair(displacement_or_metric, species=None, sigma=1.0, epsilon=5.0, alpha=5.0,
               r_onset: float = 2.0, r_cutoff: float = 2.5, per_particle: bool = False):
    """energy.py:374-397: all-pairs Morse with the multiplicative cutoff
    (absolute radii), evaluated through an all-pairs list."""
    fn = multiplicative_isotropic_cutoff(morse, float(np.float32(r_onset)),
                                         float(np.float32(r_cutoff)))
    return smap.pair(fn, displacement_or_metric, species=species, sigma=sigma, epsilon=epsilon,
                     alpha=alpha, reduce_axis=(1,) if per_particle else None)


def morse_neighbor_list(displacement_or_metric, box_size, species=None, sigma=1.0, epsilon=5.0,
                        alpha=5.0, r_onset: float = 2.0, r_cutoff: float = 2.5,
                        dr_threshold: float = 0.5, per_particle: bool = False,
                        fractional_coordinates: bool = False, format=partition.OrderedSparse,
                        neighbor_list_fn: Callable = partition.neighbor_list,
                        pair_neighbor_list_fn: Callable = smap.pair_neighbor_list,
                        **neighbor_kwargs):
    """energy.py:400-440: the radii are absolute (not multiples of sigma)."""
    r_onset = float(np.float32(r_onset))
    r_cutoff = float(np.float32(r_cutoff))
    neighbor_fn = neighbor_list_fn(displacement_or_metric, box_size, r_cutoff,
                                   float(np.float32(dr_threshold)),
                                   fractional_coordinates=fractional_coordinates, format=format,
                                   **neighbor_kwargs)
    energy_fn = pair_neighbor_list_fn(
        multiplicative_isotropic_cutoff(morse, r_onset, r_cutoff),
        space.canonicalize_displacement_or_metric(displacement_or_metric),
        ignore_unused_parameters=True, species=species, sigma=sigma, epsilon=epsilon, alpha=alpha,
        reduce_axis=(1,) if per_particle else None)
    return neighbor_fn, energy_fn
