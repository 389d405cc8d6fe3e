"""Spaces: periodic and free boundary conditions (jax_md/space.py).

``periodic(side)`` and ``free()`` return ``(displacement_fn, shift_fn)`` with
the reference's call signatures (space.py:258-329).  The returned callables
also carry the geometry (``box``, ``periodic``, ``dim``) so the neighbour-list
and pair kernels can be configured from them; applied to tensors they compute
the reference's formulas on the tensor's device.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import _native as N


class UnexpectedBoxException(Exception):
    """space.py: raised when a box keyword reaches space.periodic."""


def _as_box(side):
    if isinstance(side, torch.Tensor):
        side = side.detach().cpu().double().reshape(-1).tolist()
        return side[0] if len(side) == 1 else side
    try:
        return float(side)
    except TypeError:
        return [float(s) for s in side]


def square_distance(dR: torch.Tensor) -> torch.Tensor:
    """space.py:227-235."""
    return (dR * dR).sum(-1)


def distance(dR: torch.Tensor) -> torch.Tensor:
    """space.py:238-247 (safe at zero)."""
    dr = square_distance(dR)
    return torch.where(dr > 0, torch.sqrt(torch.where(dr > 0, dr, torch.ones_like(dr))),
                       torch.zeros_like(dr))


def _side_tensor(side, like: torch.Tensor):
    return torch.as_tensor(side, dtype=like.dtype, device=like.device)


def periodic_displacement(side, dR: torch.Tensor) -> torch.Tensor:
    """space.py:213-224: mod(dR + L/2, L) - L/2."""
    L = _side_tensor(side, dR)
    return torch.remainder(dR + L * 0.5, L) - 0.5 * L


def periodic_shift(side, R: torch.Tensor, dR: torch.Tensor) -> torch.Tensor:
    """space.py:250-252: mod(R + dR, L)."""
    return torch.remainder(R + dR, _side_tensor(side, R))


class Displacement:
    """Displacement function carrying its geometry."""

    def __init__(self, box, periodic: bool):
        self.box = box
        self.periodic = periodic

    def __call__(self, Ra, Rb, perturbation: Optional[torch.Tensor] = None, **kwargs):
        if 'box' in kwargs and self.periodic:
            raise UnexpectedBoxException('`space.periodic` does not accept a box argument. '
                                         'Perhaps you meant to use `space.periodic_general`?')
        dR = Ra - Rb
        if self.periodic:
            dR = periodic_displacement(self.box, dR)
        if perturbation is not None:
            p = torch.as_tensor(perturbation, dtype=dR.dtype, device=dR.device)
            dR = dR * p if p.dim() <= 1 else torch.einsum('ij,...j->...i', p, dR)
        return dR

    def space(self, dim: int) -> N.Space:
        s = N.Space()
        s.dim = dim
        s.periodic = 1 if self.periodic else 0
        b = self.box
        if isinstance(b, (list, tuple)):
            if len(b) != dim:
                raise ValueError(f'box has {len(b)} sides for a {dim}-dimensional system')
            for d in range(dim):
                s.box[d] = float(b[d])
        else:
            for d in range(dim):
                s.box[d] = float(b) if b is not None else 0.0
        return s


class Shift:
    """Shift function carrying its geometry (space.py:304-327)."""

    def __init__(self, box, periodic: bool, wrapped: bool = True):
        self.box = box
        self.periodic = periodic
        self.wrapped = wrapped

    def __call__(self, R, dR, **kwargs):
        if 'box' in kwargs and self.periodic:
            raise UnexpectedBoxException('`space.periodic` does not accept a box argument.')
        if self.periodic and self.wrapped:
            return periodic_shift(self.box, R, dR)
        return R + dR


def periodic(side, wrapped: bool = True):
    """space.periodic (space.py:275-329)."""
    box = _as_box(side)
    return Displacement(box, True), Shift(box, True, wrapped)


def free():
    """space.free (space.py:258-272)."""
    return Displacement(None, False), Shift(None, False)


def metric(displacement):
    """space.py:475-477."""
    def m(Ra, Rb, **kwargs):
        return distance(displacement(Ra, Rb, **kwargs))
    m.displacement = displacement
    return m


def canonicalize_displacement_or_metric(displacement_or_metric):
    """space.py:505-522: keeps our geometry-carrying displacement as is."""
    return displacement_or_metric


def geometry_of(displacement_or_metric):
    """The Displacement object behind a displacement or metric function."""
    d = displacement_or_metric
    if isinstance(d, Displacement):
        return d
    inner = getattr(d, 'displacement', None)
    if isinstance(inner, Displacement):
        return inner
    raise TypeError('jax_md_gb300 kernels need a displacement from jax_md_gb300.space.periodic '
                    'or space.free; got ' + repr(d))


def map_bond(fn):
    """space.py:487-491 (tensors broadcast already)."""
    return fn


def map_neighbor(fn):
    """space.py:494-502: fn(R_neigh, R) for R [N,d], R_neigh [N,M,d]."""
    def wrapped(Ra, Rb, **kwargs):
        return fn(Rb, Ra[:, None, :], **kwargs)
    return wrapped
