"""Spaces: periodic and free boundary conditions (jax_md/space.py).

``periodic(side)``, ``free()`` and ``periodic_general(box)`` return
``(displacement_fn, shift_fn)`` with the reference's call signatures
(space.py:258-468).  The returned callables
also carry the geometry (``box``, ``periodic``, ``dim``) so the neighbour-list
and pair kernels can be configured from them; applied to tensors they compute
the reference's formulas on the tensor's device.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
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

    def space(self, dim: int, box=None, new_box=None) -> N.Space:
        if (box is not None or new_box is not None) and self.periodic:
            raise UnexpectedBoxException('`space.periodic` does not accept a box argument. '
                                         'Perhaps you meant to use `space.periodic_general`?')
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


def inverse(box):
    """space.py:109-119: 1 / box for a scalar or sides, the matrix inverse
    for a cell matrix."""
    b = box if isinstance(box, torch.Tensor) else torch.as_tensor(box, dtype=torch.float64)
    return torch.linalg.inv(b) if b.dim() == 2 else 1.0 / b


class _Transform(torch.autograd.Function):
    """x = T u row by row, with the reference's derivative (space.py:155-185):
    the position tangent passes through unchanged, so gradients taken with
    respect to fractional positions are real-space gradients."""

    @staticmethod
    def forward(ctx, box, R):
        ctx.save_for_backward(box, R)
        return R * box if box.dim() <= 1 else torch.einsum('ij,...j->...i', box, R)

    @staticmethod
    def backward(ctx, g):
        box, R = ctx.saved_tensors
        gb = None
        if ctx.needs_input_grad[0]:
            if box.dim() == 0:
                gb = (g * R).sum()
            elif box.dim() == 1:
                gb = (g * R).reshape(-1, R.shape[-1]).sum(0)
            else:
                gb = torch.einsum('...i,...j->ij', g, R)
        return gb, g


def transform(box, R: torch.Tensor) -> torch.Tensor:
    """space.py:125-185: R * box for a scalar or per-axis sides, R @ box^T
    for a cell matrix (x = T u), with the reference's pass-through
    derivative in R."""
    b = torch.as_tensor(box, dtype=R.dtype, device=R.device)
    return _Transform.apply(b, R)


def cell_matrix(box, dim: int) -> np.ndarray:
    """The cell T as a [dim, dim] float64 matrix: a scalar or per-axis sides
    become a diagonal (space.py:125-148 treats them as such)."""
    b = box.detach().cpu().double().numpy() if isinstance(box, torch.Tensor) else np.asarray(
        box, np.float64)
    if b.ndim == 0 or b.size == 1:
        return np.eye(dim) * float(b.reshape(-1)[0])
    if b.ndim == 1:
        if b.size != dim:
            raise ValueError(f'box has {b.size} sides for a {dim}-dimensional system')
        return np.diag(b)
    if b.shape != (dim, dim):
        raise ValueError(f'cell matrix of shape {b.shape} for a {dim}-dimensional system')
    return b


def general_space(box, dim: int) -> N.Space:
    """The kernels' geometry of a general cell with fractional coordinates:
    minimum image in the unit cube, displacement T d, shift by T^-1 dR.  The
    kernels take upper-triangular cells (the reference's is_box_valid,
    partition.py:676-681)."""
    T = cell_matrix(box, dim)
    if not np.array_equal(np.triu(T), T):
        raise ValueError('the kernels take upper-triangular cell matrices (partition.is_box_valid)')
    if np.any(np.diag(T) <= 0):
        raise ValueError('the cell matrix needs a positive diagonal')
    Ti = np.linalg.inv(T)
    s = N.Space()
    s.dim = dim
    s.periodic = N.GENERAL_CELL
    for d in range(3):
        s.box[d] = 1.0
    for a in range(dim):
        for b in range(dim):
            s.cell[3 * a + b] = float(np.float32(T[a, b]))
            s.inv_cell[3 * a + b] = float(np.float32(Ti[a, b]))
    if dim == 2:
        s.cell[8] = s.inv_cell[8] = 1.0
    return s


class GeneralDisplacement:
    """Displacement of space.periodic_general (space.py:413-434)."""

    periodic = True

    def __init__(self, box, fractional_coordinates: bool):
        self.box = box
        self.inv_box = inverse(box)
        self.fractional_coordinates = fractional_coordinates

    def space(self, dim: int, box=None, new_box=None) -> N.Space:
        """Kernel geometry; ``box`` / ``new_box`` replace the cell as the
        keywords of the displacement do (space.py:417-429)."""
        T = new_box if new_box is not None else (box if box is not None else self.box)
        if self.fractional_coordinates:
            return general_space(T, dim)
        # real coordinates: the kernels bin and wrap in the cell's own frame
        # only for an orthorhombic cell (then T^-1 x, d_U and T give the
        # minimum image of space.periodic)
        if new_box is not None:
            raise NotImplementedError('new_box with real coordinates is not implemented by the '
                                      'kernels')
        M = cell_matrix(T, dim)
        if not np.array_equal(np.diag(np.diag(M)), M):
            raise NotImplementedError('general cells in the kernels take fractional coordinates '
                                      '(periodic_general(box, fractional_coordinates=True))')
        s = N.Space()
        s.dim = dim
        s.periodic = 1
        for d in range(dim):
            s.box[d] = float(M[d, d])
        return s

    def __call__(self, Ra, Rb, perturbation=None, **kwargs):
        box, inv = self.box, self.inv_box
        if 'box' in kwargs:
            box = kwargs['box']
            if not self.fractional_coordinates:
                inv = inverse(box)
        if 'new_box' in kwargs:
            box = kwargs['new_box']
        if not self.fractional_coordinates:
            Ra, Rb = transform(inv, Ra), transform(inv, Rb)
        dR = transform(box, periodic_displacement(1.0, Ra - Rb))
        if perturbation is not None:
            p = torch.as_tensor(perturbation, dtype=dR.dtype, device=dR.device)
            dR = dR * p if p.dim() <= 1 else torch.einsum('ij,...j->...i', p, dR)
        return dR


class GeneralShift:
    """Shift of space.periodic_general (space.py:436-466): dR lives in the
    cell; R in the unit cube (fractional) or in the cell."""

    def space(self, dim: int, box=None) -> N.Space:
        """Kernel geometry of the shift (see GeneralDisplacement.space);
        ``box`` replaces the cell, as the shift's keyword does."""
        T = self.box if box is None else box
        if self.fractional_coordinates and self.wrapped:
            return general_space(T, dim)
        if box is not None:
            raise NotImplementedError('a box keyword with real coordinates is not implemented by '
                                      'the integrator kernels')
        M = cell_matrix(self.box, dim)
        if self.fractional_coordinates or not np.array_equal(np.diag(np.diag(M)), M):
            raise NotImplementedError('the integrator kernels take wrapped fractional coordinates '
                                      'for general cells')
        s = N.Space()
        s.dim = dim
        s.periodic = 1 if self.wrapped else 0
        if self.wrapped:
            for d in range(dim):
                s.box[d] = float(M[d, d])
        return s

    def __init__(self, box, fractional_coordinates: bool, wrapped: bool):
        self.box = box
        self.inv_box = inverse(box)
        self.fractional_coordinates = fractional_coordinates
        self.wrapped = wrapped

    def __call__(self, R, dR, **kwargs):
        if not self.fractional_coordinates and not self.wrapped:
            return R + dR
        box, inv = self.box, self.inv_box
        if 'box' in kwargs:
            box = kwargs['box']
            inv = inverse(box)
        if 'new_box' in kwargs:
            box = kwargs['new_box']
        dR = transform(inv, dR)
        if not self.fractional_coordinates:
            R = transform(inv, R)
        R = periodic_shift(1.0, R, dR) if self.wrapped else R + dR
        if not self.fractional_coordinates:
            R = transform(box, R)
        return R


def periodic_general(box, fractional_coordinates: bool = True, wrapped: bool = True):
    """space.periodic_general (space.py:332-468): periodic boundary conditions
    on the cell T [0, 1]^d (T a scalar, per-axis sides or a cell matrix),
    positions in the unit cube (fractional_coordinates) or in the cell.  These
    are tensor functions and carry the geometry for the kernels (fractional
    coordinates with an upper-triangular cell; real coordinates with an
    orthorhombic one)."""
    return (GeneralDisplacement(box, fractional_coordinates),
            GeneralShift(box, fractional_coordinates, wrapped))


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
    if isinstance(d, GeneralDisplacement):
        return d
    if isinstance(inner, GeneralDisplacement):
        return inner
    raise TypeError('jax_md_gb300 kernels need a displacement from jax_md_gb300.space.periodic '
                    'or space.free; got ' + repr(d))


def map_product(fn):
    """space.py:480-484: fn over all pairs, out[b, a] = fn(Ra[a], Rb[b]) (the
    reference's nested vmaps put Rb on the first axis)."""
    def wrapped(Ra, Rb, **kwargs):
        return fn(Ra[None, :, :], Rb[:, None, :], **kwargs)
    return wrapped


def map_bond(fn):
    """space.py:487-491 (tensors broadcast already)."""
    return fn


def map_neighbor(fn):
    """space.py:494-502: fn(R_neigh, R) for R [N,d], R_neigh [N,M,d]."""
    def wrapped(Ra, Rb, **kwargs):
        return fn(Rb, Ra[:, None, :], **kwargs)
    return wrapped
