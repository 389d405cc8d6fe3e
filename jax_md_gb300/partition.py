"""Cell lists and neighbour lists (jax_md/partition.py) on the GB300 kernels.

Drop-in for ``partition.cell_list`` (partition.py:296-488) and
``partition.neighbor_list`` (partition.py:801-1164): same arguments, same
``NeighborList`` fields, same ``PartitionErrorCode`` bits and sticky
``did_buffer_overflow`` semantics, same capacity rule at ``allocate``.  The
Dense ``idx`` array is identical to the reference's, entry order included.

Differences, by design:
  * ``update`` rebuilds in place: the returned ``NeighborList`` shares its
    device buffers (``idx``, ``reference_position``, ``error.code``) with the
    list it was called on, so an update costs no allocation and no host sync.
    The skin test of partition.py:1146-1154 runs on the device and gates the
    rebuild kernels through a device flag (the lax.cond).
  * ``custom_mask_function`` is not supported (it raises NotImplementedError);
    ``fractional_coordinates`` bins the unit cube of a periodic_general cell
    (upper-triangular cells, as the reference's is_box_valid requires).
"""
from __future__ import annotations

import dataclasses
import math
from enum import Enum, IntEnum
from typing import Callable, Optional

import numpy as np
import torch

from . import _native as N
from . import space as _space


class NeighborListFormat(Enum):
    """partition.py:641-657."""
    Dense = 0
    Sparse = 1
    OrderedSparse = 2


Dense = NeighborListFormat.Dense
Sparse = NeighborListFormat.Sparse
OrderedSparse = NeighborListFormat.OrderedSparse


def is_sparse(fmt: NeighborListFormat) -> bool:
    return fmt is NeighborListFormat.Sparse or fmt is NeighborListFormat.OrderedSparse


def is_format_valid(fmt):
    if fmt not in list(NeighborListFormat):
        raise ValueError(f'Neighbor list format must be a member of NeighborListFormat found {fmt}.')


class PartitionErrorCode(IntEnum):
    """partition.py:494-520."""
    NONE = 0
    NEIGHBOR_LIST_OVERFLOW = 1 << 0
    CELL_LIST_OVERFLOW = 1 << 1
    CELL_SIZE_TOO_SMALL = 1 << 2
    MALFORMED_BOX = 1 << 3


PEC = PartitionErrorCode


@dataclasses.dataclass
class PartitionError:
    """partition.py:523-561; ``code`` is a uint8 device tensor."""
    code: torch.Tensor

    def update(self, bit: PartitionErrorCode, pred) -> 'PartitionError':
        pred = torch.as_tensor(pred, device=self.code.device)
        return PartitionError(self.code | torch.where(pred, torch.tensor(int(bit), dtype=torch.uint8,
                                                                        device=self.code.device),
                                                      torch.zeros((), dtype=torch.uint8,
                                                                  device=self.code.device)))

    def __str__(self) -> str:
        c = int(self.code)
        if not c:
            return ''
        if c & PEC.NEIGHBOR_LIST_OVERFLOW:
            return 'Partition Error: Neighbor list buffer overflow.'
        if c & PEC.CELL_LIST_OVERFLOW:
            return 'Partition Error: Cell list buffer overflow'
        if c & PEC.CELL_SIZE_TOO_SMALL:
            return 'Partition Error: Cell size too small'
        if c & PEC.MALFORMED_BOX:
            return 'Partition Error: Incorrect box format. Expecting upper triangular.'
        raise ValueError(f'Unexpected Error Code {c}.')

    __repr__ = __str__


# ---------------------------------------------------------------- helpers --
def _f32(x) -> np.float32:
    return np.float32(x)


def _box_list(box, dim):
    if isinstance(box, (list, tuple)):
        return [float(b) for b in box]
    if isinstance(box, (np.ndarray, torch.Tensor)):
        b = np.asarray(box.detach().cpu() if isinstance(box, torch.Tensor) else box, np.float64)
        if b.ndim == 0 or b.size == 1:
            return [float(b.reshape(-1)[0])] * dim
        if b.ndim == 2:
            if not np.allclose(b, np.diag(np.diag(b))):
                raise NotImplementedError('general (triclinic) boxes need periodic_general, '
                                          'which the kernels do not implement yet')
            b = np.diag(b)
        return [float(v) for v in b.reshape(-1)[:dim]]
    return [float(box)] * dim


def cell_dimensions(dim, box, minimum_cell_size):
    """partition.py:146-188 in float32: (cells_per_side, cell_size, count)."""
    L = np.array(_box_list(box, dim), np.float32)
    m = _f32(minimum_cell_size)
    cps = np.floor(L / m)
    cs = (L / cps).astype(np.float32)
    cps = cps.astype(np.int64)
    return cps, cs, int(np.prod(cps))


def _rows(R: torch.Tensor):
    """(tensor, row stride) with contiguous rows; float32 on CUDA."""
    N.require_cuda(R)
    if R.dtype != torch.float32:
        raise TypeError('jax_md_gb300 kernels compute in float32; pass float32 positions')
    if R.dim() != 2 or R.stride(1) != 1:
        R = R.contiguous()
    return R, R.stride(0)


def padded_rows(R: torch.Tensor) -> torch.Tensor:
    """A [N, d] view over float4 rows ([N, 4] storage, w = 0): the fast layout."""
    n, d = R.shape
    buf = torch.zeros((n, 4), dtype=torch.float32, device=R.device)
    buf[:, :d] = R
    return buf[:, :d]


def fractional_cell_size(box, cutoff):
    """partition.py:595-634 (_fractional_cell_size) in float32: the cell edge,
    in units of the unit cube, whose perpendicular width in the cell T is at
    least ``cutoff``."""
    b = np.asarray(box.detach().cpu() if isinstance(box, torch.Tensor) else box, np.float32)
    c = _f32(cutoff)
    if b.ndim == 0 or b.size == 1 and b.ndim < 2:
        return _f32(c / _f32(b.reshape(-1)[0]))
    if b.ndim == 1:
        return _f32(c / b.min())
    if b.shape[0] == 1:
        return _f32(_f32(1) / np.floor(b[0, 0] / c))
    if b.shape[0] == 2:
        xx, yy = b[0, 0], b[1, 1]
        xy = _f32(b[0, 1] / yy)
        nx = _f32(xx / np.sqrt(_f32(1) + xy * xy))
        nmin = np.floor(min(nx, yy) / c)
    elif b.shape[0] == 3:
        xx, yy, zz = b[0, 0], b[1, 1], b[2, 2]
        xy, xz, yz = _f32(b[0, 1] / yy), _f32(b[0, 2] / zz), _f32(b[1, 2] / zz)
        nx = _f32(xx / np.sqrt(_f32(1) + xy * xy + (xy * yz - xz) ** 2))
        ny = _f32(yy / np.sqrt(_f32(1) + yz * yz))
        nmin = np.floor(min(nx, ny, zz) / c)
    else:
        raise ValueError(f'Expected box to be either 1-, 2-, or 3-dimensional found {b.shape[0]}')
    nmin = _f32(1) if nmin == 0 else _f32(nmin)
    return _f32(_f32(1) / nmin)


def _cell_size(box, minimum_cell_size):
    """partition.py:589-592: box / floor(box / minimum)."""
    return _f32(_f32(box) / np.floor(_f32(box) / _f32(minimum_cell_size)))


def _space_struct(displacement, dim, box, cell=None) -> N.Space:
    """Kernel geometry of a list: ``box`` is the list's box argument; for a
    periodic_general displacement ``cell`` (the ``box`` keyword of a call)
    replaces the displacement's own cell."""
    geo = _space.geometry_of(displacement)
    if isinstance(geo, _space.GeneralDisplacement):
        return geo.space(dim, box=cell)
    s = N.Space()
    s.dim = dim
    s.periodic = 1 if geo.periodic else 0
    b = _box_list(box if box is not None else geo.box, dim)
    for d in range(dim):
        s.box[d] = b[d]
    return s


# -------------------------------------------------------------- cell list --
@dataclasses.dataclass
class CellList:
    """partition.py:78-133."""
    position_buffer: torch.Tensor
    id_buffer: torch.Tensor
    particle_cell_id: torch.Tensor
    named_buffer: dict
    did_buffer_overflow: torch.Tensor
    cell_capacity: int
    cell_size: object
    update_fn: Callable

    def update(self, position, **kwargs):
        return self.update_fn(position, self, **kwargs)

    @property
    def kwarg_buffers(self):
        return self.named_buffer


@dataclasses.dataclass
class CellListFns:
    allocate: Callable
    update: Callable

    def __iter__(self):
        return iter((self.allocate, self.update))


def _cell_nl(dim, box, minimum_cell_size, cap, periodic=True) -> N.NList:
    cps, cs, count = cell_dimensions(dim, box, minimum_cell_size)
    nl = N.NList()
    nl.space.dim = dim
    nl.space.periodic = 1 if periodic else 0
    for d, b in enumerate(_box_list(box, dim)):
        nl.space.box[d] = b
    nl.use_cell_list = 1
    for d in range(dim):
        nl.cells_per_side[d] = int(cps[d])
        nl.cell_size[d] = float(cs[d])
    nl.cell_capacity = int(cap)
    nl.format = N.DENSE
    nl.mask_self = 1
    nl.max_occupancy = 0
    return nl


def _max_filling(R, rs, nl) -> int:
    n = R.shape[0]
    count = 1
    for d in range(nl.space.dim):
        count *= nl.cells_per_side[d]
    L = N.lib()
    ws = N.workspace(L.jmd_cell_workspace_bytes(n, count), R.device, 'cells')
    out = torch.zeros((), dtype=torch.int32, device=R.device)
    N.check(L.jmd_cell_max_filling(R.data_ptr(), rs, n, C_ref(nl), out.data_ptr(), ws.data_ptr(),
                                   ws.numel(), N.stream_ptr()), 'cell_max_filling')
    return int(out)


def C_ref(s):
    import ctypes
    return ctypes.byref(s)


def cell_list(box_size, minimum_cell_size, buffer_size_multiplier: float = 1.25) -> CellListFns:
    """partition.cell_list (partition.py:296-488)."""

    def build(position, capacity, overflow_in, kwargs):
        R, rs = _rows(position)
        n, dim = R.shape
        if dim not in (2, 3):
            raise ValueError(f'Cell list spatial dimension must be 2 or 3. Found {dim}.')
        cps, cs, count = cell_dimensions(dim, box_size, minimum_cell_size)
        if isinstance(box_size, (list, tuple, np.ndarray, torch.Tensor)) and np.ndim(
                np.asarray(box_size.cpu() if isinstance(box_size, torch.Tensor) else box_size)) >= 1:
            if np.any(cps < 3):
                raise ValueError('Box must be at least 3x the size of the grid spacing in each '
                                 'dimension.')
        nl = _cell_nl(dim, box_size, minimum_cell_size, max(capacity, 1))
        if capacity is None:
            pass
        cap = nl.cell_capacity
        dev = R.device
        ids = torch.empty(count * cap, dtype=torch.int32, device=dev)
        pos = torch.empty(count * cap * dim, dtype=torch.float32, device=dev)
        pcid = torch.empty((n, dim), dtype=torch.int32, device=dev)
        err = torch.zeros((), dtype=torch.uint8, device=dev)
        L = N.lib()
        ws = N.workspace(L.jmd_cell_workspace_bytes(n, count), dev, 'cells')
        N.check(L.jmd_cell_list_build(R.data_ptr(), rs, n, C_ref(nl), ids.data_ptr(), pos.data_ptr(),
                                      pcid.data_ptr(), err.data_ptr(), ws.data_ptr(), ws.numel(),
                                      N.stream_ptr()), 'cell_list')
        cells = tuple(int(c) for c in cps[::-1])
        id_buffer = ids.reshape(cells + (cap, 1))
        position_buffer = pos.reshape(cells + (cap, dim))
        named = {}
        flat_ids = ids.long()
        for k, v in kwargs.items():
            if not isinstance(v, torch.Tensor):
                raise ValueError(f'Data must be specified as an ndarray. Found "{k}" with type {type(v)}.')
            if v.shape[0] != n:
                raise ValueError(f'Data must be specified per-particle (an ndarray with shape ({n}, ...)).'
                                 f' Found "{k}" with shape {tuple(v.shape)}.')
            vv = v.reshape(n, -1) if v.dim() > 1 else v.reshape(n, 1)
            padv = torch.cat([vv, torch.full((1, vv.shape[1]), 10 ** 5, dtype=vv.dtype, device=dev)])
            named[k] = padv[flat_ids].reshape(cells + (cap, vv.shape[1]))
        overflow = (err & N.CELL_LIST_OVERFLOW) != 0
        if overflow_in is not None:
            overflow = overflow | torch.as_tensor(overflow_in, device=dev)
        cs_out = float(cs[0]) if np.ndim(np.asarray(box_size)) == 0 else cs
        return CellList(position_buffer, id_buffer, pcid, named, overflow, cap, cs_out, update_fn)

    def allocate_fn(position, extra_capacity: int = 0, **kwargs):
        R, rs = _rows(position)
        n, dim = R.shape
        nl = _cell_nl(dim, box_size, minimum_cell_size, 1)
        cap = int(_max_filling(R, rs, nl) * buffer_size_multiplier) + extra_capacity
        return build(R, cap, None, kwargs)

    def update_fn(position, cl_or_capacity, **kwargs):
        if isinstance(cl_or_capacity, int):
            return build(position, int(cl_or_capacity), None, kwargs)
        cl = cl_or_capacity
        return build(position, cl.cell_capacity, cl.did_buffer_overflow, kwargs)

    return CellListFns(allocate_fn, update_fn)


# --------------------------------------------------------- neighbour list --
@dataclasses.dataclass
class _Plan:
    """Static configuration and device scratch shared by a list and its updates."""
    nl: N.NList
    dim: int
    n: int
    threshold_sq: float
    always_rebuild: bool
    workspace: torch.Tensor
    occupancy: torch.Tensor    # int64 device scalar
    flag: torch.Tensor         # int32 device rebuild flag (0 between calls)
    count: Optional[torch.Tensor]  # Dense per-atom counts (int32 [N])
    ld: int
    space0: Optional[N.Space] = None  # the geometry without a box keyword


@dataclasses.dataclass
class NeighborList:
    """partition.py:684-737.

    ``idx`` may be built lazily: a device run that keeps its own private list
    (simulate.run) leaves the caller's list unbuilt and records here how to
    build it at ``reference_position``; reading ``idx`` (or updating the list)
    builds it first, so a caller that never reads it never pays for it."""
    idx: torch.Tensor
    reference_position: torch.Tensor
    error: PartitionError
    cell_list_capacity: Optional[int]
    max_occupancy: int
    format: NeighborListFormat
    cell_size: Optional[float]
    cell_list_fn: Optional[object]
    update_fn: Callable
    plan: Optional[_Plan] = None

    def __getattribute__(self, name):
        if name == 'idx':
            d = object.__getattribute__(self, '__dict__')
            pending = d.get('_pending')
            if pending is not None:
                d['_pending'] = None
                pending()
        return object.__getattribute__(self, name)

    def set_pending_build(self, build: Optional[Callable]) -> None:
        """Records (or clears) a deferred build of ``idx``."""
        object.__setattr__(self, '_pending', build)

    @property
    def has_pending_build(self) -> bool:
        return object.__getattribute__(self, '__dict__').get('_pending') is not None

    def idx_buffer(self) -> torch.Tensor:
        """``idx`` without running a pending build (for kernels that only
        write it)."""
        return object.__getattribute__(self, 'idx')

    def update(self, position, **kwargs) -> 'NeighborList':
        return self.update_fn(position, self, **kwargs)

    @property
    def did_buffer_overflow(self) -> torch.Tensor:
        return self.error.code & (PEC.NEIGHBOR_LIST_OVERFLOW | PEC.CELL_LIST_OVERFLOW)

    @property
    def cell_size_too_small(self) -> torch.Tensor:
        return self.error.code & PEC.CELL_SIZE_TOO_SMALL

    @property
    def malformed_box(self) -> torch.Tensor:
        return self.error.code & PEC.MALFORMED_BOX

    @property
    def nbr_count(self) -> Optional[torch.Tensor]:
        """Per-atom neighbour counts of a Dense list (kernel side data)."""
        return self.plan.count if self.plan is not None else None


@dataclasses.dataclass
class NeighborListFns:
    """partition.py:740-785."""
    allocate: Callable
    update: Callable

    def __call__(self, position, neighbors=None, extra_capacity: int = 0, **kwargs):
        if neighbors is None:
            return self.allocate(position, extra_capacity, **kwargs)
        return self.update(position, neighbors, **kwargs)

    def __iter__(self):
        return iter((self.allocate, self.update))


def _row_ld(width: int) -> int:
    """Dense row stride: a multiple of 8 int32 so rows start on 32-byte sectors."""
    return max(8, (width + 7) // 8 * 8)


def _run_build(plan: '_Plan', R, rs, idx, ld, error, ref, use_flag):
    """One jmd_neighbor_list_build of `plan` at positions R (row stride rs)."""
    L = N.lib()
    cnt = plan.count
    N.check(L.jmd_neighbor_list_build(
        C_ref(plan.nl), R.data_ptr(), rs, plan.n, N.ptr(idx), ld, N.ptr(cnt),
        plan.occupancy.data_ptr(), N.ptr(error), N.ptr(ref),
        ref.stride(0) if ref is not None else 0,
        plan.flag.data_ptr() if use_flag else None,
        plan.workspace.data_ptr(), plan.workspace.numel(), N.stream_ptr()), 'neighbor_list')


def build_at_reference(neighbors: 'NeighborList') -> None:
    """Builds a Dense list in place at its own reference positions (the list
    the reference would hold after its last rebuild), in the reference's
    entry order."""
    plan = neighbors.plan
    ref = neighbors.reference_position
    _run_build(plan, ref, ref.stride(0), neighbors.idx_buffer(), plan.ld, neighbors.error.code,
               ref, False)


def neighbor_list(displacement_or_metric, box, r_cutoff, dr_threshold=0.0,
                  capacity_multiplier: float = 1.25, disable_cell_list: bool = False,
                  mask_self: bool = True, custom_mask_function: Optional[Callable] = None,
                  fractional_coordinates: bool = False, format: NeighborListFormat = Dense,
                  **static_kwargs) -> NeighborListFns:
    """partition.neighbor_list (partition.py:801-1164)."""
    is_format_valid(format)
    if custom_mask_function is not None:
        raise NotImplementedError('custom_mask_function is not supported by the GB300 neighbour '
                                  'list kernels')
    general = isinstance(_space.geometry_of(displacement_or_metric), _space.GeneralDisplacement)
    r_cutoff = float(torch.as_tensor(r_cutoff).max()) if isinstance(r_cutoff, torch.Tensor) else r_cutoff
    dr_threshold = float(dr_threshold)
    always_rebuild = dr_threshold == 0
    # partition.py:880-884, float32 arithmetic of the reference's run
    cutoff = _f32(_f32(r_cutoff) + _f32(dr_threshold))
    cutoff_sq = _f32(cutoff * cutoff)
    threshold_sq = _f32((_f32(dr_threshold) / _f32(2)) ** 2)
    fmt_code = {Dense: N.DENSE, Sparse: N.SPARSE, OrderedSparse: N.ORDERED_SPARSE}[format]

    def cell_grid(dim, cell_box):
        """(use_cells, minimum cell size, binning box) as partition.py:1044-1054."""
        if disable_cell_list:
            return False, None, None
        if fractional_coordinates:
            fcs = fractional_cell_size(cell_box, cutoff)
            return bool(fcs < _f32(1) / _f32(3)), fcs, 1.0
        if general:
            b = np.asarray(cell_box.detach().cpu() if isinstance(cell_box, torch.Tensor)
                           else cell_box, np.float64)
            if b.ndim == 2:
                # a cell matrix binned without fractional coordinates: the
                # reference's all(cutoff < box / 3) fails on its zero entries
                return False, None, None
        Lbox = np.array(_box_list(cell_box, dim), np.float32)
        return bool(np.all(cutoff < Lbox / np.float32(3.0))), cutoff, cell_box

    def make_nl(dim, use_cells, cell_cap, max_occ, cell_box=None) -> N.NList:
        nl = N.NList()
        nl.space = _space_struct(displacement_or_metric, dim, box, cell_box)
        nl.cutoff_sq = float(cutoff_sq)
        nl.use_cell_list = 1 if use_cells else 0
        if use_cells:
            _, mcs, bbox = cell_grid(dim, box if cell_box is None else cell_box)
            cps, cs, _ = cell_dimensions(dim, bbox, mcs)
            for d in range(dim):
                nl.cells_per_side[d] = int(cps[d])
                nl.cell_size[d] = float(cs[d])
            nl.cell_capacity = int(cell_cap)
        nl.format = fmt_code
        nl.mask_self = 1 if mask_self else 0
        nl.max_occupancy = int(max_occ)
        return nl

    run_build = _run_build

    def allocate_fn(position, extra_capacity: int = 0, **kwargs):
        if 'box' in kwargs and not fractional_coordinates:
            raise ValueError('Neighbor list cannot accept a box keyword argument if '
                             'fractional_coordinates is not enabled.')
        cell_box = kwargs.get('box')
        R, rs = _rows(position)
        n, dim = R.shape
        dev = R.device
        use_cells, mcs, _ = cell_grid(dim, box if cell_box is None else cell_box)
        cell_cap = None
        if use_cells:
            probe = make_nl(dim, True, 1, 0, cell_box)
            cell_cap = int(_max_filling(R, rs, probe) * capacity_multiplier) + extra_capacity
        nl = make_nl(dim, use_cells, cell_cap or 1, 2 ** 62, cell_box)
        L = N.lib()
        wsz = L.jmd_neighbor_list_workspace_bytes(C_ref(nl), n)
        plan = _Plan(nl=nl, dim=dim, n=n, threshold_sq=float(threshold_sq),
                     always_rebuild=always_rebuild,
                     workspace=torch.empty(wsz, dtype=torch.uint8, device=dev),
                     occupancy=torch.zeros((), dtype=torch.int64, device=dev),
                     flag=torch.zeros((), dtype=torch.int32, device=dev),
                     count=None, ld=0)
        # count pass (the reference's first build, partition.py:1121)
        run_build(plan, R, rs, None, 0, None, None, False)
        occupancy = int(plan.occupancy)
        # capacity rule, partition.py:1090-1104
        if use_cells:
            width = (3 ** dim) * cell_cap
        else:
            width = n
        if is_sparse(format):
            width = width * n
        extra = extra_capacity if not is_sparse(format) else n * extra_capacity
        max_occ = int(_f32(occupancy) * _f32(capacity_multiplier) + extra)
        max_occ = min(max_occ, width)
        if not is_sparse(format):
            limit = n - 1 if mask_self else n
        elif format is Sparse:
            limit = n * (n - 1) if mask_self else n * n
        else:
            limit = n * (n - 1) // 2
        max_occ = max(0, min(max_occ, limit))
        nl.max_occupancy = max_occ
        error = torch.zeros((), dtype=torch.uint8, device=dev)
        ref = padded_rows(R) if dim <= 4 else R.clone()
        if is_sparse(format):
            ld = max(max_occ, 1)
            store = torch.empty((2, ld), dtype=torch.int32, device=dev)
            idx = store[:, :max_occ]
        else:
            ld = _row_ld(max_occ)
            store = torch.empty((n, ld), dtype=torch.int32, device=dev)
            idx = store[:, :max_occ]
            plan.count = torch.zeros(n, dtype=torch.int32, device=dev)
        plan.ld = ld
        run_build(plan, R, rs, store, ld, error, ref, False)
        plan.space0 = _space_struct(displacement_or_metric, dim, box)
        return NeighborList(idx, ref, PartitionError(error), cell_cap, max_occ, format,
                            float(mcs) if use_cells else None, plan if use_cells else None,
                            update_fn, plan)

    def update_fn(position, neighbors: NeighborList, **kwargs):
        if 'box' in kwargs and not fractional_coordinates:
            raise ValueError('Neighbor list cannot accept a box keyword argument if '
                             'fractional_coordinates is not enabled.')
        plan = neighbors.plan
        if plan is None:
            raise ValueError('update needs a NeighborList made by this neighbor_list allocate')
        R, rs = _rows(position)
        if R.shape[0] != plan.n or R.shape[1] != plan.dim:
            raise ValueError('position shape changed since allocate; call allocate again')
        if 'box' in kwargs:
            # partition.py:1123-1139: the new cell must not need larger cells
            # than the list was binned with; distances use the new cell
            new_box = kwargs['box']
            if plan.nl.use_cell_list and neighbors.cell_size is not None:
                cur = _cell_size(1.0, neighbors.cell_size)
                new = _cell_size(1.0, fractional_cell_size(new_box, cutoff))
                if new > cur:
                    neighbors.error.code |= int(PEC.CELL_SIZE_TOO_SMALL)
            M = _space.cell_matrix(new_box, plan.dim)
            if not np.array_equal(np.triu(M), M):
                neighbors.error.code |= int(PEC.MALFORMED_BOX)
                raise ValueError('the kernels take upper-triangular cell matrices '
                                 '(partition.is_box_valid)')
            plan.nl.space = _space_struct(displacement_or_metric, plan.dim, box, new_box)
        elif plan.space0 is not None:
            plan.nl.space = plan.space0
        ref = neighbors.reference_position
        store = neighbors.idx
        L = N.lib()
        if plan.always_rebuild:
            run_build(plan, R, rs, store, plan.ld, neighbors.error.code, ref, False)
        else:
            s = plan.nl.space
            N.check(L.jmd_skin_check(R.data_ptr(), rs, ref.data_ptr(), ref.stride(0), plan.n,
                                     C_ref(s), plan.threshold_sq, plan.flag.data_ptr(),
                                     N.stream_ptr()), 'skin_check')
            run_build(plan, R, rs, store, plan.ld, neighbors.error.code, ref, True)
        return dataclasses.replace(neighbors)

    return NeighborListFns(allocate_fn, update_fn)


def is_box_valid(box) -> bool:
    """partition.py:676-681: scalars and side vectors are valid; a cell
    matrix must be upper triangular."""
    b = np.asarray(box.detach().cpu() if isinstance(box, torch.Tensor) else box)
    if b.ndim <= 1:
        return True
    if b.ndim == 2:
        return bool(np.all(np.triu(b) == b))
    return False


def neighbor_list_mask(neighbor: NeighborList, mask_self: bool = False) -> torch.Tensor:
    """partition.py:1167-1182."""
    if is_sparse(neighbor.format):
        mask = neighbor.idx[0] < len(neighbor.reference_position)
        if mask_self:
            mask = mask & (neighbor.idx[0] != neighbor.idx[1])
        return mask
    mask = neighbor.idx < len(neighbor.idx)
    if mask_self:
        n = len(neighbor.reference_position)
        mask = mask & (neighbor.idx != torch.arange(n, device=neighbor.idx.device,
                                                   dtype=torch.int32)[:, None])
    return mask


def to_dense(neighbor: NeighborList) -> torch.Tensor:
    """partition.py:1253-1271 (Sparse -> Dense ids)."""
    if neighbor.format is not Sparse:
        raise ValueError('Can only convert sparse neighbor lists to dense ones.')
    receivers, senders = neighbor.idx.long()
    mask = neighbor_list_mask(neighbor)
    receivers = receivers[mask]
    senders = senders[mask]
    n = len(neighbor.reference_position)
    count = torch.bincount(receivers, minlength=n)
    max_count = int(count.max()) if count.numel() else 0
    offset = torch.arange(max_count, device=receivers.device).repeat(n)[: len(senders)]
    hashes = senders * max_count + offset
    dense = torch.full((n * max_count,), n, dtype=torch.int32, device=receivers.device)
    dense[hashes] = receivers.int()
    return dense.reshape(n, max_count)
