"""FP64 CPU restatement of JAX MD's short-range MD path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``jax_md_gb300``) imports
this module; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may use it, and only to check results or as the timed CPU
baseline, never in place of a kernel.

Every function restates the reference algorithm in plain NumPy and cites the
reference file:line it follows (paths relative to the jax_md project root).
Floating-point arithmetic is float64 unless a function says otherwise; where the
reference's float32 run makes an integer decision (cell binning), the oracle
can reproduce that decision bit-for-bit in float32 (``binning_dtype``).

Parity pins for this oracle (see ``tests/test_oracle_pins.py``):
  * LAMMPS LJ fixture (tests/data/lammps_lj_stress_test{,_states}): energy per
    atom and the 6-component stress, tolerance 5e-5 (tests/quantity_test.py:436-455);
  * jammed soft-sphere fixture (tests/data/simulation_test_state.npy): pressure
    0.06307342 (tests/quantity_test.py:134-150) and its stored energy;
  * closed forms of tests/energy_test.py:284-342,479-520,533-562 (LJ, soft
    sphere, Morse, the cutoff);
  * periodic_general identities of tests/space_test.py:302-350,456-600;
  * per-particle parameters, neighbour list = all pairs
    (tests/smap_test.py:1308-1340);
  * Langevin (BAOAB): the damped oscillator's mean position and momentum
    autocorrelation and the equilibrium temperature
    (tests/simulate_test.py:827-915, statistical);
  * capacity / overflow shapes of tests/partition_test.py:363-401,489-546.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

# ---------------------------------------------------------------------------
# Error codes: jax_md/partition.py:494-520 (PartitionErrorCode).
NEIGHBOR_LIST_OVERFLOW = 1
CELL_LIST_OVERFLOW = 2
CELL_SIZE_TOO_SMALL = 4
MALFORMED_BOX = 8

DENSE, SPARSE, ORDERED_SPARSE = 0, 1, 2


# ---------------------------------------------------------------------------
# space.py
def periodic_displacement(side, dR):
    """jax_md/space.py:213-224: mod(dR + L/2, L) - L/2 (floored mod)."""
    side = np.asarray(side, np.float64)
    return np.mod(dR + side * 0.5, side) - 0.5 * side


def periodic_shift(side, R, dR):
    """jax_md/space.py:250-252: mod(R + dR, L)."""
    return np.mod(R + dR, side)


def displacement(Ra, Rb, box=None):
    """Displacement Ra - Rb (free) or wrapped (periodic), space.py:275-329;
    `box` may also be a space object with a displacement method
    (PeriodicGeneral)."""
    if hasattr(box, 'displacement'):
        return box.displacement(Ra, Rb)
    dR = np.asarray(Ra, np.float64) - np.asarray(Rb, np.float64)
    if box is None:
        return dR
    return periodic_displacement(box, dR)


def transform(box, R):
    """space.py:125-148 (raw_transform): R * box for a scalar or a vector of
    sides, R @ box^T for a matrix (x = T u row by row)."""
    b = np.asarray(box, np.float64)
    R = np.asarray(R, np.float64)
    if b.size == 1 or b.ndim == 1:
        return R * b.reshape(-1) if b.ndim == 1 else R * b.item()
    return np.einsum('ij,...j->...i', b, R)


def inverse(box):
    """space.py:109-119."""
    b = np.asarray(box, np.float64)
    return np.linalg.inv(b) if b.ndim == 2 else 1.0 / b


@dataclass
class PeriodicGeneral:
    """space.periodic_general (space.py:332-468): periodic parallelepiped
    X = T [0, 1]^d.  With fractional_coordinates positions live in the unit
    cube and displacements are T d_U(u, v); otherwise positions live in X and
    are mapped to the cube by T^-1 first.  d_U wraps each component with
    mod(d + 1/2, 1) - 1/2 (space.py:205-216).  The keyword `box` replaces T
    (and, for real coordinates, T^-1); `new_box` replaces T only, which
    deforms real-coordinate displacements (space.py:417-429)."""
    box: object
    fractional_coordinates: bool = True
    wrapped: bool = True

    def displacement(self, Ra, Rb, box=None, new_box=None):
        T, Ti = self.box, inverse(self.box)
        if box is not None:
            T = box
            if not self.fractional_coordinates:
                Ti = inverse(box)
        if new_box is not None:
            T = new_box
        Ra = np.asarray(Ra, np.float64)
        Rb = np.asarray(Rb, np.float64)
        if not self.fractional_coordinates:
            Ra, Rb = transform(Ti, Ra), transform(Ti, Rb)
        return transform(T, periodic_displacement(1.0, Ra - Rb))

    def shift(self, R, dR, box=None, new_box=None):
        """space.py:439-466: dR lives in X; R in U (fractional) or X."""
        R = np.asarray(R, np.float64)
        dR = np.asarray(dR, np.float64)
        if not self.fractional_coordinates and not self.wrapped:
            return R + dR
        T, Ti = self.box, inverse(self.box)
        if box is not None:
            T, Ti = box, inverse(box)
        if new_box is not None:
            T = new_box
        dR = transform(Ti, dR)
        if not self.fractional_coordinates:
            R = transform(Ti, R)
        R = np.mod(R + dR, 1.0) if self.wrapped else R + dR
        if not self.fractional_coordinates:
            R = transform(T, R)
        return R


# ---------------------------------------------------------------------------
# partition.py: cell list
def _box_vector(box, dim):
    b = np.asarray(box)
    if b.ndim == 0:
        return np.full(dim, b.item())
    return b.reshape(-1)[:dim]


def cell_dimensions(box, minimum_cell_size, dim, dtype=np.float32):
    """jax_md/partition.py:146-188 (_cell_dimensions), arithmetic in ``dtype``.

    Returns (cells_per_side[dim] int, cell_size[dim] dtype, cell_count)."""
    L = _box_vector(box, dim).astype(dtype)
    m = dtype(minimum_cell_size)
    cps = np.floor(L / m)
    cell_size = (L / cps).astype(dtype)
    cps = cps.astype(np.int64)
    if np.asarray(box).ndim >= 1 and np.any(cps < 3):
        raise ValueError('Box must be at least 3x the size of the grid spacing in each dimension.')
    return cps, cell_size, int(np.prod(cps))


def fractional_cell_size(box, cutoff, dtype=np.float32):
    """jax_md/partition.py:595-634 (_fractional_cell_size): the unit-cube
    cell edge whose perpendicular width in the cell T is >= cutoff, in
    ``dtype``: 1 / floor(min perpendicular width / cutoff) for a matrix."""
    b = np.asarray(box, dtype)
    c = dtype(cutoff)
    if b.ndim == 0:
        return dtype(c / b)
    if b.ndim == 1:
        return dtype(c / b.min())
    if b.shape[0] == 1:
        return dtype(1 / np.floor(b[0, 0] / c))
    if b.shape[0] == 2:
        xy = dtype(b[0, 1] / b[1, 1])
        widths = [dtype(b[0, 0] / np.sqrt(dtype(1) + xy * xy)), b[1, 1]]
    else:
        xy, xz, yz = (dtype(b[0, 1] / b[1, 1]), dtype(b[0, 2] / b[2, 2]),
                      dtype(b[1, 2] / b[2, 2]))
        widths = [dtype(b[0, 0] / np.sqrt(dtype(1) + xy * xy + (xy * yz - xz) ** 2)),
                  dtype(b[1, 1] / np.sqrt(dtype(1) + yz * yz)), b[2, 2]]
    nmin = np.floor(min(widths) / c)
    nmin = dtype(1) if nmin == 0 else dtype(nmin)
    return dtype(dtype(1) / nmin)


def cell_index(R, cell_size, cps, dtype=np.float32):
    """jax_md/partition.py:421-423: int(x / cell_size) mod cells_per_side.

    The reference's float32 run divides in float32 and truncates toward zero."""
    q = (np.asarray(R, dtype) / cell_size.astype(dtype)).astype(np.int32).astype(np.int64)
    return np.mod(q, cps)


def cell_hash(idx3, cps):
    """jax_md/partition.py:212-224 (_compute_hash_constants): x fastest."""
    mult = np.cumprod(np.concatenate([[1], cps[:-1]])).astype(np.int64)
    return (idx3 * mult[None, :]).sum(axis=1)


def estimate_cell_capacity(R, box, cell_min, multiplier, dim, dtype=np.float32):
    """jax_md/partition.py:191-209,243-250."""
    cps, cs, count = cell_dimensions(box, cell_min, dim, dtype)
    h = cell_hash(cell_index(R, cs, cps, dtype), cps)
    filling = np.bincount(h, minlength=count)
    return int(filling.max() * multiplier)


@dataclass
class CellListO:
    id_buffer: np.ndarray          # [count, cap] int64 (flat cell hash major)
    position_buffer: np.ndarray    # [count, cap, dim]
    particle_cell_id: np.ndarray   # [N, dim]
    did_buffer_overflow: bool
    cell_capacity: int
    cells_per_side: np.ndarray
    cell_size: np.ndarray


def cell_list(R, box, cell_min, capacity, dtype=np.float32):
    """jax_md/partition.py:349-471 (cell_list_fn).

    Slot rule (partition.py:438-447): atoms sorted stably by hash; the atom at
    sorted position s goes to slot hash*cap + (s mod cap)."""
    R = np.asarray(R)
    N, dim = R.shape
    cps, cs, count = cell_dimensions(box, cell_min, dim, dtype)
    idx = cell_index(R, cs, cps, dtype)
    h = cell_hash(idx, cps)
    order = np.argsort(h, kind='stable')
    slot = h[order] * capacity + (np.arange(N) % capacity)
    ids = np.full(count * capacity, N, np.int64)
    pos = np.zeros((count * capacity, dim), R.dtype)
    ids[slot] = order
    pos[slot] = R[order]
    occ = np.bincount(h, minlength=count)
    return CellListO(ids.reshape(count, capacity), pos.reshape(count, capacity, dim),
                     idx, bool(occ.max() > capacity), capacity, cps, cs)


def neighboring_cells(dim):
    """jax_md/partition.py:232-240 (_neighboring_cells_arr): first axis slowest."""
    g = np.stack(np.meshgrid(*([np.arange(3)] * dim), indexing='ij'), axis=-1)
    return g.reshape(-1, dim) - 1


# ---------------------------------------------------------------------------
# partition.py: neighbour list
@dataclass
class NeighborListO:
    idx: np.ndarray
    reference_position: np.ndarray
    error: int
    cell_list_capacity: Optional[int]
    max_occupancy: int
    format: int
    use_cell_list: bool
    occupancy: int = 0


class NeighborListOracle:
    """Restates jax_md/partition.py:801-1164 (neighbor_list) for one box.

    ``box=None`` means free space (space.free): no minimum image; the cell list
    still bins with ``cell_box`` (partition.py:1044-1054 uses ``box``).
    ``space`` (a PeriodicGeneral) replaces the displacement; with
    ``fractional`` the cell list bins the unit cube with the cell edge of
    fractional_cell_size(box, cutoff) (partition.py:1046-1051)."""

    def __init__(self, box, r_cutoff, dr_threshold=0.0, capacity_multiplier=1.25,
                 disable_cell_list=False, mask_self=True, fmt=DENSE,
                 periodic=True, binning_dtype=np.float32, space=None, fractional=False):
        self.box = np.asarray(box, np.float64)
        self.periodic = periodic
        self.space = space
        self.r_cutoff = float(r_cutoff)
        self.dr_threshold = float(dr_threshold)
        self.cutoff = self.r_cutoff + self.dr_threshold
        self.cutoff_sq = self.cutoff ** 2
        self.threshold_sq = (self.dr_threshold / 2.0) ** 2
        self.capacity_multiplier = capacity_multiplier
        self.disable_cell_list = disable_cell_list
        self.mask_self = mask_self
        self.fmt = fmt
        self.bdt = binning_dtype
        if fractional:
            self.bin_box = np.float64(1.0)
            self.bin_min = float(fractional_cell_size(box, self.cutoff, binning_dtype))
        else:
            self.bin_box, self.bin_min = self.box, self.cutoff

    # d^2 between every candidate, partition.py:911-951 / 960-975.
    def _d2(self, Ri, Rj):
        d = displacement(Ri, Rj, self.space if self.space is not None else
                         (self.box if self.periodic else None))
        return (d * d).sum(-1)

    def _candidates(self, R, cl):
        """[N, W] candidate ids (sentinel N) before distance/self masks."""
        N, dim = R.shape
        if cl is None:  # partition.py:893-898 candidate_fn
            return np.broadcast_to(np.arange(N)[None, :], (N, N)).copy(), False
        shifts = neighboring_cells(dim)
        cps = cl.cells_per_side
        shifted = np.mod(cl.particle_cell_id[:, None, :] + shifts[None], cps)
        mult = np.cumprod(np.concatenate([[1], cps[:-1]]))
        cell1d = (shifted * mult).sum(-1)                        # [N, 3^d]
        cand = cl.id_buffer[cell1d].reshape(N, -1)               # [N, 3^d*cap]
        return cand, True

    def build(self, R, max_occupancy=None, err=0, cl_capacity=None,
              extra_capacity=0, use_cell_list=None):
        R = np.asarray(R)
        N, dim = R.shape
        cl = None
        if use_cell_list is None:
            use_cell_list = (not self.disable_cell_list) and bool(
                np.all(self.bin_min < _box_vector(self.bin_box, dim) / 3.0))
        if use_cell_list:
            if cl_capacity is None:
                cl_capacity = estimate_cell_capacity(
                    R, self.bin_box, self.bin_min, self.capacity_multiplier, dim,
                    self.bdt) + extra_capacity
            cl = cell_list(R, self.bin_box, self.bin_min, cl_capacity, self.bdt)
            if cl.did_buffer_overflow:
                err |= CELL_LIST_OVERFLOW
        cand, _ = self._candidates(R, cl)
        # distance mask (partition.py:951 strict '<')
        valid = cand < N
        safe = np.where(valid, cand, 0)
        d2 = self._d2(R[:, None, :], R[safe])
        mask = valid & (d2 < self.cutoff_sq)
        if self.mask_self:                                       # :953-958
            mask &= cand != np.arange(N)[:, None]
        if self.fmt == DENSE:                                    # :960-977
            counts = mask.sum(1)
            occupancy = int(counts.max()) if N else 0
            width = cand.shape[1]
            out = np.full((N, width), N, np.int64)
            for i in range(N):
                sel = cand[i][mask[i]]
                out[i, :len(sel)] = sel
        else:                                                    # :979-1032
            if self.fmt == ORDERED_SPARSE:
                mask &= cand < np.arange(N)[:, None]
            rows = np.broadcast_to(np.arange(N)[:, None], cand.shape)
            recv = cand[mask]
            send = rows[mask]
            occupancy = int(mask.sum())
            width = cand.size
            out = np.full((2, width), N, np.int64)
            out[0, :occupancy] = recv
            out[1, :occupancy] = send
        if max_occupancy is None:                                # :1090-1104
            extra = extra_capacity if self.fmt == DENSE else N * extra_capacity
            max_occupancy = int(np.float32(occupancy) * np.float32(self.capacity_multiplier)
                                + extra)
            max_occupancy = min(max_occupancy, width)
            if self.fmt == DENSE:
                limit = N - 1 if self.mask_self else N
            elif self.fmt == SPARSE:
                limit = N * (N - 1) if self.mask_self else N * N
            else:
                limit = N * (N - 1) // 2
            max_occupancy = min(max_occupancy, limit)
        if occupancy > max_occupancy:
            err |= NEIGHBOR_LIST_OVERFLOW
        out = out[..., :max_occupancy] if out.shape[-1] >= max_occupancy else np.pad(
            out, [(0, 0), (0, max_occupancy - out.shape[-1])], constant_values=N)
        return NeighborListO(out, R.copy(), err, cl_capacity, max_occupancy,
                             self.fmt, use_cell_list, occupancy)

    def dense_rows(self, R, atoms, cl_capacity):
        """Dense rows of `atoms` only, in the reference's entry order
        (partition.py:911-977 restricted to those rows): the cell list of all
        atoms, then the candidates, masks and compaction of the chosen rows.
        For systems too large for build()'s [N, 3^d cap] candidate array.
        Returns (rows [len(atoms), 3^d cap] with sentinel N, counts)."""
        R = np.asarray(R)
        N, dim = R.shape
        atoms = np.asarray(atoms, np.int64)
        cl = cell_list(R, self.bin_box, self.bin_min, cl_capacity, self.bdt)
        shifts = neighboring_cells(dim)
        cps = cl.cells_per_side
        shifted = np.mod(cl.particle_cell_id[atoms][:, None, :] + shifts[None], cps)
        mult = np.cumprod(np.concatenate([[1], cps[:-1]]))
        cand = cl.id_buffer[(shifted * mult).sum(-1)].reshape(len(atoms), -1)
        valid = cand < N
        d2 = self._d2(R[atoms][:, None, :], R[np.where(valid, cand, 0)])
        mask = valid & (d2 < self.cutoff_sq)
        if self.mask_self:
            mask &= cand != atoms[:, None]
        out = np.full(cand.shape, N, np.int64)
        for k in range(len(atoms)):
            sel = cand[k][mask[k]]
            out[k, :len(sel)] = sel
        return out, mask.sum(1)

    def allocate(self, R, extra_capacity=0):
        return self.build(R, extra_capacity=extra_capacity)

    def update(self, R, nbrs: NeighborListO):
        """partition.py:1141-1154: rebuild iff any |R - R_ref|^2 > (skin/2)^2."""
        if self.dr_threshold != 0.0:
            d = displacement(R, nbrs.reference_position, self.space if self.space is not None
                             else (self.box if self.periodic else None))
            if not np.any((d * d).sum(-1) > self.threshold_sq):
                return nbrs
        return self.build(R, nbrs.max_occupancy, nbrs.error, nbrs.cell_list_capacity,
                          use_cell_list=nbrs.use_cell_list)


def did_buffer_overflow(err):
    """partition.py:725-729."""
    return bool(err & (NEIGHBOR_LIST_OVERFLOW | CELL_LIST_OVERFLOW))


def neighbor_sets(nbrs: NeighborListO, N):
    """Per-atom sorted neighbour id lists (for order-free comparisons)."""
    out = [[] for _ in range(N)]
    if nbrs.format == DENSE:
        for i in range(N):
            out[i] = sorted(int(j) for j in nbrs.idx[i] if j < N)
    else:
        for j, i in zip(nbrs.idx[0], nbrs.idx[1]):
            if j < N:
                out[int(i)].append(int(j))
        out = [sorted(s) for s in out]
    return out


# ---------------------------------------------------------------------------
# energy.py: pair potentials (f64), with analytic dU/dr and d2U/dr2.
def multiplicative_cutoff(r, r_onset, r_cutoff):
    """jax_md/energy.py:534-580: S(r) and dS/dr, d2S/dr2."""
    rc2, ro2 = r_cutoff ** 2, r_onset ** 2
    r2 = r * r
    den = (rc2 - ro2) ** 3
    inner = (rc2 - r2) ** 2 * (rc2 + 2 * r2 - 3 * ro2) / den
    # d/dr of inner: d/dr2 * 2r
    # f(u)= (rc2-u)^2 (rc2+2u-3ro2)/den ; f'(u) = [-2(rc2-u)(rc2+2u-3ro2) + 2(rc2-u)^2]/den
    fu = (-2 * (rc2 - r2) * (rc2 + 2 * r2 - 3 * ro2) + 2 * (rc2 - r2) ** 2) / den
    # f''(u) = [2(rc2+2u-3ro2) - 4(rc2-u) - 4(rc2-u)]/den
    fuu = (2 * (rc2 + 2 * r2 - 3 * ro2) - 8 * (rc2 - r2)) / den
    dS = fu * 2 * r
    d2S = fuu * 4 * r2 + fu * 2
    S = np.where(r < r_onset, 1.0, np.where(r < r_cutoff, inner, 0.0))
    dS = np.where(r < r_onset, 0.0, np.where(r < r_cutoff, dS, 0.0))
    d2S = np.where(r < r_onset, 0.0, np.where(r < r_cutoff, d2S, 0.0))
    return S, dS, d2S


def lennard_jones(r, sigma=1.0, epsilon=1.0):
    """jax_md/energy.py:246-272: 4 eps ((s/r)^12 - (s/r)^6), with U', U''."""
    with np.errstate(divide='ignore', invalid='ignore', over='ignore'):
        ir = sigma / r
        i6 = ir ** 6
        i12 = i6 * i6
        U = 4 * epsilon * (i12 - i6)
        dU = 4 * epsilon * (-12 * i12 + 6 * i6) / r
        d2U = 4 * epsilon * (156 * i12 - 42 * i6) / (r * r)
    return np.nan_to_num(U), np.nan_to_num(dU), np.nan_to_num(d2U)


def lennard_jones_sigma_eps_derivs(r, sigma, epsilon):
    """dU/dsigma, dU/depsilon of the bare LJ term (for the parameter adjoint)."""
    ir = sigma / r
    i6 = ir ** 6
    i12 = i6 * i6
    dUds = 4 * epsilon * (12 * i12 - 6 * i6) / sigma
    dUde = 4 * (i12 - i6)
    return dUds, dUde


def soft_sphere(r, sigma=1.0, epsilon=1.0, alpha=2.0):
    """jax_md/energy.py:125-173: eps/alpha (1 - r/sigma)^alpha for r < sigma."""
    x = r / sigma
    inside = x < 1.0
    base = np.where(inside, 1.0 - x, 0.0)
    U = np.where(inside, epsilon / alpha * base ** alpha, 0.0)
    dU = np.where(inside, -epsilon / sigma * base ** (alpha - 1.0), 0.0)
    d2U = np.where(inside, epsilon * (alpha - 1.0) / sigma ** 2 * base ** (alpha - 2.0), 0.0)
    return U, dU, d2U


def morse(r, sigma=1.0, epsilon=5.0, alpha=5.0):
    """jax_md/energy.py:346-371: eps (1 - exp(-alpha (r - sigma)))^2 - eps, the
    minimum -eps at r = sigma; with U', U''."""
    e = np.exp(-alpha * (r - sigma))
    U = epsilon * (1.0 - e) ** 2 - epsilon
    dU = 2.0 * epsilon * alpha * e * (1.0 - e)
    d2U = 2.0 * epsilon * alpha ** 2 * e * (2.0 * e - 1.0)
    return U, dU, d2U


@dataclass
class PairSpec:
    """Which potential and its parameters (scalar or [S,S] species matrices).
    For 'morse' the radii are absolute (energy.py:374-440), not multiples of
    max sigma."""
    kind: str = 'lj'                 # 'lj' | 'lj_truncated' | 'soft_sphere' | 'morse'
    sigma: object = 1.0
    epsilon: object = 1.0
    alpha: object = 2.0
    r_onset: float = 2.0             # multiplied by max sigma (energy.py:319-320)
    r_cutoff: float = 2.5
    per_pair_cutoff: bool = False    # r_on/r_c scaled by sigma_ij instead of max sigma
    species: Optional[np.ndarray] = None

    def params(self, si, sj, ai=None, aj=None):
        """Per-pair parameters: scalars as they are, [S,S] matrices by the
        species of the two atoms, and per-particle [N] arrays combined as
        0.5 (p_i + p_j) from the atom indices ai, aj (the default combinator,
        smap.py:833-838 with smap.py:704-713)."""
        def look(p):
            p = np.asarray(p, np.float64)
            if p.ndim == 1:
                if ai is None:
                    raise ValueError('per-particle parameters need the atom indices')
                return 0.5 * (p[ai] + p[aj])
            if p.ndim == 0 or self.species is None:
                return p
            return p[si, sj]
        return look(self.sigma), look(self.epsilon), look(self.alpha)

    def max_sigma(self):
        return float(np.max(np.asarray(self.sigma)))


def pair_terms(spec: PairSpec, r, si=None, sj=None, ai=None, aj=None):
    """U, U', U'' per pair (f64); si / sj species, ai / aj atom indices of the
    pairs (for per-particle parameters)."""
    sig, eps, alp = spec.params(si, sj, ai, aj)
    if spec.kind == 'soft_sphere':
        return soft_sphere(r, sig, eps, alp)
    if spec.kind == 'morse':
        # morse_pair / morse_neighbor_list: multiplicative_isotropic_cutoff
        # with the radii as given (energy.py:388-389, 434-435)
        U, dU, d2U = morse(r, sig, eps, alp)
        S, dS, d2S = multiplicative_cutoff(r, spec.r_onset, spec.r_cutoff)
        return U * S, dU * S + U * dS, d2U * S + 2 * dU * dS + U * d2S
    U, dU, d2U = lennard_jones(r, sig, eps)
    if spec.kind == 'lj_truncated':
        ms = spec.max_sigma()
        m = r < spec.r_cutoff * ms
        return np.where(m, U, 0.0), np.where(m, dU, 0.0), np.where(m, d2U, 0.0)
    if spec.per_pair_cutoff:
        ro, rc = spec.r_onset * sig, spec.r_cutoff * sig
    else:
        ms = spec.max_sigma()
        ro, rc = spec.r_onset * ms, spec.r_cutoff * ms
    S, dS, d2S = multiplicative_cutoff(r, ro, rc)
    return U * S, dU * S + U * dS, d2U * S + 2 * dU * dS + U * d2S


def pair_force_abs_sum(spec: PairSpec, R, nbrs_idx, fmt, box=None):
    """Per-atom sum over its pairs of |F_ij|: the scale of the rounding error
    an fp32 force sum can carry (the condition number of the sum)."""
    R = np.asarray(R, np.float64)
    N = R.shape[0]
    if fmt == DENSE:
        i = np.repeat(np.arange(N), nbrs_idx.shape[1])
        j = nbrs_idx.reshape(-1)
    else:
        j, i = nbrs_idx[0], nbrs_idx[1]
    m = j < N
    i, j = i[m], j[m]
    dR = displacement(R[j], R[i], box)
    r = np.sqrt((dR * dR).sum(-1))
    si = spec.species[i] if spec.species is not None else None
    sj = spec.species[j] if spec.species is not None else None
    _, dU, _ = pair_terms(spec, r, si, sj, i, j)
    out = np.zeros(N)
    np.add.at(out, i, np.abs(dU))
    np.add.at(out, j, np.abs(dU))
    return out if fmt != DENSE else out / 2


def pair_energy_forces(spec: PairSpec, R, nbrs_idx, fmt, box=None,
                       per_particle=False):
    """smap.pair_neighbor_list (jax_md/smap.py:922-979) + grad (quantity.py:58-60).

    Returns (E, F[N,d], W[d,d]) with W = dU/d(strain) = sum_pairs U'(r)/r dR (x) dR
    (the quantity.stress oracle, quantity.py:238-282), all f64.  For per_particle
    the first output is the per-atom energy (reduce_axis=(1,))."""
    R = np.asarray(R, np.float64)
    N, dim = R.shape
    species = spec.species
    if fmt == DENSE:
        i = np.repeat(np.arange(N), nbrs_idx.shape[1])
        j = nbrs_idx.reshape(-1)
        norm = 2.0
    else:
        j, i = nbrs_idx[0], nbrs_idx[1]
        norm = 1.0 if fmt == ORDERED_SPARSE else 2.0
    m = j < N
    i, j = i[m], j[m]
    dR = displacement(R[j], R[i], box)                 # R_j - R_i (smap.py:937-938)
    r = np.sqrt((dR * dR).sum(-1))
    si = species[i] if species is not None else None
    sj = species[j] if species is not None else None
    U, dU, _ = pair_terms(spec, r, si, sj, i, j)
    with np.errstate(invalid='ignore', divide='ignore'):
        g = np.where(r > 0, dU / r, 0.0)              # U'(r)/r
    # E = sum U / norm ; dE/dR_j = U'/r * dR / norm ; dE/dR_i = -U'/r dR / norm
    gv = (g[:, None] * dR) / norm
    F = np.zeros((N, dim))
    np.add.at(F, j, -gv)
    np.add.at(F, i, gv)
    W = np.einsum('p,pa,pb->ab', g / norm, dR, dR)
    if per_particle:
        # Dense: reduce over the neighbour axis (smap.py:957-962); Sparse:
        # segment_sum over idx[0] (smap.py:977).
        Ei = np.zeros(N)
        np.add.at(Ei, i if fmt == DENSE else j, U / norm)
        return Ei, F, W
    return U.sum() / norm, F, W


def all_pairs_energy_forces(spec: PairSpec, R, box=None):
    """smap.pair (jax_md/smap.py:548-691) over all i != j; the oracle of the oracle."""
    R = np.asarray(R, np.float64)
    N = R.shape[0]
    idx = np.array([[j for j in range(N) if j != i] for i in range(N)], np.int64)
    return pair_energy_forces(spec, R, idx, DENSE, box)


def pair_force_vjp(spec: PairSpec, R, nbrs_idx, fmt, lam, box=None):
    """VJP of F(R, sigma, eps) against cotangent lam[N,d].

    Returns (gR[N,d], g_sigma[S,S] or scalar, g_eps[S,S] or scalar) with
    gR = (dF/dR)^T lam = -H lam.  For each pair, with u = dR/r (dR=R_j-R_i):
    dF_i/dR_j = U''uu^T + U'/r (I - uu^T) (and symmetric blocks)."""
    R = np.asarray(R, np.float64)
    N, dim = R.shape
    if fmt == DENSE:
        i = np.repeat(np.arange(N), nbrs_idx.shape[1])
        j = nbrs_idx.reshape(-1)
        norm = 2.0
    else:
        j, i = nbrs_idx[0], nbrs_idx[1]
        norm = 1.0 if fmt == ORDERED_SPARSE else 2.0
    m = j < N
    i, j = i[m], j[m]
    dR = displacement(R[j], R[i], box)
    r = np.sqrt((dR * dR).sum(-1))
    u = dR / r[:, None]
    si = spec.species[i] if spec.species is not None else None
    sj = spec.species[j] if spec.species is not None else None
    U, dU, d2U = pair_terms(spec, r, si, sj, i, j)
    dl = lam[j] - lam[i]                                   # (lam_j - lam_i)
    ul = (u * dl).sum(-1)
    # F_i += U' u ; F_j -= U' u  (per entry /norm). d(U' u)/dR_j = H_p, /dR_i = -H_p
    # lam . F contribution per entry = (lam_i - lam_j) . U' u / norm
    # gradient wrt R_j: -(H_p^T (lam_j - lam_i))/norm ... assemble directly:
    Hdl = (d2U * ul)[:, None] * u + (dU / r)[:, None] * (dl - ul[:, None] * u)
    gR = np.zeros((N, dim))
    np.add.at(gR, j, -Hdl / norm)
    np.add.at(gR, i, Hdl / norm)
    # parameter gradients of L = lam . F  = sum_entries (lam_i - lam_j).u * U'/norm
    # dL/dtheta = sum (lam_i - lam_j).u * dU'/dtheta / norm  (finite-diff in theta)
    return gR, (-ul / norm), (i, j, r, si, sj)


# ---------------------------------------------------------------------------
# simulate.py
def velocity_verlet(force_fn, R, P, F, mass, dt, box):
    """jax_md/simulate.py:227-243 with periodic_shift (space.py:250-252), or
    the shift of a PeriodicGeneral ``box`` (space.py:436-466)."""
    P = P + 0.5 * dt * F
    if hasattr(box, 'shift'):
        R = box.shift(R, dt * P / mass)
        F = force_fn(R)
        return R, P + 0.5 * dt * F, F
    R = R + dt * P / mass
    if box is not None:
        R = np.mod(R, box)
    F = force_fn(R)
    P = P + 0.5 * dt * F
    return R, P, F


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11) on uint32 arrays:
    ten rounds of two 32x32 -> 64-bit products, word swaps and XORs with
    the key, the key bumped by the Weyl constants after each round."""
    m0, m1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    w0, w1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
    mask = np.uint64(0xFFFFFFFF)
    c = [np.asarray(x, np.uint64) & mask for x in (c0, c1, c2, c3)]
    k0 = np.asarray(k0, np.uint64) & mask
    k1 = np.asarray(k1, np.uint64) & mask
    for _ in range(10):
        p0, p1 = m0 * c[0], m1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + w0) & mask
        k1 = (k1 + w1) & mask
    return [x.astype(np.uint32) for x in c]


def word_to_unit(w):
    """A 32-bit word as the uniform the device forms: the top 23 bits k give
    (2k + 1) / 2^24, exact in float32 (so f64 here is the same number)."""
    w = np.asarray(w, np.uint64)
    return (2.0 * (w >> np.uint64(9)).astype(np.float64) + 1.0) / 16777216.0


def normals_from_words(w):
    """Box-Muller on word pairs (0, 1) and (2, 3) of w [n, 4]:
    sqrt(-2 ln u0) (cos, sin)(2 pi u1), in f64."""
    w = np.asarray(w, np.uint64).reshape(-1, 4)
    u = [word_to_unit(w[:, k]) for k in range(4)]
    z = np.empty((len(w), 4))
    for h in range(2):
        rad = np.sqrt(-2.0 * np.log(u[2 * h]))
        z[:, 2 * h] = rad * np.cos(2 * np.pi * u[2 * h + 1])
        z[:, 2 * h + 1] = rad * np.sin(2 * np.pi * u[2 * h + 1])
    return z


def langevin_normals(seed, step, n):
    """The device's Langevin draws restated: atom i at `step` under `seed`
    takes Philox4x32-10 on counter (i, 0, step lo, step hi) and key
    (seed lo, seed hi); each word pair (u0, u1) -> sqrt(-2 ln u0)
    (cos, sin)(2 pi u1) with u = (2 (w >> 9) + 1) / 2^24.  Returns the
    words [n, 4] (uint32) and the normals [n, 4] (f64)."""
    i = np.arange(n, dtype=np.uint64)
    lo, hi = np.uint64(step & 0xFFFFFFFF), np.uint64(step >> 32)
    w = philox4x32_10(i, np.zeros_like(i), np.full_like(i, lo), np.full_like(i, hi),
                      np.uint64(seed & 0xFFFFFFFF), np.uint64(seed >> 32))
    w = np.stack(w, 1)
    return w, normals_from_words(w)


def nvt_langevin_step(force_fn, R, P, F, mass, dt, kT, gamma, box, xi):
    """jax_md/simulate.py:1161-1171 (BAOAB, Davidchack, Ouldridge and
    Tretyakov 2015): half kick, half drift, the O step
    p <- c1 p + sqrt(kT (1 - c1^2) m) xi with c1 = exp(-gamma dt)
    (stochastic_step, simulate.py:1102-1110), half drift, force, half kick.
    xi is the standard-normal draw of the O step, passed in so that a device
    run can be replayed exactly from the noise it drew."""
    m = np.asarray(mass, np.float64)
    if m.ndim == 1:
        m = m[:, None]
    h = 0.5 * dt
    P = P + h * F
    R = R + h * P / m
    if box is not None:
        R = np.mod(R, box)
    c1 = math.exp(-gamma * dt)
    c2 = math.sqrt(kT * (1.0 - c1 * c1))
    P = c1 * P + c2 * np.sqrt(m) * xi
    R = R + h * P / m
    if box is not None:
        R = np.mod(R, box)
    F = force_fn(R)
    P = P + h * F
    return R, P, F


SUZUKI_YOSHIDA_WEIGHTS = {
    # Suzuki-Yoshida decomposition weights (Suzuki 1991 / Yoshida 1990), the
    # values jax_md/simulate.py:328-347 uses.
    1: [1.0],
    3: [0.828981543588751, -0.657963087177502, 0.828981543588751],
    5: [0.2967324292201065, 0.2967324292201065, -0.186929716880426,
        0.2967324292201065, 0.2967324292201065],
    7: [0.784513610477560, 0.235573213359357, -1.17767998417887,
        1.31518632068391, -1.17767998417887, 0.235573213359357, 0.784513610477560],
}


@dataclass
class ChainO:
    xi: np.ndarray
    p_xi: np.ndarray
    Q: np.ndarray
    tau: float
    KE: float
    dof: int


def nhc_init(dof, KE, kT, tau, chain_length):
    """simulate.py:436-442."""
    Q = kT * tau ** 2 * np.ones(chain_length)
    Q[0] *= dof
    return ChainO(np.zeros(chain_length), np.zeros(chain_length), Q, tau, KE, dof)


def nhc_substep(delta, P, c: ChainO, kT):
    """simulate.py:444-490 (one Suzuki-Yoshida substep of the chain)."""
    xi, p, Q, KE, DOF = c.xi.copy(), c.p_xi.copy(), c.Q, c.KE, c.dof
    M = len(p) - 1
    d2, d4, d8 = delta / 2, delta / 4, delta / 8
    G = p[M - 1] ** 2 / Q[M - 1] - kT
    p[M] += d4 * G
    pnew = p[M]
    for m in range(M - 1, 0, -1):
        G = p[m - 1] ** 2 / Q[m - 1] - kT
        scale = math.exp(-d8 * pnew / Q[m + 1])
        pnew = scale * (scale * p[m] + d4 * G)
        p[m] = pnew
    G = 2 * KE - DOF * kT
    scale = math.exp(-d8 * p[1] / Q[1])
    p[0] = scale * (scale * p[0] + d4 * G)
    scale = math.exp(-d2 * p[0] / Q[0])
    KE = KE * scale ** 2
    P = P * scale
    xi = xi + d2 * p / Q
    G = 2 * KE - DOF * kT
    for m in range(M):
        scale = math.exp(-d8 * p[m + 1] / Q[m + 1])
        p[m] = scale * (scale * p[m] + d4 * G)
        G = p[m] ** 2 / Q[m] - kT
    p[M] += d4 * G
    return P, ChainO(xi, p, Q, c.tau, KE, DOF)


def nhc_half_step(P, c, kT, dt, chain_steps, sy_steps):
    """simulate.py:492-507."""
    if chain_steps == 1 and sy_steps == 1:
        return nhc_substep(dt, P, c, kT)
    delta = dt / chain_steps
    ws = SUZUKI_YOSHIDA_WEIGHTS[sy_steps]
    for k in range(chain_steps * sy_steps):
        P, c = nhc_substep(delta * ws[k % sy_steps], P, c, kT)
    return P, c


def kinetic_energy(P, mass=1.0):
    """quantity.py:124-159."""
    return 0.5 * float(np.sum(P ** 2 / mass))


def nvt_nose_hoover_step(force_fn, R, P, F, mass, c, dt, kT, box,
                         chain_steps=2, sy_steps=3):
    """simulate.py:649-667 (apply_fn)."""
    Q = kT * c.tau ** 2 * np.ones(len(c.Q))
    Q[0] *= c.dof
    c = ChainO(c.xi, c.p_xi, Q, c.tau, c.KE, c.dof)
    P, c = nhc_half_step(P, c, kT, dt, chain_steps, sy_steps)
    R, P, F = velocity_verlet(force_fn, R, P, F, mass, dt, box)
    c = ChainO(c.xi, c.p_xi, c.Q, c.tau, kinetic_energy(P, mass), c.dof)
    P, c = nhc_half_step(P, c, kT, dt, chain_steps, sy_steps)
    return R, P, F, c


def sinhx_x(x):
    """simulate.py:763-772 (Taylor series of sinh(x) / x)."""
    return 1 + x ** 2 / 6 + x ** 4 / 120 + x ** 6 / 5040 + x ** 8 / 362_880 + x ** 10 / 39_916_800


def _chain_masses(c: ChainO, kT):
    """simulate.py:509-517 (update_mass): Q = kT tau^2, Q_0 x dof."""
    Q = kT * c.tau ** 2 * np.ones(len(c.Q))
    Q[0] *= c.dof
    return ChainO(c.xi, c.p_xi, Q, c.tau, c.KE, c.dof)


def npt_init(force_stress, R, P, box, mass, kT, dt, chain_length=3):
    """simulate.py:862-903 (init_fn of npt_nose_hoover) from given momenta:
    box_position = box_momentum = 0, box mass d (N + 1) kT tau_b^2, a
    one-degree barostat chain (tau_b = 1000 dt) and a thermostat chain on
    N d degrees of freedom (tau = 100 dt)."""
    R = np.asarray(R, np.float64)
    P = np.asarray(P, np.float64)
    n, dim = R.shape
    ref = np.asarray(box, np.float64)
    if ref.ndim == 0:
        ref = np.eye(dim) * float(ref)
    _, F, dUdV = force_stress(R, ref)
    tau_b, tau_t = 1000 * dt, 100 * dt
    return {'R': R, 'P': P, 'F': F, 'mass': mass, 'ref': ref, 'R_b': 0.0, 'P_b': 0.0,
            'M_b': dim * (n + 1) * kT * tau_b ** 2, 'dUdV': dUdV,
            'bc': nhc_init(1, 0.0, kT, tau_b, chain_length),
            'tc': nhc_init(n * dim, kinetic_energy(P, mass), kT, tau_t, chain_length)}


def npt_box(s):
    """simulate.py:786-792."""
    dim = s['R'].shape[1]
    V0 = float(np.linalg.det(s['ref']))
    V = V0 * np.exp(dim * s['R_b'])
    return (V / V0) ** (1 / dim) * s['ref'], V


def npt_nose_hoover_step(force_stress, s, pressure, kT, dt, chain_steps=2, sy_steps=3):
    """simulate.py:938-1001 (inner_step and apply_fn of npt_nose_hoover) in
    FP64; positions fractional in the cell, shifted by the
    PeriodicGeneral shift with the new cell."""
    s = dict(s)
    R, P, F, m = s['R'], s['P'], s['F'], s['mass']
    n, dim = R.shape
    dt_2 = dt / 2
    bc, tc = _chain_masses(s['bc'], kT), _chain_masses(s['tc'], kT)
    M_b = dim * (n + 1) * kT * bc.tau ** 2
    P_b, bc = nhc_half_step(s['P_b'], bc, kT, dt, chain_steps, sy_steps)
    P, tc = nhc_half_step(P, tc, kT, dt, chain_steps, sy_steps)
    V0 = float(np.linalg.det(s['ref']))
    alpha = 1 + 1 / n
    R_b, dUdV = s['R_b'], s['dUdV']

    def G(vol, P, dUdV):
        return alpha * float(np.sum(P ** 2 / m)) - dUdV - pressure * vol * dim

    def exp_iL2(P, F, v_b):
        x = alpha * v_b * dt_2
        return P * np.exp(-x) + dt_2 * F * sinhx_x(x / 2) * np.exp(-x / 2)
    vol = V0 * np.exp(dim * R_b)
    P_b = P_b + dt_2 * G(vol, P, dUdV)
    P = exp_iL2(P, F, P_b / M_b)
    R_b = R_b + P_b / M_b * dt
    vol = V0 * np.exp(dim * R_b)
    box = (vol / V0) ** (1 / dim) * s['ref']
    x = P_b / M_b * dt
    dR = R * (np.exp(x) - 1) + dt * (P / m) * np.exp(x / 2) * sinhx_x(x / 2)
    R = PeriodicGeneral(s['ref']).shift(R, dR, box=box)
    _, F, dUdV = force_stress(R, box)
    P = exp_iL2(P, F, P_b / M_b)
    P_b = P_b + dt_2 * G(vol, P, dUdV)
    tc = ChainO(tc.xi, tc.p_xi, tc.Q, tc.tau, kinetic_energy(P, m), tc.dof)
    bc = ChainO(bc.xi, bc.p_xi, bc.Q, bc.tau, P_b ** 2 / (2 * M_b), bc.dof)
    P, tc = nhc_half_step(P, tc, kT, dt, chain_steps, sy_steps)
    P_b, bc = nhc_half_step(P_b, bc, kT, dt, chain_steps, sy_steps)
    s.update(R=R, P=P, F=F, R_b=R_b, P_b=float(P_b), M_b=M_b, dUdV=dUdV, bc=bc, tc=tc)
    return s


def npt_invariant(PE, s, pressure, kT):
    """simulate.py:1007-1047."""
    _, V = npt_box(s)
    n, dim = s['R'].shape
    E = PE + kinetic_energy(s['P'], s['mass'])
    c = s['tc']
    E += c.p_xi[0] ** 2 / (2 * c.Q[0]) + n * dim * kT * c.xi[0]
    for x, p, q in zip(c.xi[1:], c.p_xi[1:], c.Q[1:]):
        E += p ** 2 / (2 * q) + kT * x
    c = s['bc']
    for x, p, q in zip(c.xi, c.p_xi, c.Q):
        E += p ** 2 / (2 * q) + kT * x
    return E + pressure * V + s['P_b'] ** 2 / (2 * s['M_b'])


def nvt_invariant(PE, P, mass, c: ChainO, kT):
    """simulate.py:672-701."""
    E = PE + kinetic_energy(P, mass)
    E += c.p_xi[0] ** 2 / (2 * c.Q[0]) + c.dof * kT * c.xi[0]
    for x, p, q in zip(c.xi[1:], c.p_xi[1:], c.Q[1:]):
        E += p ** 2 / (2 * q) + kT * x
    return E


# ---------------------------------------------------------------------------
# minimize.py
@dataclass
class FireO:
    R: np.ndarray
    P: np.ndarray
    F: np.ndarray
    mass: float
    dt: float
    alpha: float
    n_pos: int


def fire_step(force_fn, s: FireO, box, dt_max=0.4, n_min=5, f_inc=1.1, f_dec=0.5,
              alpha_start=0.1, f_alpha=0.99):
    """jax_md/minimize.py:181-224 (fire_descent apply_fn)."""
    R, P, F = velocity_verlet(force_fn, s.R, s.P, s.F, s.mass, s.dt, box)
    dt, alpha, n_pos = s.dt, s.alpha, s.n_pos
    F_norm = math.sqrt(float(np.sum(F ** 2)) + 1e-6)
    P_norm = math.sqrt(float(np.sum(P ** 2)))
    F_dot_P = float(np.sum(F * P))
    P = P + alpha * (F * P_norm / F_norm - P)
    n_pos = n_pos + 1 if F_dot_P >= 0 else 0
    if F_dot_P > 0 and n_pos > n_min:
        dt = min(dt * f_inc, dt_max)
        alpha = alpha * f_alpha
    if F_dot_P < 0:
        dt = dt * f_dec
        alpha = alpha_start
    if not F_dot_P >= 0:
        P = P * 0.0
    return FireO(R, P, F, s.mass, dt, alpha, n_pos)


# ---------------------------------------------------------------------------
# quantity.py
def stress(W, P, mass, volume):
    """quantity.py:238-282: (sum m v v^T - dU/deps) / V, with v = P/m."""
    V = P / mass
    VxV = np.einsum('n,na,nb->ab', np.broadcast_to(np.asarray(mass, np.float64).reshape(-1),
                                                  (len(P),)), V, V)
    return (VxV - W) / volume


def pressure(W, KE, dim, volume):
    """quantity.py:202-235: (2 KE - tr(dU/deps)) / (d V)."""
    return (2 * KE - np.trace(W)) / (dim * volume)


# ---------------------------------------------------------------------------
# Seeded generators for the benchmark workloads (shapes from the benchmark's configs)
def fcc_lattice(n_cells, density=0.8442, jitter=0.05, seed=0, dtype=np.float32):
    """FCC n^3 x 4 atoms at reduced density; jitter U(+-jitter)."""
    a = (4.0 / density) ** (1.0 / 3.0)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(n_cells)] * 3, indexing='ij'), -1).reshape(-1, 1, 3)
    R = ((g + basis[None]) * a).reshape(-1, 3)
    L = n_cells * a
    rng = np.random.default_rng(seed)
    R = R + rng.uniform(-jitter, jitter, R.shape)
    R = np.mod(R, L)
    return R.astype(dtype), np.float32(L)


def maxwell_boltzmann(N, dim, kT, seed=1, mass=1.0, dtype=np.float32):
    rng = np.random.default_rng(seed)
    P = np.sqrt(mass * kT) * rng.standard_normal((N, dim))
    P -= P.mean(0, keepdims=True)
    return P.astype(dtype)


def bidisperse_2d(N, phi=0.84, seed=0, dtype=np.float32):
    """50:50 bidisperse disks d in {1.0, 1.4} at packing fraction phi."""
    rng = np.random.default_rng(seed)
    species = np.zeros(N, np.int32)
    species[N // 2:] = 1
    rng.shuffle(species)
    d = np.where(species == 0, 1.0, 1.4)
    L = math.sqrt(np.sum(np.pi * d ** 2 / 4) / phi)
    R = rng.uniform(0, L, (N, 2))
    return R.astype(dtype), np.float32(L), species


def kob_andersen(N, density=1.2, seed=0, dtype=np.float32):
    rng = np.random.default_rng(seed)
    species = np.zeros(N, np.int32)
    species[int(0.8 * N):] = 1
    L = (N / density) ** (1.0 / 3.0)
    R = rng.uniform(0, L, (N, 3))
    sigma = np.array([[1.0, 0.8], [0.8, 0.88]])
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    return R.astype(dtype), np.float32(L), species, sigma, eps
