"""NVE and Nose-Hoover NVT integrators (jax_md/simulate.py) on the GB300 kernels.

``nve`` and ``nvt_nose_hoover`` keep the reference signatures and return
``(init_fn, apply_fn)``.  With a CUDA-backed energy (from
``jax_md_gb300.energy`` / ``smap``) and a shift from ``jax_md_gb300.space``,
``apply_fn(state, neighbor=nbrs)`` runs the velocity-Verlet step as three
kernels: a fused half-kick + drift (with the pending Nose-Hoover rescale), the
pair-force kernel, and the second half-kick.

State tensors are updated in place: the state returned by ``apply_fn`` shares
its buffers with the one passed in (``state.copy()`` gives an independent
snapshot).  Positions, momenta and forces are [N, d] views over float4 rows.
The Nose-Hoover chain lives in one f64 device buffer.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Callable, Optional

import numpy as np
import torch

from . import _native as N
from . import partition, quantity, smap
from . import space as _space

SUZUKI_YOSHIDA_WEIGHTS = {
    # Suzuki-Yoshida weights, the values of jax_md/simulate.py:328-347.
    1: [1.0],
    3: [0.828981543588751, -0.657963087177502, 0.828981543588751],
    5: [0.2967324292201065, 0.2967324292201065, -0.186929716880426, 0.2967324292201065,
        0.2967324292201065],
    7: [0.784513610477560, 0.235573213359357, -1.17767998417887, 1.31518632068391,
        -1.17767998417887, 0.235573213359357, 0.784513610477560],
}


class _StateMixin:
    def set(self, **kwargs):
        return dataclasses.replace(self, **kwargs)

    def copy(self):
        def c(v):
            if isinstance(v, torch.Tensor):
                # float4-row views stay float4 rows (the kernels' layout)
                if v.dim() == 2 and v.shape[1] < 4 and v.stride() == (4, 1):
                    return partition.padded_rows(v)
                return v.clone()
            return v.copy() if hasattr(v, 'copy') else v
        return dataclasses.replace(self, **{f.name: c(getattr(self, f.name))
                                            for f in dataclasses.fields(self)})


@dataclasses.dataclass
class NVEState(_StateMixin):
    """simulate.py:249-276."""
    position: torch.Tensor
    momentum: torch.Tensor
    force: torch.Tensor
    mass: object

    @property
    def velocity(self):
        return self.momentum / _mass_col(self.mass)


@dataclasses.dataclass
class NoseHooverChain(_StateMixin):
    """simulate.py:350-374, stored as one f64 buffer
    [xi(16) | p_xi(16) | Q(16) | spare(16) | KE | kT]."""
    buffer: torch.Tensor
    chain_length: int
    tau: float
    degrees_of_freedom: int

    @property
    def position(self):
        return self.buffer[0:self.chain_length]

    @property
    def momentum(self):
        return self.buffer[16:16 + self.chain_length]

    @property
    def mass(self):
        return self.buffer[32:32 + self.chain_length]

    @property
    def kinetic_energy(self):
        return self.buffer[64]

    def copy(self):
        return dataclasses.replace(self, buffer=self.buffer.clone())


@dataclasses.dataclass
class NVTNoseHooverState(_StateMixin):
    """simulate.py:538-562."""
    position: torch.Tensor
    momentum: torch.Tensor
    force: torch.Tensor
    mass: object
    chain: NoseHooverChain

    @property
    def velocity(self):
        return self.momentum / _mass_col(self.mass)


def _mass_col(mass):
    if isinstance(mass, torch.Tensor) and mass.numel() > 1:
        return mass.reshape(-1, 1)
    return mass


def canonicalize_mass(mass, n, device):
    """simulate.py:119-138: scalar stays a float, arrays become [N] float32."""
    if isinstance(mass, (int, float)):
        return float(mass)
    m = torch.as_tensor(mass, dtype=torch.float32, device=device)
    if m.numel() == 1:
        return float(m)
    if m.dim() == 2 and m.shape[1] == 1:
        m = m[:, 0]
    if m.dim() != 1 or m.shape[0] != n:
        raise ValueError('Expected mass to be either a floating point number or a one-dimensional '
                         f'ndarray. Found {tuple(m.shape)}.')
    return m.contiguous()


def _mass_ptr(mass):
    if isinstance(mass, torch.Tensor):
        return mass.data_ptr(), 1.0
    return None, float(mass)


def _rows4(t: torch.Tensor) -> torch.Tensor:
    """Float4-row copy of an [N, d] tensor, returned as an [N, d] view."""
    return partition.padded_rows(t.detach().to(torch.float32))


def _shift_space(shift_fn, dim) -> N.Space:
    s = N.Space()
    s.dim = dim
    periodic = isinstance(shift_fn, _space.Shift) and shift_fn.periodic and shift_fn.wrapped
    if isinstance(shift_fn, _space.GeneralShift):
        return shift_fn.space(dim)
    if not isinstance(shift_fn, _space.Shift):
        raise NotImplementedError('the GB300 integrators need a shift_fn from jax_md_gb300.space')
    s.periodic = 1 if periodic else 0
    if periodic:
        b = partition._box_list(shift_fn.box, dim)
        for d in range(dim):
            s.box[d] = b[d]
    return s


def canonicalize_momenta(state, momenta):
    """simulate.py:162-165: the state with the given momenta (as float4
    rows), or unchanged without them."""
    if momenta is None:
        return state
    return state.set(momentum=_rows4(momenta))


def initialize_momenta(R, mass, key, kT):
    """simulate.py:141-159 with torch's generator (the JAX PRNG is not reproducible here)."""
    g = key if isinstance(key, torch.Generator) else None
    if g is None:
        g = torch.Generator(device=R.device)
        g.manual_seed(int(key) if key is not None else 0)
    m = _mass_col(mass)
    m = m if isinstance(m, torch.Tensor) else torch.tensor(m, device=R.device)
    P = torch.sqrt(m * kT) * torch.randn(R.shape, generator=g, device=R.device, dtype=R.dtype)
    if R.shape[0] > 1:
        P = P - P.mean(0, keepdim=True)
    return P


class _Stepper:
    """Kernel plumbing shared by nve / nvt_nose_hoover."""

    def __init__(self, energy_or_force_fn, shift_fn, dt):
        self.energy_fn = energy_or_force_fn
        self.force_fn = quantity.canonicalize_force(energy_or_force_fn)
        self.kernel_force = quantity._kernel_energy(energy_or_force_fn)
        self.shift_fn = shift_fn
        self.dt = float(np.float32(dt))

    def forces_into(self, R, out, **kwargs):
        if self.kernel_force:
            e = self.energy_fn
            if isinstance(e, smap.PairAllEnergy):
                e.forces(R, out=out, **kwargs)
            else:
                nb = kwargs.pop('neighbor')
                e.forces(R, nb, out=out, **kwargs)
        else:
            out.copy_(self.force_fn(R, **kwargs))
        return out

    def kick_drift(self, state, dt, p_scale=None):
        R, P, F = state.position, state.momentum, state.force
        n, dim = R.shape
        s = _shift_space(self.shift_fn, dim)
        mptr, m0 = _mass_ptr(state.mass)
        N.check(N.lib().jmd_verlet_kick_drift(
            R.data_ptr(), R.stride(0), P.data_ptr(), P.stride(0), F.data_ptr(), F.stride(0), mptr, m0,
            n, ctypes.byref(s), dt, N.ptr(p_scale), None, 0, 0.0, None, N.stream_ptr()),
            'verlet_kick_drift')

    def kick(self, state, dt_half):
        P, F = state.momentum, state.force
        n, dim = P.shape
        N.check(N.lib().jmd_momentum_step(P.data_ptr(), P.stride(0), F.data_ptr(), F.stride(0), n,
                                          dim, dt_half, N.stream_ptr()), 'momentum_step')

    def velocity_verlet(self, state, dt=None, p_scale=None, **kwargs):
        """simulate.py:227-243."""
        dt = self.dt if dt is None else float(np.float32(dt))
        self.kick_drift(state, dt, p_scale)
        self.forces_into(state.position, state.force, **kwargs)
        self.kick(state, float(np.float32(dt / 2)))
        return state

    def new_state_tensors(self, R, **kwargs):
        N.require_cuda(R)
        R4 = _rows4(R)
        F4 = _rows4(torch.zeros_like(R4))
        self.forces_into(R4, F4, **kwargs)
        return R4, F4


class dispatch_by_state:
    """simulate.py:100-116: wraps a step function and dispatches on the type
    of ``state.position``; ``fn.register(T)(impl)`` installs ``impl`` for
    positions of type T (the reference's plug-in point for custom position
    types, e.g. rigid bodies)."""

    def __init__(self, fn):
        self._fn = fn
        self._registry = {}
        self.__doc__ = fn.__doc__
        self.__name__ = getattr(fn, '__name__', 'step')

    def __call__(self, state, *args, **kwargs):
        impl = self._registry.get(type(state.position))
        if impl is not None:
            return impl(state, *args, **kwargs)
        return self._fn(state, *args, **kwargs)

    def register(self, oftype):
        def register_fn(fn):
            self._registry[oftype] = fn
            return fn
        return register_fn


@dispatch_by_state
def momentum_step(state, dt):
    """simulate.py:168-173 (in place)."""
    P, F = state.momentum, state.force
    N.check(N.lib().jmd_momentum_step(P.data_ptr(), P.stride(0), F.data_ptr(), F.stride(0),
                                      P.shape[0], P.shape[1], float(dt), N.stream_ptr()),
            'momentum_step')
    return state


@dispatch_by_state
def kinetic_energy(state):
    """simulate.py:192-195: quantity.kinetic_energy of a state."""
    return quantity.kinetic_energy(momentum=state.momentum, mass=state.mass)


@dispatch_by_state
def temperature(state):
    """simulate.py:198-201: quantity.temperature of a state."""
    return quantity.temperature(momentum=state.momentum, mass=state.mass)


@dispatch_by_state
def position_step(state, shift_fn, dt, **kwargs):
    """simulate.py:176-188 (in place)."""
    R, P = state.position, state.momentum
    s = _shift_space(shift_fn, R.shape[1])
    mptr, m0 = _mass_ptr(state.mass)
    N.check(N.lib().jmd_position_step(R.data_ptr(), R.stride(0), P.data_ptr(), P.stride(0), mptr,
                                      m0, R.shape[0], ctypes.byref(s), float(dt), N.stream_ptr()),
            'position_step')
    return state


def velocity_verlet(force_fn, shift_fn, dt, state, **kwargs):
    """simulate.py:227-243 for any force function (in place)."""
    st = _Stepper(force_fn, shift_fn, dt)
    return st.velocity_verlet(state, **kwargs)


def nve(energy_or_force_fn, shift_fn, dt=1e-3, **sim_kwargs):
    """simulate.nve (simulate.py:279-317)."""
    st = _Stepper(energy_or_force_fn, shift_fn, dt)

    def init_fn(key, R, kT=None, mass=1.0, momenta=None, **kwargs):
        R4, F4 = st.new_state_tensors(R, **kwargs)
        m = canonicalize_mass(mass, R.shape[0], R.device)
        if momenta is None:
            P = initialize_momenta(R4, m, key, kT)
        else:
            P = momenta
        return NVEState(R4, _rows4(P), F4, m)

    def apply_fn(state, **kwargs):
        dt_ = kwargs.pop('dt', None)
        return st.velocity_verlet(state, dt_, **kwargs)

    init_fn.stepper = st
    apply_fn.stepper = st
    return init_fn, apply_fn


class _Chain:
    """Device-side Nose-Hoover chain (simulate.py:384-517)."""

    def __init__(self, dt, chain_length, chain_steps, sy_steps, tau):
        if chain_length < 2 or chain_length > 16:
            raise ValueError('chain_length must be between 2 and 16')
        if sy_steps not in SUZUKI_YOSHIDA_WEIGHTS:
            raise ValueError('sy_steps must be 1, 3, 5 or 7')
        self.dt = dt
        self.M1 = chain_length
        self.chain_steps = chain_steps
        self.sy_steps = sy_steps
        self.tau = tau

    def init(self, dof, KE, kT, device):
        buf = torch.zeros(66, dtype=torch.float64, device=device)
        buf[32:32 + self.M1] = kT * self.tau ** 2
        buf[32] = buf[32] * dof
        buf[64] = KE
        buf[65] = kT
        return NoseHooverChain(buf, self.M1, self.tau, dof)

    def half_step(self, chain: NoseHooverChain, p_scale, ke=None, update_mass=False):
        c = N.Nhc()
        c.chain_length = self.M1
        c.chain_steps = self.chain_steps
        c.sy_steps = self.sy_steps
        c.dof = chain.degrees_of_freedom
        c.dt = self.dt
        c.tau = chain.tau
        N.check(N.lib().jmd_nhc_half_step(ctypes.byref(c), chain.buffer.data_ptr(), N.ptr(ke),
                                          1 if update_mass else 0, p_scale.data_ptr(),
                                          N.stream_ptr()), 'nhc_half_step')


def nvt_nose_hoover(energy_or_force_fn, shift_fn, dt, kT, chain_length: int = 5,
                    chain_steps: int = 2, sy_steps: int = 3, tau: Optional[float] = None,
                    **sim_kwargs):
    """simulate.nvt_nose_hoover (simulate.py:565-669)."""
    st = _Stepper(energy_or_force_fn, shift_fn, dt)
    dt32 = float(np.float32(dt))
    if tau is None:
        tau = dt32 * 100
    tau = float(np.float32(tau))
    chain_fns = _Chain(dt32, chain_length, chain_steps, sy_steps, tau)

    def init_fn(key, R, mass=1.0, momenta=None, **kwargs):
        _kT = kwargs.pop('kT', kT)
        R4, F4 = st.new_state_tensors(R, **kwargs)
        m = canonicalize_mass(mass, R.shape[0], R.device)
        P = initialize_momenta(R4, m, key, _kT) if momenta is None else momenta
        P4 = _rows4(P)
        dof = quantity.count_dof(R)
        KE = float(quantity._ke_f64(P4, m))
        chain = chain_fns.init(dof, KE, float(_kT), R.device)
        return NVTNoseHooverState(R4, P4, F4, m, chain)

    def apply_fn(state, **kwargs):
        chain = state.chain
        if 'kT' in kwargs:
            chain.buffer[65] = float(kwargs.pop('kT'))
        scale = torch.empty((), dtype=torch.float64, device=state.position.device)
        # update_mass + first half step (simulate.py:653-656); the rescale is
        # applied inside the fused kick-drift kernel.
        chain_fns.half_step(chain, scale, update_mass=True)
        st.velocity_verlet(state, p_scale=scale, **kwargs)
        ke = quantity._ke_f64(state.momentum, state.mass, out=chain.buffer[64])
        chain_fns.half_step(chain, scale, ke=None)
        P = state.momentum
        N.check(N.lib().jmd_scale_momentum(P.data_ptr(), P.stride(0), P.shape[0], P.shape[1],
                                           scale.data_ptr(), N.stream_ptr()), 'scale_momentum')
        return state

    init_fn.stepper = st
    apply_fn.stepper = st
    apply_fn.chain_fns = chain_fns
    return init_fn, apply_fn


def _nvt_struct(chain_fns: '_Chain', state: 'NVTNoseHooverState') -> N.Nvt:
    """jmd_nvt of a state: chain constants, its device buffer, a persistent
    scale scratch and a reduction workspace (kept on the state so a replayed
    graph sees the same pointers)."""
    chain = state.chain
    dev = state.position.device
    scratch = getattr(state, '_nvt_scratch', None)
    n = state.position.shape[0]
    if scratch is None:
        ws = torch.empty(N.lib().jmd_reduce_workspace_bytes(n), dtype=torch.uint8, device=dev)
        scratch = (torch.ones((), dtype=torch.float64, device=dev), ws)
        object.__setattr__(state, '_nvt_scratch', scratch)
    v = N.Nvt()
    v.chain.chain_length = chain_fns.M1
    v.chain.chain_steps = chain_fns.chain_steps
    v.chain.sy_steps = chain_fns.sy_steps
    v.chain.dof = chain.degrees_of_freedom
    v.chain.dt = chain_fns.dt
    v.chain.tau = chain.tau
    v.chain_state = chain.buffer.data_ptr()
    v.p_scale = scratch[0].data_ptr()
    v.reduce_workspace = scratch[1].data_ptr()
    v.reduce_workspace_bytes = scratch[1].numel()
    return v


@dataclasses.dataclass
class NVTLangevinState(_StateMixin):
    """simulate.py:1075-1099.  The reference's PRNG key becomes the
    counter-based generator's (seed, step): step k of a run draws from
    (seed, k, atom), so a run is reproducible from its seed."""
    position: torch.Tensor
    momentum: torch.Tensor
    force: torch.Tensor
    mass: object
    seed: int
    step: int

    @property
    def velocity(self):
        return self.momentum / _mass_col(self.mass)


@dispatch_by_state
def stochastic_step(state, dt, kT, gamma):
    """simulate.py:1102-1110, the O step (in place): p <- c1 p +
    sqrt(kT (1 - c1^2) m) xi with c1 = exp(-gamma dt), xi drawn on the device
    from (state.seed, state.step, atom); advances state.step."""
    c1 = math.exp(-gamma * dt)
    c2 = math.sqrt(kT * (1.0 - c1 * c1))
    P = state.momentum
    mptr, m0 = _mass_ptr(state.mass)
    N.check(N.lib().jmd_langevin_o_step(P.data_ptr(), P.stride(0), P.shape[0], P.shape[1], mptr,
                                        m0, float(np.float32(c1)), float(np.float32(c2)),
                                        state.seed, state.step, None, N.stream_ptr()),
            'langevin_o_step')
    state.step += 1
    return state


def _mix64(x: int) -> int:
    """SplitMix64's finaliser (Steele, Lea and Flood 2014): a bijective 64-bit
    hash, used to derive independent seeds from one key."""
    x &= 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return x ^ (x >> 31)


def split_key(key, stream: int) -> int:
    """The seed of `stream` under `key`: the role random.split plays in the
    reference (simulate.py:1157), so the initial momenta and the O-step noise
    of one key are independent.  `key` is an int, a torch.Generator (its
    initial seed) or None (0)."""
    if isinstance(key, torch.Generator):
        base = key.initial_seed()
    else:
        base = 0 if key is None else int(key)
    return _mix64(_mix64(base) ^ (0x9E3779B97F4A7C15 * (stream + 1)))


def nvt_langevin(energy_or_force_fn, shift_fn, dt, kT, gamma=0.1, center_velocity=True,
                 **sim_kwargs):
    """simulate.nvt_langevin (simulate.py:1113-1171): BAOAB (Davidchack,
    Ouldridge and Tretyakov 2015) -- half kick, half drift, the O step
    p <- c1 p + sqrt(kT (1 - c1^2) m) xi with c1 = exp(-gamma dt), half drift,
    force, half kick.  The O step is one kernel drawing xi from a counter-based
    generator (jmd_langevin_o_step); `key` seeds it and the initial momenta
    through two independent streams (split_key).
    The reference's draws come from jax.random, so trajectories agree with it
    in distribution, not draw for draw."""
    st = _Stepper(energy_or_force_fn, shift_fn, dt)

    def init_fn(key, R, mass=1.0, momenta=None, **kwargs):
        _kT = kwargs.pop('kT', kT)
        R4, F4 = st.new_state_tensors(R, **kwargs)
        m = canonicalize_mass(mass, R.shape[0], R.device)
        # two streams of one key, as the reference splits its key: the O-step
        # noise (stream 0) and the initial momenta (stream 1, or the caller's
        # Generator itself)
        seed = split_key(key, 0)
        if momenta is None:
            mkey = key if isinstance(key, torch.Generator) else split_key(key, 1)
            P = initialize_momenta(R4, m, mkey, _kT)
        else:
            P = momenta
        return NVTLangevinState(R4, _rows4(P), F4, m, seed, 0)

    def apply_fn(state, **kwargs):
        _dt = float(np.float32(kwargs.pop('dt', st.dt)))
        _kT = float(kwargs.pop('kT', kT))
        h = float(np.float32(_dt / 2))
        momentum_step(state, h)
        position_step(state, shift_fn, h)
        stochastic_step(state, _dt, _kT, gamma)
        position_step(state, shift_fn, h)
        st.forces_into(state.position, state.force, **kwargs)
        momentum_step(state, h)
        return state

    init_fn.stepper = st
    apply_fn.stepper = st
    return init_fn, apply_fn


def nvt_nose_hoover_invariant(energy_fn, state: NVTNoseHooverState, kT, **kwargs):
    """simulate.py:672-701 (f64)."""
    if quantity._kernel_energy(energy_fn):
        if isinstance(energy_fn, smap.PairAllEnergy):
            PE = energy_fn.compute(state.position, force=False)[0]
        else:
            PE = energy_fn.energy_f64(state.position, kwargs.pop('neighbor'), **kwargs)
    else:
        PE = energy_fn(state.position, **kwargs).double()
    KE = quantity._ke_f64(state.momentum, state.mass)
    c = state.chain
    dof = quantity.count_dof(state.position)
    E = PE + KE
    E = E + c.momentum[0] ** 2 / (2 * c.mass[0]) + dof * kT * c.position[0]
    for r, p, m in zip(c.position[1:], c.momentum[1:], c.mass[1:]):
        E = E + p ** 2 / (2 * m) + kT * r
    return E


# ---------------------------------------------------------------------------
# NPT: simulate.py:704-1047
@dataclasses.dataclass
class NPTNoseHooverState(_StateMixin):
    """simulate.py:704-760.  Particle arrays live on the device; the box
    degrees of freedom (box_position = (1/d) log(V / V_0), its momentum and
    mass, and dU/dV of the last force evaluation) are host f64 scalars, since
    every kernel launch takes the current cell by value.  The two chains are
    device chains (the thermostat's with N d degrees of freedom, the
    barostat's with one)."""
    position: torch.Tensor
    momentum: torch.Tensor
    force: torch.Tensor
    mass: object
    reference_box: np.ndarray
    box_position: float
    box_momentum: float
    box_mass: float
    dUdV: float
    barostat: NoseHooverChain
    thermostat: NoseHooverChain

    @property
    def velocity(self):
        return self.momentum / _mass_col(self.mass)

    @property
    def box(self):
        return npt_box(self)


def sinhx_x(x: float) -> float:
    """simulate.py:763-772: the Taylor series of sinh(x) / x."""
    return 1 + x ** 2 / 6 + x ** 4 / 120 + x ** 6 / 5040 + x ** 8 / 362_880 + x ** 10 / 39_916_800


def _npt_box_info(state: NPTNoseHooverState):
    """simulate.py:775-783: (V, V -> box)."""
    dim = state.position.shape[1]
    ref = state.reference_box
    V_0 = quantity.volume(dim, ref)
    V = V_0 * math.exp(dim * state.box_position)
    return V, (lambda v: (v / V_0) ** (1 / dim) * ref)


def npt_box(state: NPTNoseHooverState) -> np.ndarray:
    """simulate.py:786-792: the current cell."""
    V, box_fn = _npt_box_info(state)
    return box_fn(V)


def _force_stress(energy_fn, R, box, F_out, **kwargs):
    """(E, dU/dV) at R in the cell ``box``, with -dE/dR written into F_out:
    the kernel's energy, forces and virial; dU/dV of the reference's
    perturbation (1 + eps) (simulate.py:852-860) is the virial's trace."""
    if isinstance(energy_fn, smap.PairAllEnergy):
        e, F, _, W = energy_fn.compute(R, force=True, virial=True, box=box, **kwargs)
    elif isinstance(energy_fn, smap.PairNeighborListEnergy):
        nbrs = kwargs.pop('neighbor')
        e, F, _, W = energy_fn.compute(R, nbrs, force=True, virial=True, box=box, **kwargs)
    else:
        raise NotImplementedError('npt_nose_hoover needs an energy from jax_md_gb300.energy')
    F_out.copy_(F)
    dim = R.shape[1]
    return e, float(W[:dim].sum())


def npt_nose_hoover(energy_fn, shift_fn, dt, pressure, kT, barostat_kwargs=None,
                    thermostat_kwargs=None):
    """simulate.npt_nose_hoover (simulate.py:795-1004): NPT with one
    Nose-Hoover chain on the particles and one on the box (isotropic volume
    moves of a periodic_general cell, fractional coordinates).  The forces,
    virial and the exp(iL) maps of every step are kernels; the box scalars
    are updated on the host between them."""
    if not isinstance(shift_fn, _space.GeneralShift):
        raise NotImplementedError('npt_nose_hoover needs the shift of space.periodic_general')
    dt32 = float(np.float32(dt))
    dt_2 = float(np.float32(dt / 2))

    def nhc_kwargs(tau, overrides):
        kw = {'chain_length': 3, 'chain_steps': 2, 'sy_steps': 3, 'tau': tau}  # simulate.py:520-537
        kw.update(overrides or {})
        return kw
    bk = nhc_kwargs(1000 * dt, barostat_kwargs)
    tk = nhc_kwargs(100 * dt, thermostat_kwargs)
    bchain = _Chain(dt32, bk['chain_length'], bk['chain_steps'], bk['sy_steps'],
                    float(np.float32(bk['tau'])))
    tchain = _Chain(dt32, tk['chain_length'], tk['chain_steps'], tk['sy_steps'],
                    float(np.float32(tk['tau'])))
    L = N.lib()

    def box_mass(n, dim, kT_):
        return dim * (n + 1) * kT_ * bchain.tau ** 2

    def init_fn(key, R, box, mass=1.0, momenta=None, **kwargs):
        _kT = float(kwargs.pop('kT', kT))
        n, dim = R.shape
        R4 = _rows4(R.detach().to(torch.float32))
        F4 = _rows4(torch.zeros_like(R4))
        ref = _space.cell_matrix(box, dim)
        _, dUdV = _force_stress(energy_fn, R4, ref, F4, **kwargs)
        m = canonicalize_mass(mass, n, R.device)
        P = initialize_momenta(R4, m, key, _kT) if momenta is None else momenta
        P4 = _rows4(P)
        KE = float(quantity._ke_f64(P4, m))
        barostat = bchain.init(1, 0.0, _kT, R.device)
        thermostat = tchain.init(quantity.count_dof(R), KE, _kT, R.device)
        return NPTNoseHooverState(R4, P4, F4, m, ref, 0.0, 0.0, box_mass(n, dim, _kT), dUdV,
                                  barostat, thermostat)

    def apply_fn(state: NPTNoseHooverState, **kwargs):
        _kT = float(kwargs.pop('kT', kT))
        _pressure = float(kwargs.pop('pressure', pressure))
        R, P, F, m = state.position, state.momentum, state.force, state.mass
        n, dim = R.shape
        dev = R.device
        mptr, m0 = _mass_ptr(m)
        scale = torch.empty((), dtype=torch.float64, device=dev)
        # update_mass (both chains and the box), then the first half steps
        # (simulate.py:975-985)
        state.barostat.buffer[65] = _kT
        state.thermostat.buffer[65] = _kT
        M_b = box_mass(n, dim, _kT)
        bchain.half_step(state.barostat, scale, update_mass=True)
        P_b = state.box_momentum * float(scale)
        tchain.half_step(state.thermostat, scale, update_mass=True)
        N.check(L.jmd_scale_momentum(P.data_ptr(), P.stride(0), n, dim, scale.data_ptr(),
                                     N.stream_ptr()), 'scale_momentum')
        # inner step (simulate.py:938-973)
        ref = state.reference_box
        V_0 = quantity.volume(dim, ref)
        alpha = 1 + 1 / n
        R_b, dUdV = state.box_position, state.dUdV

        def G_e(vol):  # box_force, simulate.py:915-923
            KE2 = 2 * float(quantity._ke_f64(P, m))
            return alpha * KE2 - dUdV - _pressure * vol * dim

        def exp_iL2(v_b):
            x = alpha * v_b * dt_2
            c0 = math.exp(-x)
            c1 = dt_2 * sinhx_x(x / 2) * math.exp(-x / 2)
            N.check(L.jmd_npt_map(1, None, P.data_ptr(), F.data_ptr(), mptr, m0, n,
                                  ctypes.byref(sp), c0, c1, N.stream_ptr()), 'npt_map')
        vol = V_0 * math.exp(dim * R_b)
        P_b = P_b + dt_2 * G_e(vol)
        sp = shift_fn.space(dim, box=ref)   # exp_iL2 ignores the geometry
        exp_iL2(P_b / M_b)
        R_b = R_b + P_b / M_b * dt32
        vol = V_0 * math.exp(dim * R_b)
        box = (vol / V_0) ** (1 / dim) * ref
        x = P_b / M_b * dt32
        sp = shift_fn.space(dim, box=box)
        N.check(L.jmd_npt_map(0, R.data_ptr(), P.data_ptr(), None, mptr, m0, n,
                              ctypes.byref(sp), math.exp(x) - 1,
                              dt32 * math.exp(x / 2) * sinhx_x(x / 2), N.stream_ptr()), 'npt_map')
        _, dUdV = _force_stress(energy_fn, R, box, F, **kwargs)
        exp_iL2(P_b / M_b)
        P_b = P_b + dt_2 * G_e(vol)
        # second half steps (simulate.py:987-1001)
        quantity._ke_f64(P, m, out=state.thermostat.buffer[64])
        state.barostat.buffer[64] = P_b ** 2 / (2 * M_b)
        tchain.half_step(state.thermostat, scale)
        N.check(L.jmd_scale_momentum(P.data_ptr(), P.stride(0), n, dim, scale.data_ptr(),
                                     N.stream_ptr()), 'scale_momentum')
        bchain.half_step(state.barostat, scale)
        P_b = P_b * float(scale)
        state.box_position, state.box_momentum, state.box_mass, state.dUdV = R_b, P_b, M_b, dUdV
        return state

    apply_fn.chains = (bchain, tchain)
    return init_fn, apply_fn


def npt_nose_hoover_invariant(energy_fn, state: NPTNoseHooverState, pressure, kT, **kwargs):
    """simulate.py:1007-1047 (f64): potential and kinetic energy, both
    chains, P V and the box's kinetic energy."""
    V, box_fn = _npt_box_info(state)
    box = box_fn(V)
    if isinstance(energy_fn, smap.PairAllEnergy):
        PE = float(energy_fn.compute(state.position, force=False, box=box, **kwargs)[0])
    elif isinstance(energy_fn, smap.PairNeighborListEnergy):
        nbrs = kwargs.pop('neighbor')
        PE = float(energy_fn.compute(state.position, nbrs, force=False, box=box, **kwargs)[0])
    else:
        PE = float(energy_fn(state.position, box=box, **kwargs))
    E = PE + float(quantity._ke_f64(state.momentum, state.mass))
    dof = quantity.count_dof(state.position)
    c = state.thermostat
    xi, p, Q = (c.position.cpu().numpy(), c.momentum.cpu().numpy(), c.mass.cpu().numpy())
    E += p[0] ** 2 / (2 * Q[0]) + dof * kT * xi[0]
    for r, pp, mm in zip(xi[1:], p[1:], Q[1:]):
        E += pp ** 2 / (2 * mm) + kT * r
    c = state.barostat
    xi, p, Q = (c.position.cpu().numpy(), c.momentum.cpu().numpy(), c.mass.cpu().numpy())
    for r, pp, mm in zip(xi, p, Q):
        E += pp ** 2 / (2 * mm) + kT * r
    E += pressure * V + state.box_momentum ** 2 / (2 * state.box_mass)
    return E


# ---------------------------------------------------------------------------
# Device-resident runner
def _nve_system(st: '_Stepper', state: NVEState, nbrs, alt: torch.Tensor) -> N.NveSystem:
    e = st.energy_fn
    if not isinstance(e, smap.PairNeighborListEnergy):
        raise NotImplementedError('run() needs a neighbour-list energy from jax_md_gb300.energy')
    if nbrs.format is not partition.Dense or nbrs.plan is None:
        raise NotImplementedError('run() needs a Dense NeighborList from jax_md_gb300.partition')
    R, P, F = state.position, state.momentum, state.force
    for t, name in ((R, 'position'), (P, 'momentum'), (F, 'force')):
        if t.stride(0) != 4 or t.data_ptr() % 16:
            raise ValueError(f'state.{name} must be float4 rows (use init_fn of this module)')
    n, dim = R.shape
    plan = nbrs.plan
    species, pair = e._resolve(R, {})
    s = N.NveSystem()
    s.n = n
    s.space = _shift_space(st.shift_fn, dim)
    s.position = R.data_ptr()
    s.position_alt = alt.data_ptr()
    s.momentum = P.data_ptr()
    s.force = F.data_ptr()
    mptr, m0 = _mass_ptr(state.mass)
    s.mass = mptr
    s.mass_scalar = m0
    s.species = N.ptr(species)
    s.pair = pair
    s.nlist = plan.nl
    s.idx = nbrs.idx_buffer().data_ptr()
    s.idx_ld = plan.ld
    s.nbr_count = plan.count.data_ptr()
    s.reference_position = nbrs.reference_position.data_ptr()
    s.error_code = nbrs.error.code.data_ptr()
    s.occupancy = plan.occupancy.data_ptr()
    s.rebuild_flag = plan.flag.data_ptr()
    s.nl_workspace = plan.workspace.data_ptr()
    s.nl_workspace_bytes = plan.workspace.numel()
    s.dt = st.dt
    s.threshold_sq = -1.0 if plan.always_rebuild else plan.threshold_sq
    return s, species


# Cells per segment of the segment-local engine list (jmd_segment_plan): the
# default, and the (cells, threads) choices the autotuner
# (tune.autotune_segment) records per cell grid.
SEGMENT_CELLS_DEFAULT = 5
_segment_choice = {}


def _grid_key(nl: N.NList):
    d = nl.space.dim
    return (d, tuple(nl.cells_per_side[:d]), nl.cell_capacity)


def segment_threads_default(cells: int, cell_capacity: int) -> int:
    """Threads per segment CTA: about the own atoms of a segment (cells x
    0.8 x cell capacity, the capacity being 1.25 x the fullest cell at
    allocation), in whole warps, 64 to 256."""
    t = int(math.ceil(cells * cell_capacity * 0.8 / 32.0)) * 32
    return max(64, min(256, t))


def segment_plan(nl: N.NList, cells: int):
    """(n_segments, capacity_atoms, smem_bytes, cells_used, list_bytes) of the
    segment layout for a cell grid, or None when it does not apply."""
    ns, cap, cu = N.I32(), N.I32(), N.I32()
    sm, lb = N.I64(), N.I64()
    rc = N.lib().jmd_segment_plan(ctypes.byref(nl), int(cells), ctypes.byref(ns), ctypes.byref(cap),
                                  ctypes.byref(sm), ctypes.byref(cu), ctypes.byref(lb))
    if rc != 0:
        return None
    return ns.value, cap.value, sm.value, cu.value, lb.value


def segment_list_smem(nl: N.NList, cells: int, n_atoms: int) -> int:
    """Shared-memory bytes for staging a segment's list block with its
    positions: a block of 1.2 x the mean own atoms of a segment (rounded to
    8) at the list's full chunk depth; segments with larger blocks read
    theirs from global memory."""
    d = nl.space.dim
    ncell = 1
    for k in range(d):
        ncell *= int(nl.cells_per_side[k])
    own = 1.2 * cells * n_atoms / max(1, ncell)
    P = (int(math.ceil(own)) + 7) // 8 * 8
    nch = max(1, (int(nl.max_occupancy) + 7) // 8)
    return 16 + 2 * P + nch * P * 16


class _SortedBuffers:
    """Engine-private, cell-ordered copy of a system (see jmd_nve_run_sorted).
    With `seg_cells` the private list is the segment-local one (16-bit staged
    slots, 8-entry chunks); otherwise the tiled int32 list."""

    def __init__(self, n, ld, species: bool, workspace_bytes: int, device, seg_cells=None,
                 seg_threads=128, seg_list_bytes=0, seg_list_smem=0, seg_half=0):
        f4 = lambda: torch.empty((n, 4), dtype=torch.float32, device=device)
        i4 = lambda: torch.empty(n, dtype=torch.int32, device=device)
        self.n, self.ld = n, ld
        self.xa, self.xb, self.p, self.f, self.ref, self.t4a, self.t4b = (f4() for _ in range(7))
        self.perm, self.tia, self.tib = i4(), i4(), i4()
        self.species = i4() if species else None
        self.seg_cells = seg_cells
        self.seg_threads = seg_threads
        self.seg_list_smem = seg_list_smem
        self.seg_half = int(seg_half)
        if seg_cells is None:
            self.idx = torch.empty(((n + 31) // 32) * 32 * ld, dtype=torch.int32, device=device)
            self.seg = None
        else:
            self.idx = None
            self.seg = torch.empty(max(16, seg_list_bytes), dtype=torch.uint8, device=device)
        self.seg_status = torch.zeros((), dtype=torch.int32, device=device)
        self.flags = 0
        self.cnt = i4()
        self.err = torch.zeros((), dtype=torch.uint8, device=device)
        self.occ = torch.zeros((), dtype=torch.int64, device=device)
        self.flag = torch.zeros((), dtype=torch.int32, device=device)
        self.ws = torch.empty(workspace_bytes, dtype=torch.uint8, device=device)

    def struct(self) -> N.SortedState:
        z = N.SortedState()
        z.position_a, z.position_b = self.xa.data_ptr(), self.xb.data_ptr()
        z.momentum, z.force = self.p.data_ptr(), self.f.data_ptr()
        z.reference_position = self.ref.data_ptr()
        z.scratch4a, z.scratch4b = self.t4a.data_ptr(), self.t4b.data_ptr()
        z.species = N.ptr(self.species)
        z.perm, z.scratch_i_a, z.scratch_i_b = self.perm.data_ptr(), self.tia.data_ptr(), self.tib.data_ptr()
        z.idx, z.idx_ld, z.nbr_count = N.ptr(self.idx), self.ld, self.cnt.data_ptr()
        z.error_code, z.occupancy = self.err.data_ptr(), self.occ.data_ptr()
        z.rebuild_flag = self.flag.data_ptr()
        z.workspace, z.workspace_bytes = self.ws.data_ptr(), self.ws.numel()
        if self.seg is not None:
            z.seg_list, z.seg_list_bytes = self.seg.data_ptr(), self.seg.numel()
            z.seg_cells, z.seg_threads = self.seg_cells, self.seg_threads
            z.seg_list_smem = self.seg_list_smem
            z.seg_half = self.seg_half
        z.seg_status = self.seg_status.data_ptr()
        z.flags = self.flags
        return z


def _segment_shape(nbrs, layout):
    """(cells per segment, threads per CTA, list bytes, list staging bytes,
    half lists) for a run, or None for the tiled list.  `layout`: None
    (autotuned choice, else full segment lists with the default width),
    'segment' / 'half' (full / half lists, default width), an int (cells), a
    (cells, threads[, stage_lists[, half]]) tuple, or 'tiled'."""
    if layout == 'tiled':
        return None
    nl = nbrs.plan.nl
    threads, stage, half = None, True, False
    if layout is None:
        # untuned default: full lists, which are bitwise reproducible run to
        # run (the half lists' cross-segment force sums are float atomics)
        choice = _segment_choice.get(_grid_key(nl), (SEGMENT_CELLS_DEFAULT, None, True, False))
        if choice == 'tiled':
            return None
        cells, threads, stage, half = (tuple(choice) + (True, False))[:4]
    elif layout in ('segment', 'half'):
        cells, half = SEGMENT_CELLS_DEFAULT, layout == 'half'
    elif isinstance(layout, (tuple, list)):
        cells, threads = int(layout[0]), int(layout[1])
        stage = bool(layout[2]) if len(layout) > 2 else True
        half = bool(layout[3]) if len(layout) > 3 else False
    else:
        cells = int(layout)
    plan = segment_plan(nl, cells)
    if plan is None:
        if layout not in (None, 'segment', 'half'):
            raise ValueError('the segment layout does not apply to this cell grid')
        return None
    cells = plan[3]
    if threads is None:
        threads = segment_threads_default(cells, nl.cell_capacity)
    smem = segment_list_smem(nl, cells, nbrs.plan.n) if (stage and not half) else 0
    if smem and plan[2] + smem + 4096 > 227 * 1024:
        smem = 0   # positions and list block do not fit one CTA together
    return cells, threads, plan[4], smem, int(half)


def _sorted_buffers(state, nbrs, species, seg=None):
    plan = nbrs.plan
    key = (plan.ld, species is not None, plan.workspace.numel(), seg)
    b = getattr(state, '_sorted', None)
    if b is None or b.n != state.position.shape[0] or getattr(b, 'key', None) != key:
        b = _SortedBuffers(state.position.shape[0], plan.ld, species is not None,
                           plan.workspace.numel(), state.position.device,
                           *(() if seg is None else seg))
        b.key = key
        object.__setattr__(state, '_sorted', b)
    return b


def last_run_status(state) -> int:
    """Status word of the last sorted run on `state`: 0, or bit 1 (a segment
    neighbourhood exceeded its staging capacity; the run's list also carries
    the cell-list overflow bit) / bit 2 (a staging copy timed out)."""
    b = getattr(state, '_sorted', None)
    return 0 if b is None else int(b.seg_status)


def _run_loop(apply_fn, state, neighbor, n_steps, neighbor_fn, max_reallocations):
    """nbrs = nbrs.update(x); state = apply_fn(state, neighbor=nbrs), n_steps
    times, repeated from the start with a re-allocated list on overflow."""
    snapshot = state.copy() if neighbor_fn is not None else None
    for attempt in range(max_reallocations + 1):
        for _ in range(int(n_steps)):
            neighbor = neighbor.update(state.position)
            state = apply_fn(state, neighbor=neighbor)
        if neighbor_fn is None or not bool(neighbor.did_buffer_overflow):
            return state, neighbor
        state = snapshot.copy()
        extra = (attempt + 1) * max(1, neighbor.max_occupancy // 8)
        neighbor = neighbor_fn.allocate(state.position, extra_capacity=extra)
    raise RuntimeError('neighbour list kept overflowing after re-allocation')


def run(apply_fn, state, neighbor, n_steps: int, neighbor_fn=None, use_graph: bool = True,
        max_reallocations: int = 4, sort=None, layout=None, lazy_list: bool = True,
        warm_start: bool = True):
    """Runs the reference loop body ``n_steps`` times on the device:

        nbrs = nbrs.update(state.position); state = apply_fn(state, neighbor=nbrs)

    (jax_md/partition.py:841-854) as fused kernels, replayed from a CUDA graph
    whose per-step rebuild sits in a device-side conditional node.  With
    ``neighbor_fn``, overflow is handled as the reference's host loop does:
    the run is repeated from its starting state with a list re-allocated there.

    ``sort`` (default: when the mass is a scalar and a cell grid exists) keeps
    the atoms in cell order inside the run so neighbour gathers are
    coalesced; on return the state is back in the caller's order and the
    caller's list is rebuilt, in the reference's entry order, at the
    positions of the last rebuild -- when it is first read (``lazy_list``) or
    before returning.  ``layout`` picks the private list of a sorted run:
    None / 'segment' (the segment-local list wherever it applies, with the
    autotuned or default cells per segment), an int (that many cells per
    segment), or 'tiled' (the tiled int32 list).  A sorted run that continues
    the previous run of the same state and list keeps its private cell order
    and list (``warm_start``) and rebuilds only when the skin test asks;
    ``warm_start=False`` re-sorts and rebuilds at the start of every run (one
    CUDA graph per run length instead of two).  Returns (state, neighbor)."""
    st = apply_fn.stepper
    e = st.energy_fn
    if isinstance(e, smap.PairNeighborListEnergy) and e.has_particle_arrays():
        # per-particle parameter arrays: the generic pair kernels, step by
        # step -- the reference's own loop (partition.py:841-854)
        return _run_loop(apply_fn, state, neighbor, n_steps, neighbor_fn, max_reallocations)
    if isinstance(st.shift_fn, _space.GeneralShift) or isinstance(
            getattr(e, 'geometry', None), _space.GeneralDisplacement):
        # periodic_general cells: the same loop on the generic kernels
        return _run_loop(apply_fn, state, neighbor, n_steps, neighbor_fn, max_reallocations)
    nvt = isinstance(state, NVTNoseHooverState)
    if not (isinstance(state, NVEState) or nvt):
        raise NotImplementedError('run() drives NVE and Nose-Hoover NVT states')
    if nvt and getattr(apply_fn, 'chain_fns', None) is None:
        raise ValueError('an NVT state needs the apply_fn of simulate.nvt_nose_hoover')
    snapshot = state.copy() if neighbor_fn is not None else None
    chain0 = state.chain.buffer.clone() if (nvt and neighbor_fn is not None) else None
    for attempt in range(max_reallocations + 1):
        alt = getattr(state, '_alt', None)
        if alt is None or alt.shape[0] != state.position.shape[0]:
            alt = torch.empty((state.position.shape[0], 4), dtype=torch.float32,
                              device=state.position.device)
            object.__setattr__(state, '_alt', alt)
        sysd, species = _nve_system(st, state, neighbor, alt)
        use_sort = sort
        if use_sort is None:
            use_sort = (not isinstance(state.mass, torch.Tensor)) and bool(sysd.nlist.use_cell_list)
        v = _nvt_struct(apply_fn.chain_fns, state) if nvt else None
        if use_sort:
            seg = _segment_shape(neighbor, layout)
            sb = _sorted_buffers(state, neighbor, species, seg)
            # the private copy continues the previous run of this state on
            # this list: its first rebuild is taken only if the skin test
            # (or a pending flag, an error) asks for it
            warm_key = (id(neighbor.plan), neighbor.plan.nl.max_occupancy,
                        neighbor.plan.nl.cell_capacity, seg, nvt)
            warm = warm_start and getattr(sb, 'warm_key', None) == warm_key
            sb.flags = ((N.RUN_SKIP_EXIT_LIST if lazy_list else 0) |
                        (N.RUN_WARM_START if warm else 0))
            z = sb.struct()
            neighbor.set_pending_build(None)
            if nvt:
                N.check(N.lib().jmd_nvt_run_sorted(ctypes.byref(sysd), ctypes.byref(z),
                                                   ctypes.byref(v), int(n_steps),
                                                   1 if use_graph else 0, N.stream_ptr()),
                        'nvt_run_sorted')
            else:
                N.check(N.lib().jmd_nve_run_sorted(ctypes.byref(sysd), ctypes.byref(z),
                                                   int(n_steps), 1 if use_graph else 0,
                                                   N.stream_ptr()), 'nve_run_sorted')
            sb.warm_key = warm_key
            if lazy_list:
                nb = neighbor
                neighbor.set_pending_build(lambda: partition.build_at_reference(nb))
        elif nvt:
            neighbor.idx  # a deferred build of the caller's list must land first
            N.check(N.lib().jmd_nvt_run(ctypes.byref(sysd), ctypes.byref(v), int(n_steps),
                                        1 if use_graph else 0, N.stream_ptr()), 'nvt_run')
        else:
            neighbor.idx
            N.check(N.lib().jmd_nve_run(ctypes.byref(sysd), int(n_steps), 1 if use_graph else 0,
                                        N.stream_ptr()), 'nve_run')
        if neighbor_fn is None:
            return state, neighbor
        if use_sort and last_run_status(state) & 2:
            raise N.NativeError('a segment staging copy did not complete within its wait limit')
        if not bool(neighbor.did_buffer_overflow):
            return state, neighbor
        # overflow: restore the starting state, re-allocate there (with growing
        # headroom, so a block whose occupancy peaks above the start's fits), repeat
        state.position.copy_(snapshot.position)
        state.momentum.copy_(snapshot.momentum)
        state.force.copy_(snapshot.force)
        if chain0 is not None:
            state.chain.buffer.copy_(chain0)
        extra = (attempt + 1) * max(1, neighbor.max_occupancy // 8)
        neighbor = neighbor_fn.allocate(state.position, extra_capacity=extra)
    raise RuntimeError('neighbour list kept overflowing after re-allocation')
