"""FIRE minimisation (jax_md/minimize.py:97-226) on the GB300 kernels.

``fire_descent(energy_or_force, shift_fn, dt_start, dt_max, n_min, f_inc,
f_dec, alpha_start, f_alpha)`` returns ``(init_fn, apply_fn)`` like the
reference.  The minimiser's scalars (dt, alpha, n_pos) stay on the device, so a
FIRE step costs no host synchronisation: the step is a fused kick + drift, the
force kernel, and one reduction + mixing pass.  ``state.dt``, ``state.alpha``
and ``state.n_pos`` read the device values (a host sync when accessed).
State tensors are updated in place, as in ``simulate``.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np
import torch

from . import _native as N
from . import quantity
from . import simulate as _sim


@dataclasses.dataclass
class FireDescentState(_sim._StateMixin):
    """minimize.py:97-121; ``scalars`` holds [dt, alpha, n_pos, keep, alpha_mix, ratio]."""
    position: torch.Tensor
    momentum: torch.Tensor
    force: torch.Tensor
    mass: object
    scalars: torch.Tensor

    @property
    def dt(self):
        return self.scalars[0]

    @property
    def alpha(self):
        return self.scalars[1]

    @property
    def n_pos(self):
        return self.scalars[2].to(torch.int32)


def gradient_descent(energy_or_force, shift_fn, step_size: float):
    """minimize.gradient_descent (minimize.py:65-94): R <- shift(R,
    step_size F(R)); the state is the positions themselves."""
    force = quantity.canonicalize_force(energy_or_force)

    def init_fn(R, **unused_kwargs):
        return R

    def apply_fn(R, **kwargs):
        return shift_fn(R, step_size * force(R, **kwargs), **kwargs)

    return init_fn, apply_fn


def fire_descent(energy_or_force, shift_fn, dt_start=0.1, dt_max=0.4, n_min=5, f_inc=1.1,
                 f_dec=0.5, alpha_start=0.1, f_alpha=0.99):
    """minimize.fire_descent (minimize.py:124-226)."""
    st = _sim._Stepper(energy_or_force, shift_fn, dt_start)
    c = [float(np.float32(v)) for v in (dt_start, dt_max, n_min, f_inc, f_dec, alpha_start, f_alpha)]
    dt_start, dt_max, n_min, f_inc, f_dec, alpha_start, f_alpha = c

    def init_fn(R, mass=1.0, **kwargs):
        R4, F4 = st.new_state_tensors(R, **kwargs)
        P4 = _sim._rows4(torch.zeros_like(R4))
        m = _sim.canonicalize_mass(mass, R.shape[0], R.device)
        scalars = torch.tensor([dt_start, alpha_start, 0.0, 1.0, 0.0, 0.0], dtype=torch.float32,
                               device=R.device)
        return FireDescentState(R4, P4, F4, m, scalars)

    def apply_fn(state: FireDescentState, **kwargs):
        R, P, F = state.position, state.momentum, state.force
        for t, name in ((R, 'position'), (P, 'momentum'), (F, 'force')):
            if t.stride(0) != 4 or t.data_ptr() % 16:
                raise ValueError(f'state.{name} must be float4 rows (use init_fn of this module)')
        n, dim = R.shape
        L = N.lib()
        sp = _sim._shift_space(st.shift_fn, dim)
        mptr, m0 = _sim._mass_ptr(state.mass)
        N.check(L.jmd_fire_kick_drift(R.data_ptr(), P.data_ptr(), F.data_ptr(), mptr, m0, n,
                                      ctypes.byref(sp), state.scalars.data_ptr(), N.stream_ptr()),
                'fire_kick_drift')
        st.forces_into(R, F, **kwargs)
        ws = N.workspace(L.jmd_fire_workspace_bytes(n), R.device, 'fire')
        N.check(L.jmd_fire_update(P.data_ptr(), F.data_ptr(), n, dim, state.scalars.data_ptr(),
                                  dt_max, n_min, f_inc, f_dec, alpha_start, f_alpha,
                                  ws.data_ptr(), ws.numel(), N.stream_ptr()), 'fire_update')
        return state

    init_fn.stepper = st
    apply_fn.stepper = st
    return init_fn, apply_fn
