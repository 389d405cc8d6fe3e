"""Differentiating NVE trajectories: a device-resident adjoint of velocity Verlet.

The forward pass is the reference's loop (simulate.py:227-243, with the
neighbour update of partition.py:841-854 before every step):

    q_s     = p_s + h F(x_s)            h = dt / 2
    x_{s+1} = shift(x_s, dt q_s / m)
    p_{s+1} = q_s + h F(x_{s+1})

jax.grad through that loop keeps every intermediate on a tape.  Here the
forward runs in the engine (jmd_nve_run_recorded: one CUDA graph per segment,
positions written straight into trajectory slots), and the reverse pass is
jmd_nve_adjoint_segment, which needs one force VJP per step because F(x_s)
enters the closing half kick of step s-1 and the opening half kick of step s
with the same cotangent:

    xbar += h VJP(x_n, pbar)
    for s = n-1 .. 0:   qbar = pbar + (dt/m) xbar
                        xbar += w_s VJP(x_s, qbar)     w_s = dt (s > 0), h (s = 0)
                        pbar = qbar

The periodic wrap is the identity for derivatives.  The trajectory is kept in
HBM when it fits (``checkpoint_every=None`` picks the longest segment that
fits a quarter of free device memory); otherwise (position, momentum, force)
is checkpointed at each segment start and the segment is replayed before its
reverse pass.  Every segment starts with a forced list rebuild, so a replay
repeats the forward bit for bit.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _native as N
from . import partition, quantity, simulate, smap
from .smap import _bins_to_grads, _param_tensor


def rebuild_now(neighbor_fn, nbrs, R):
    """Rebuilds ``nbrs`` at R unconditionally (same capacities), in place."""
    nbrs.plan.flag.fill_(1)
    return neighbor_fn.update(R, nbrs)


class _Buffers:
    """Device buffers of one trajectory computation (reused across calls so
    the engine's cached graphs stay valid)."""

    def __init__(self, n, dim, k, n_seg, device):
        f4 = lambda *s: torch.zeros(s + (n, 4), dtype=torch.float32, device=device)
        self.n, self.dim, self.k, self.n_seg = n, dim, k, n_seg
        self.x, self.p, self.f, self.alt = f4(), f4(), f4(), f4()
        self.traj = f4(k + 1)
        self.ck_x, self.ck_p, self.ck_f = f4(n_seg), f4(n_seg), f4(n_seg)
        self.xbar, self.pbar = f4(), f4()
        self.rec = torch.zeros((2 * n, 4), dtype=torch.float32, device=device)
        self.bins = torch.zeros(130, dtype=torch.float64, device=device)
        self.busy = False

    def fits(self, n, dim, k, n_seg, device):
        return (not self.busy and self.n == n and self.dim == dim and self.k == k
                and self.n_seg == n_seg and self.x.device == device)


class _Lease:
    """Marks a buffer set busy while an autograd graph may still need it."""

    def __init__(self, buf):
        self.buf = buf
        buf.busy = True

    def __del__(self):
        self.buf.busy = False


def _run(sysd, traj, steps):
    N.check(N.lib().jmd_nve_run_recorded(ctypes.byref(sysd), N.ptr(traj), int(steps), 1, 1,
                                         N.stream_ptr()), 'nve_run_recorded')


class _TrajectoryFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, R0, P0, sigma, epsilon, cfg):
        tf, nbrs, dyn = cfg
        R0d, P0d = R0.detach(), P0.detach()
        n, dim = R0d.shape
        buf, segs = tf.buffers(n, dim, R0d.device)
        lease = _Lease(buf)
        buf.x.zero_()
        buf.p.zero_()
        buf.x[:, :dim].copy_(R0d)
        buf.p[:, :dim].copy_(P0d)
        mass = simulate.canonicalize_mass(tf.mass, n, R0d.device)
        nb = rebuild_now(tf.neighbor_fn, nbrs, buf.x[:, :dim])
        tf.energy_fn.forces(buf.x[:, :dim], nb, out=buf.f[:, :dim], **dyn)
        sysd, species = tf.system(buf, nb, dyn, mass)
        for c, (s0, s1) in enumerate(segs):
            last = c == len(segs) - 1
            if not last:
                buf.ck_x[c].copy_(buf.x)
                buf.ck_p[c].copy_(buf.p)
                buf.ck_f[c].copy_(buf.f)
            _run(sysd, buf.traj if last else None, s1 - s0)
        if bool(nb.did_buffer_overflow):
            raise RuntimeError('neighbour list overflowed during the trajectory; allocate it '
                               'with more capacity (extra_capacity) and call again')
        out = buf.x[:, :dim].clone(), buf.p[:, :dim].clone()
        if any(ctx.needs_input_grad[:4]):
            ctx.lease = lease
            ctx.cfg = (tf, nb, sysd, species, mass, segs, buf)
            ctx.has = (sigma is not None, epsilon is not None)
            ctx.save_for_backward(sigma if sigma is not None else torch.empty(0),
                                  epsilon if epsilon is not None else torch.empty(0))
        else:
            del lease
        return out

    @staticmethod
    def backward(ctx, gx, gp):
        tf, nb, sysd, species, mass, segs, buf = ctx.cfg
        sigma, epsilon = ctx.saved_tensors
        sigma = sigma if ctx.has[0] else None
        epsilon = epsilon if ctx.has[1] else None
        dim = buf.dim
        buf.xbar.zero_()
        buf.pbar.zero_()
        if gx is not None:
            buf.xbar[:, :dim].copy_(gx)
        if gp is not None:
            buf.pbar[:, :dim].copy_(gp)
        want = sigma is not None or epsilon is not None
        if want:
            buf.bins.zero_()
        L = N.lib()
        for c in reversed(range(len(segs))):
            s0, s1 = segs[c]
            last = c == len(segs) - 1
            if not last:
                buf.x.copy_(buf.ck_x[c])
                buf.p.copy_(buf.ck_p[c])
                buf.f.copy_(buf.ck_f[c])
                _run(sysd, buf.traj, s1 - s0)
            N.check(L.jmd_nve_adjoint_segment(ctypes.byref(sysd), buf.traj.data_ptr(), s1 - s0,
                                              1 if last else 0, 1 if c == 0 else 0,
                                              buf.xbar.data_ptr(), buf.pbar.data_ptr(),
                                              buf.rec.data_ptr(),
                                              buf.bins.data_ptr() if want else None, 1,
                                              N.stream_ptr()), 'nve_adjoint_segment')
        gs, ge = _bins_to_grads(buf.bins, None, sigma, epsilon) if want else (None, None)
        gR, gP = buf.xbar[:, :dim].clone(), buf.pbar[:, :dim].clone()
        ctx.lease = None
        return gR, gP, gs, ge, None


class Trajectory:
    """``traj(R0, P0, nbrs, sigma=None, epsilon=None) -> (x_n, p_n)``: n_steps of
    NVE from (R0, P0), differentiable with respect to R0, P0 and sigma /
    epsilon tensors that require grad (species matrices or scalars).

    ``nbrs`` is a Dense list of ``neighbor_fn`` (it is rebuilt in place during
    the call and left valid).  One buffer set per concurrent autograd graph is
    kept for reuse, so repeated calls replay cached CUDA graphs."""

    def __init__(self, energy_fn, neighbor_fn, shift_fn, dt, n_steps, checkpoint_every=None,
                 mass=1.0):
        if not isinstance(energy_fn, smap.PairNeighborListEnergy):
            raise NotImplementedError('nve_trajectory needs a neighbour-list energy from '
                                      'jax_md_gb300.energy')
        if int(n_steps) < 1:
            raise ValueError('n_steps must be >= 1')
        self.energy_fn, self.neighbor_fn, self.shift_fn = energy_fn, neighbor_fn, shift_fn
        self.dt, self.n_steps = dt, int(n_steps)
        self.checkpoint_every = checkpoint_every
        self.mass = mass
        self.integrator = simulate.nve(energy_fn, shift_fn, dt)
        self.pool = []

    def segment_length(self, n):
        if self.checkpoint_every is not None:
            return max(1, min(int(self.checkpoint_every), self.n_steps))
        free, _ = torch.cuda.mem_get_info()
        k = int(free // 4 // (16 * max(n, 1))) - 1
        return max(1, min(k, self.n_steps))

    def buffers(self, n, dim, device):
        k = self.segment_length(n)
        segs = [(s0, min(s0 + k, self.n_steps)) for s0 in range(0, self.n_steps, k)]
        for b in self.pool:
            if b.fits(n, dim, k, len(segs), device):
                return b, segs
        b = _Buffers(n, dim, k, len(segs), device)
        self.pool.append(b)
        return b, segs

    def system(self, buf, nb, dyn, mass):
        _, apply = self.integrator
        st = simulate.NVEState(buf.x[:, :buf.dim], buf.p[:, :buf.dim], buf.f[:, :buf.dim], mass)
        sysd, _ = simulate._nve_system(apply.stepper, st, nb, buf.alt)
        species, pair = self.energy_fn._resolve(st.position, dyn)
        sysd.pair = pair
        sysd.species = N.ptr(species)
        return sysd, species

    def __call__(self, R0, P0, nbrs, sigma=None, epsilon=None):
        if nbrs.format is not partition.Dense:
            raise NotImplementedError('the adjoint runs on Dense neighbour lists')
        dyn = {}
        if sigma is not None:
            dyn['sigma'] = sigma
        if epsilon is not None:
            dyn['epsilon'] = epsilon
        return _TrajectoryFn.apply(R0, P0, _param_tensor(sigma), _param_tensor(epsilon),
                                   (self, nbrs, dyn))


def nve_trajectory(energy_fn, neighbor_fn, shift_fn, dt: float, n_steps: int,
                   checkpoint_every: Optional[int] = None, mass=1.0) -> Trajectory:
    """Differentiable NVE run (see Trajectory).  ``checkpoint_every=None`` keeps
    the whole trajectory on the device when it fits in a quarter of free memory
    and otherwise splits the run into the longest segments that do."""
    return Trajectory(energy_fn, neighbor_fn, shift_fn, dt, n_steps, checkpoint_every, mass)


# ---------------------------------------------------------------------------
# Nose-Hoover NVT (simulate.py:565-669)
#
# Forward step k from (x_k, p_k, chain_k), H the chain half step:
#     (chain', s1) = H(chain_k, KE(p_k))          update_mass, as apply_fn
#     q = s1 p_k + h F(x_k);  x_{k+1} = shift(x_k, dt q / m);  r = q + h F(x_{k+1})
#     (chain_{k+1}, s2) = H(chain', KE(r));  p_{k+1} = s2 r
# Reverse, with the chain cotangent pxibar (the chain momenta) and
# J_H^T from jmd_nhc_half_step_vjp:
#     sbar2 = pbar . r;  rbar = s2 pbar;  (pxibar', kebar) = J_H^T(pxibar, sbar2)
#     rbar += kebar r / m
#     xbar += VJP(x_{k+1}, h (rbar + qbar_{k+1}))      both kicks at x_{k+1}
#     qbar = rbar + (dt/m) xbar;  sbar1 = qbar . p_k;  pbar = s1 qbar
#     (pxibar, kebar) = J_H^T(pxibar', sbar1);  pbar += kebar p_k / m
# and finally xbar += VJP(x_0, h qbar_0).


def _nvt_steps(tf, st, nb, dyn, count, scale, tape=None):
    """``count`` steps of the Nose-Hoover integrator on ``st`` in place (the
    loop of NvtTrajectory's forward); with ``tape`` each step's
    (x_k, p_k, chain_a, s1, r, chain_b, s2) is appended."""
    init, apply = tf.integrator
    stepper, chain_fns = apply.stepper, apply.chain_fns
    P = st.momentum
    dim = P.shape[1]
    for _ in range(count):
        nb = nb.update(st.position)
        if tape is not None:
            x_k, p_k = st.position.clone(), st.momentum.clone()
            chain_a = st.chain.buffer.clone()
        chain_fns.half_step(st.chain, scale, update_mass=True)
        s1 = scale.clone() if tape is not None else None
        stepper.velocity_verlet(st, p_scale=scale, neighbor=nb, **dyn)
        r = st.momentum.clone() if tape is not None else None
        quantity._ke_f64(st.momentum, st.mass, out=st.chain.buffer[64])
        chain_b = st.chain.buffer.clone() if tape is not None else None
        chain_fns.half_step(st.chain, scale, ke=None)
        N.check(N.lib().jmd_scale_momentum(P.data_ptr(), P.stride(0), P.shape[0], dim,
                                           scale.data_ptr(), N.stream_ptr()), 'scale_momentum')
        if tape is not None:
            tape.append((x_k, p_k, chain_a, s1, r, chain_b, scale.clone()))
    return nb


def _nvt_checkpoint(st):
    return (st.position.clone(), st.momentum.clone(), st.force.clone(), st.chain.buffer.clone())


def _nvt_restore(st, ck):
    st.position.copy_(ck[0])
    st.momentum.copy_(ck[1])
    st.force.copy_(ck[2])
    st.chain.buffer.copy_(ck[3])


class _NvtTrajectoryFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, R0, P0, sigma, epsilon, cfg):
        tf, nbrs, dyn = cfg
        init, apply = tf.integrator
        R0d, P0d = R0.detach(), P0.detach()
        nb = rebuild_now(tf.neighbor_fn, nbrs, simulate._rows4(R0d))
        st = init(0, R0d, mass=tf.mass, momenta=P0d.clone(), neighbor=nb, **dyn)
        scale = torch.empty((), dtype=torch.float64, device=R0d.device)
        seg = tf.segment_length()
        tape, checkpoints = [], []
        done = 0
        while done < tf.n_steps:
            count = min(seg, tf.n_steps - done)
            if seg < tf.n_steps:
                # a segment starts from a fresh list, so its replay in the
                # reverse pass repeats these steps bit for bit
                nb = rebuild_now(tf.neighbor_fn, nb, st.position)
                checkpoints.append(_nvt_checkpoint(st))
            nb = _nvt_steps(tf, st, nb, dyn, count, scale, tape if seg >= tf.n_steps else None)
            done += count
        if bool(nb.did_buffer_overflow):
            raise RuntimeError('neighbour list overflowed during the trajectory; allocate it '
                               'with more capacity')
        ctx.cfg = (tf, nb, dyn, tape, checkpoints, seg, st, st.position.clone())
        ctx.has = (sigma is not None, epsilon is not None)
        ctx.save_for_backward(sigma if sigma is not None else torch.empty(0),
                              epsilon if epsilon is not None else torch.empty(0))
        return st.position.clone(), st.momentum.clone()

    @staticmethod
    def backward(ctx, gx, gp):
        tf, nb, dyn, full_tape, checkpoints, seg, st, x_n = ctx.cfg
        chain, mass = st.chain, st.mass
        sigma, epsilon = ctx.saved_tensors
        sigma = sigma if ctx.has[0] else None
        epsilon = epsilon if ctx.has[1] else None
        n, dim = x_n.shape
        dev = x_n.device
        dt = float(np.float32(tf.dt))
        h = float(np.float32(dt / 2))
        inv_m = (1.0 / mass[:, None]) if isinstance(mass, torch.Tensor) else 1.0 / float(mass)
        xbar = torch.zeros((n, 4), dtype=torch.float32, device=dev)[:, :dim]
        if gx is not None:
            xbar += gx
        pbar = torch.zeros((n, dim), dtype=torch.float32, device=dev)
        if gp is not None:
            pbar += gp
        bins = torch.zeros(130, dtype=torch.float64, device=dev)
        c = N.Nhc()
        c.chain_length, c.chain_steps, c.sy_steps = (tf.chain_length, tf.chain_steps,
                                                      tf.sy_steps)
        c.dof, c.dt, c.tau = chain.degrees_of_freedom, tf.dt32, chain.tau
        pxibar = torch.zeros(16, dtype=torch.float64, device=dev)
        pxibar1 = torch.zeros(16, dtype=torch.float64, device=dev)
        kebar = torch.zeros((), dtype=torch.float64, device=dev)
        scale = torch.empty((), dtype=torch.float64, device=dev)
        L = N.lib()

        def chain_vjp(chain_in, update_mass, cot_p, cot_s, out_p):
            N.check(L.jmd_nhc_half_step_vjp(ctypes.byref(c), chain_in.data_ptr(),
                                            chain_in[64:].data_ptr(), update_mass,
                                            cot_p.data_ptr(), cot_s.data_ptr(), out_p.data_ptr(),
                                            kebar.data_ptr(), N.stream_ptr()),
                    'nhc_half_step_vjp')

        def vjp_at(x, lam):
            nonlocal nb
            nb = nb.update(x)
            tf.energy_fn.force_vjp(x, nb, lam.contiguous(), 1.0, grad_R=xbar, grad_params=bins,
                                   **dyn)

        pending = None
        # segments in reverse; a checkpointed segment is replayed from its
        # checkpoint to rebuild its tape
        starts = list(range(0, tf.n_steps, seg)) if checkpoints else [0]
        x_end = x_n
        x_first = x_n
        for si in range(len(starts) - 1, -1, -1):
            if checkpoints:
                _nvt_restore(st, checkpoints[si])
                nb = rebuild_now(tf.neighbor_fn, nb, st.position)
                tape = []
                nb = _nvt_steps(tf, st, nb, dyn, min(seg, tf.n_steps - starts[si]), scale, tape)
            else:
                tape = full_tape
            for k in range(len(tape) - 1, -1, -1):
                x_k, p_k, chain_a, s1, r, chain_b, s2 = tape[k]
                x1 = tape[k + 1][0] if k + 1 < len(tape) else x_end
                sbar2 = (pbar.double() * r.double()).sum()
                rbar = pbar * s2.float()
                chain_vjp(chain_b, 0, pxibar, sbar2, pxibar1)
                rbar = rbar + (kebar.float() * r) * inv_m
                lam = h * (rbar if pending is None else rbar + pending)
                vjp_at(x1, lam)
                qbar = rbar + (dt * inv_m) * xbar
                sbar1 = (qbar.double() * p_k.double()).sum()
                pbar = qbar * s1.float()
                chain_vjp(chain_a, 1, pxibar1, sbar1, pxibar)
                pbar = pbar + (kebar.float() * p_k) * inv_m
                pending = qbar
            if tape:
                x_end = tape[0][0].clone()
                x_first = x_end
        vjp_at(x_first, h * pending if pending is not None else
               torch.zeros((n, dim), dtype=torch.float32, device=dev))
        gs, ge = _bins_to_grads(bins, None, sigma, epsilon)
        return xbar.contiguous(), pbar.contiguous(), gs, ge, None


class NvtTrajectory:
    """``traj(R0, P0, nbrs, sigma=None, epsilon=None) -> (x_n, p_n)``: n_steps
    of simulate.nvt_nose_hoover from (R0, P0) with a fresh chain, differentiable
    with respect to R0, P0 and sigma / epsilon tensors that require grad,
    through the reverse pass of the chain (jmd_nhc_half_step_vjp) and of the
    Verlet step (jmd_pair_force_vjp).  Every step is recorded (positions,
    momenta and the chain) when ``checkpoint_every`` is None, so memory grows
    with n_steps; with ``checkpoint_every=k`` only (position, momentum, force,
    chain) at every k-th step is kept and each k-step segment is replayed
    (from a forced list rebuild, as in the forward) before its reverse pass,
    so memory is O(n_steps / k + k) states at the price of one extra forward."""

    def __init__(self, energy_fn, neighbor_fn, shift_fn, dt, kT, n_steps, chain_length=5,
                 chain_steps=2, sy_steps=3, tau=None, mass=1.0, checkpoint_every=None):
        if not isinstance(energy_fn, smap.PairNeighborListEnergy):
            raise NotImplementedError('nvt_trajectory needs a neighbour-list energy from '
                                      'jax_md_gb300.energy')
        if not 2 <= int(chain_length) <= 7:
            raise NotImplementedError('the chain adjoint supports chain_length 2..7')
        if int(n_steps) < 1:
            raise ValueError('n_steps must be >= 1')
        self.energy_fn, self.neighbor_fn, self.shift_fn = energy_fn, neighbor_fn, shift_fn
        self.dt, self.kT, self.n_steps = dt, kT, int(n_steps)
        self.dt32 = float(np.float32(dt))
        self.chain_length, self.chain_steps, self.sy_steps = (int(chain_length), int(chain_steps),
                                                              int(sy_steps))
        self.mass = mass
        self.checkpoint_every = checkpoint_every
        self.integrator = simulate.nvt_nose_hoover(energy_fn, shift_fn, dt, kT, chain_length,
                                                   chain_steps, sy_steps, tau)

    def segment_length(self):
        if self.checkpoint_every is None:
            return self.n_steps
        return max(1, min(int(self.checkpoint_every), self.n_steps))

    def __call__(self, R0, P0, nbrs, sigma=None, epsilon=None):
        if nbrs.format is not partition.Dense:
            raise NotImplementedError('the trajectory adjoint runs on Dense neighbour lists')
        dyn = {}
        if sigma is not None:
            dyn['sigma'] = sigma
        if epsilon is not None:
            dyn['epsilon'] = epsilon
        return _NvtTrajectoryFn.apply(R0, P0, _param_tensor(sigma), _param_tensor(epsilon),
                                      (self, nbrs, dyn))


def nvt_trajectory(energy_fn, neighbor_fn, shift_fn, dt: float, kT: float, n_steps: int,
                   chain_length: int = 5, chain_steps: int = 2, sy_steps: int = 3, tau=None,
                   mass=1.0, checkpoint_every: Optional[int] = None) -> NvtTrajectory:
    """Differentiable Nose-Hoover NVT run (see NvtTrajectory)."""
    return NvtTrajectory(energy_fn, neighbor_fn, shift_fn, dt, kT, n_steps, chain_length,
                         chain_steps, sy_steps, tau, mass, checkpoint_every)
