"""Differentiable rollouts: hand-written adjoint with checkpointed recomputation.

The reference differentiates whole rollouts with ``jax.grad`` (integer
neighbour indices carry no gradient, so the list is frozen per step;
``notebooks/iclr24_grads.ipynb``, ``notebooks/iclr24_inverse.ipynb``) and
keeps the whole tape in memory. Here the forward rollout keeps a device
snapshot of the engine's state (particles in their binned order, binning,
candidate lists) every ``checkpoint_every`` steps; the reverse sweep restores
each segment's snapshot, re-runs the segment forward (bit-identical to the
original forward, pair sums in the same order), records its steps on the GPU
tape and applies the hand-written reverse step (``sph_adjoint_step``,
``csrc/sph_adjoint.cu``) from the last step to the first. Memory is one
segment of per-step data plus the snapshots.

``rollout`` wraps it as a ``torch.autograd.Function``: the gradient of any
torch loss of the final positions flows back to the initial velocity.
"""

import torch

from . import _lib
from .simulate import Simulation


class AdjointRollout:
    """``steps`` si_euler steps of one case, differentiable w.r.t. the initial
    positions and velocities.

    Covers the SPH solver with density summation, any transport-velocity
    factor and, optionally, the no-slip generalized wall BC with a velocity
    ``bc_fn`` (the reference's lid-driven cavity). ``forward(u0)`` starts from
    the case's initial state with ``u = v = u0`` (the reference initialises
    ``v`` with ``u``, case_setup.py:167-168) and ``dudt = dvdt = 0``; ``run``
    starts from any state.
    """

    def __init__(self, setup, steps, checkpoint_every=10, device="cuda", autotune=False):
        self.setup = setup
        self.steps = int(steps)
        self.k = int(checkpoint_every)
        # a segment restarts from a device snapshot of the engine's state, so
        # its recomputation equals the forward rollout bit for bit; the block
        # size changes no result
        self.sim = Simulation(setup, device=device, autotune=autotune)
        self.engine = self.sim.engine
        self.engine.adjoint_init(self.k)
        self.segments = -(-self.steps // self.k)
        if self.segments > 1:
            self.engine.snapshot_init(self.segments - 1)
        self.device = torch.device(device)
        self.start = None
        self._base = None

    def _initial(self, u0):
        """The case's initial state on the device with u = v = u0, dudt = 0."""
        if self._base is None:
            self._base = {k: v.to(self.device) for k, v in self.setup.state.items()}
        st = dict(self._base)
        u0 = u0.detach().to(device=self.device, dtype=torch.float32).contiguous()
        st["u"] = u0
        st["v"] = u0
        st["dudt"] = torch.zeros_like(st["dudt"])
        st["dvdt"] = torch.zeros_like(st["dvdt"])
        return st

    def run(self, state0):
        """Run the rollout from ``state0`` (a state dict); returns the final
        state (device tensors, original order), keeping the checkpoints: the
        initial state, then a device snapshot at every segment boundary."""
        self.sim.load([state0])  # capacities, as the reference's allocate
        # the first segment starts where its recomputation will: a loaded state
        self.start = self.sim.state(split=False)
        self.sim.restore(self.start)
        done = 0
        for seg in range(self.segments):
            if seg > 0:
                self.engine.snapshot_save(seg - 1)
            n = min(self.k, self.steps - done)
            self.engine.step(n)
            done += n
        code = self.engine.read_status(clear=True)
        if code & (_lib.ERR_NONFINITE | _lib.ERR_INVALID_ARG | _lib.ERR_CUDA):
            raise _lib.SphError(code, "rollout failed")
        return self.sim.state(split=False)

    def forward(self, u0):
        """Run the rollout from initial velocity ``u0``; returns the final positions."""
        return self.run(self._initial(u0))["r"].clone()

    def backward(self, lam_r, lam_u=None, timer=None):
        """Adjoints of the initial state for those of the final positions
        (``lam_r``) and velocities (``lam_u``): returns (d loss/d u0,
        d loss/d r0); those of the initial dudt and dvdt are kept in
        ``self.lam_dudt`` and ``self.lam_dvdt``. ``timer``: a list that gets,
        per checkpoint segment, three CUDA events recorded before the
        recomputation, between it and the reverse sweep, and after the sweep."""
        shape = lam_r.shape
        lr = lam_r.detach().to(self.device, torch.float32).contiguous().clone()
        lu = (torch.zeros_like(lr) if lam_u is None else
              lam_u.detach().to(self.device, torch.float32).contiguous().clone())
        la, lb = torch.zeros_like(lr), torch.zeros_like(lr)
        for seg in reversed(range(self.segments)):
            # recompute the segment from its checkpoint, recording its steps,
            # then sweep it backwards (one library call each)
            if seg == 0:
                self.sim.restore(self.start)
            else:
                self.engine.snapshot_restore(seg - 1)
            n = min(self.k, self.steps - seg * self.k)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)] if timer is not None else None
            if ev:
                ev[0].record()
            self.engine.tape_segment(n)
            if ev:
                ev[1].record()
            self.engine.adjoint_segment(n, lr, lu, la, lb)
            if ev:
                ev[2].record()
                timer.append(ev)
        code = self.engine.read_status(clear=True)
        if code & _lib.ERR_INVALID_ARG:
            raise _lib.SphError(code, "a particle has more neighbours than the adjoint tape holds")
        self.lam_dudt, self.lam_dvdt = la.reshape(shape), lb.reshape(shape)
        # u0 enters the first step as u; v0 does not reach the dynamics (the
        # kick recomputes v from u and dvdt)
        return lu.reshape(shape), lr.reshape(shape)


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, roll):
        ctx.roll = roll
        return roll.forward(u0).to(u0.device)

    @staticmethod
    def backward(ctx, grad_r):
        lu, _ = ctx.roll.backward(grad_r.contiguous())
        return lu.to(grad_r.device), None


def rollout(u0, roll):
    """Final positions of ``roll`` started from ``u0``, differentiable in ``u0``."""
    return _RolloutFn.apply(u0, roll)


def position_mse(r, target, box):
    """Mean over particles of the squared minimum-image distance to ``target``."""
    side = torch.as_tensor(box, dtype=r.dtype, device=r.device)
    d = r - target
    d = d - side * torch.round(d / side)
    return (d * d).sum(1).mean()
