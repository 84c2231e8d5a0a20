"""Periodic space: the ``(displacement_fn, shift_fn)`` pair of ``space.periodic``.

Mirrors ``jax_sph/jax_md/space.py:232-286``. The returned callables work on
torch tensors (any device) for user-side post-processing; the GPU hot path
reads only their ``side`` attribute and evaluates the same arithmetic inside
its kernels (``jmod``/``pdisp`` in ``csrc/sph_internal.cuh``).
"""

import numpy as np
import torch


def _mod(x, side):
    # jnp.mod semantics: fmod, then add the divisor to a negative remainder
    t = torch.fmod(x, side)
    return torch.where((t != 0) & (t < 0), t + side, t)


def square_distance(dR):
    """``jnp.sum(dR**2, axis=-1)`` (jax_md/space.py:184-192)."""
    return (dR * dR).sum(-1)


def distance(dR):
    """``safe_mask(dr > 0, sqrt, dr)`` (jax_md/space.py:195-204)."""
    d2 = square_distance(dR)
    return torch.where(d2 > 0, torch.sqrt(torch.clamp(d2, min=0)), torch.zeros_like(d2))


class PeriodicDisplacement:
    """``displacement_fn(Ra, Rb) = mod(Ra - Rb + side/2, side) - side/2``."""

    def __init__(self, side):
        self.side = np.asarray(side, dtype=np.float64).reshape(-1)

    def _side(self, like):
        return torch.as_tensor(self.side, dtype=like.dtype, device=like.device)

    def __call__(self, Ra, Rb, **unused):
        if "box" in unused:
            raise ValueError("space.periodic does not accept a box argument")
        s = self._side(Ra)
        return _mod(Ra - Rb + s * 0.5, s) - 0.5 * s


class PeriodicShift:
    """``shift_fn(R, dR) = mod(R + dR, side)`` (jax_md/space.py:207-209)."""

    def __init__(self, side, wrapped=True):
        self.side = np.asarray(side, dtype=np.float64).reshape(-1)
        self.wrapped = wrapped

    def __call__(self, R, dR, **unused):
        if "box" in unused:
            raise ValueError("space.periodic does not accept a box argument")
        if not self.wrapped:
            return R + dR
        s = torch.as_tensor(self.side, dtype=R.dtype, device=R.device)
        return _mod(R + dR, s)


def periodic(side, wrapped=True):
    """``space.periodic(side, wrapped)`` -> ``(displacement_fn, shift_fn)``."""
    return PeriodicDisplacement(side), PeriodicShift(side, wrapped)
