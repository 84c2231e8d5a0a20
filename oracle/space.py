"""Periodic space restated from ``jax_sph/jax_md/space.py`` (test oracle only).

All arithmetic is done per op in the tensor dtype (float32 or float64), so that
float32 results round exactly like the reference's jitted float32 program with
no fused multiply-adds.
"""

import torch


def jnp_mod(x, side):
    """``jnp.mod`` for floats: C ``fmod`` then a sign fix.

    jax.numpy's ``remainder`` computes ``lax.rem`` (exact fmod) and adds the
    divisor when the remainder is non-zero and its sign differs from the
    divisor's. Used by ``periodic_displacement`` (jax_md/space.py:181) and
    ``periodic_shift`` (jax_md/space.py:207-209).
    """
    t = torch.fmod(x, side)
    fix = (t != 0) & ((t < 0) != (side < 0))
    return torch.where(fix, t + side, t)


def periodic_displacement(side, dR):
    """``mod(dR + side/2, side) - side/2`` (jax_md/space.py:170-181)."""
    half = side * 0.5
    return jnp_mod(dR + half, side) - half


def square_distance(dR):
    """``sum(dR**2, -1)`` (jax_md/space.py:184-192), summed left to right."""
    sq = dR * dR
    acc = sq[..., 0]
    for k in range(1, dR.shape[-1]):
        acc = acc + sq[..., k]
    return acc


def distance(dR):
    """``safe_mask(dr > 0, sqrt, dr)`` (jax_md/space.py:195-204, util.py:37-40)."""
    dr = square_distance(dR)
    pos = dr > 0
    return torch.where(pos, torch.sqrt(torch.where(pos, dr, torch.zeros_like(dr))),
                       torch.zeros_like(dr))


def periodic_shift(side, R, dR):
    """``mod(R + dR, side)`` (jax_md/space.py:207-209)."""
    return jnp_mod(R + dR, side)


class Periodic:
    """``space.periodic(side)`` (jax_md/space.py:232-286): displacement and shift."""

    def __init__(self, side):
        self.side = side

    def displacement(self, Ra, Rb):
        return periodic_displacement(self.side, Ra - Rb)

    def shift(self, R, dR):
        return periodic_shift(self.side, R, dR)
