"""The staged force pass (senders staged in shared memory one plane of cells
at a time, ``SPH_FORCE_STAGED``) against the gathering force pass
(``SPH_FORCE_GATHER``, the default).

Both evaluate each receiver's pairs in the order of the density pass's list
with the same arithmetic, so rollouts through either are the same bits:
every state field after the steps is compared with ``torch.equal``. Cases:
the benchmark's 3D transport-velocity Taylor-Green vortex on 64^3 (16-bit
lists) with candidate rebuilds inside the steps, the 2D vortex, artificial
viscosity, a dense clump (receivers on the slow paths, stages whose rows
hold more senders than the tile), and the 32-bit list format (80^3).
"""

import numpy as np
import pytest
import torch

from jaxsph_gb300 import _lib, cases, simulate
from test_gpu_lean_paths import _clumped_tgv

pytestmark = pytest.mark.gpu


def _rollout(setup, variant, steps):
    sim = simulate.Simulation(setup)
    sim.engine.set_force_variant(variant)
    code = sim.run(steps, check_every=steps)
    assert code & (0x4 | 0x8 | 0x800) == 0, code
    return sim.engine.list_format(), {k: v.cpu() for k, v in sim.state()[0].items()}


def _same_bits(setup, steps, fmt):
    f_a, a = _rollout(setup, _lib.FORCE_GATHER, steps)
    f_b, b = _rollout(setup, _lib.FORCE_STAGED, steps)
    assert f_a == f_b == fmt
    assert a.keys() == b.keys()
    for k in a:
        assert torch.equal(a[k], b[k]), k


def test_tgv3d_64_bitwise():
    _same_bits(cases.tgv(dim=3, dx=2 * np.pi / 64), 12, 1)


def test_tgv2d_bitwise():
    _same_bits(cases.tgv(dim=2, dx=1.0 / 128), 12, 1)


def test_artificial_viscosity_bitwise():
    _same_bits(cases.tgv(dim=3, dx=2 * np.pi / 32, artificial_alpha=0.1), 8, 1)


def test_dense_clump_bitwise():
    _same_bits(_clumped_tgv(), 4, 1)


def test_32bit_lists_bitwise():
    _same_bits(cases.tgv(dim=3, dx=2 * np.pi / 80), 3, 2)
