"""The lean passes' less travelled paths, on the GPU against the oracle.

* Slow paths: a receiver with more neighbours than the step's list holds
  re-derives them from its candidates, and one with more candidates than the
  candidate list holds walks the cells of the last binning. A dense clump of
  100 particles (spacing dx / 4) in the 3D Taylor-Green lattice forces both:
  its particles have ~130 neighbours and candidates, their lattice neighbours
  more than the list's 40 slots.
* The 32-bit list format, taken when a few planes of cells hold more
  particles than 16-bit offsets reach: the 3D Taylor-Green vortex on 80^3
  (reach 38,400 > 32,767; the benchmark's 64^3 uses 16-bit offsets).

Bars as at the measured sizes (tests/test_gpu_full_size.py): neighbour sets
bit-exact against the float32 oracle, the per-particle sizes of the sets the
passes summed over equal to the oracle's, one forward pass within the
float32 tolerances against the float64 oracle (or 10x the float32 oracle's
own error).
"""

import numpy as np
import pytest
import torch

from jaxsph_gb300 import cases, simulate
from test_gpu_full_size import _check_sets, _forward_parity, _receiver_counts

pytestmark = pytest.mark.gpu


def _clumped_tgv():
    setup = cases.tgv(dim=3, dx=2 * np.pi / 24)
    r = setup.state["r"].clone()
    g = torch.Generator().manual_seed(3)
    pick = torch.randperm(setup.n, generator=g)[:100]
    c = torch.full((3,), float(np.pi), dtype=torch.float64)
    q = 0.25 * setup.dx
    grid = torch.stack(torch.meshgrid(torch.arange(5), torch.arange(5), torch.arange(4),
                                      indexing="ij"), -1).reshape(-1, 3).double()
    r[pick] = (c + q * (grid - grid.mean(0))).to(r.dtype)
    setup.state["r"] = r
    return setup


def _sets_and_counts(setup, fmt):
    sim = simulate.Simulation(setup)
    assert sim.engine.list_format() == fmt
    sim.engine.forward()
    got = sim.engine.neighbour_counts("cuda").cpu().long()
    ref = _check_sets(setup, setup.state["r"].cuda())
    want = _receiver_counts(ref.idx, setup.n)
    assert torch.equal(got, want)
    return want


def test_dense_clump_takes_the_slow_paths():
    setup = _clumped_tgv()
    counts = _sets_and_counts(setup, 1)
    # more neighbours than the step's list (40) and candidates than the
    # candidate list (80 slots) hold
    assert int(counts.max()) > 100 and int((counts > 41).sum()) >= 100
    st = {k: v for k, v in setup.state.items()}
    _forward_parity(setup, st)


@pytest.fixture(scope="module")
def tgv80():
    return cases.tgv(dim=3, dx=2 * np.pi / 80)


def test_32bit_lists_sets_bit_exact(tgv80):
    counts = _sets_and_counts(tgv80, 2)
    # 27 lattice points closer than 2 dx (self included) plus the exact ties
    # whose float32 metric falls below cutoff^2 (which of them depends on
    # the lattice's rounding)
    assert int(counts.min()) == 27 and 27 < int(counts.max()) <= 33


def test_32bit_lists_forward_and_steps(tgv80):
    setup = tgv80
    sim = simulate.Simulation(setup)
    assert sim.engine.list_format() == 2
    sim.run(4)
    st = {k: v.cpu() for k, v in sim.state()[0].items()}
    got = sim.engine.neighbour_counts("cuda").cpu().long()
    ref = _check_sets(setup, st["r"].cuda().contiguous())
    assert torch.equal(got, _receiver_counts(ref.idx, setup.n))
    _forward_parity(setup, st)
