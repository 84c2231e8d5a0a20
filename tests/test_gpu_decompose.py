"""Slab decomposition on one GPU: every slab advanced by its own engine on its
owned particles plus a halo of two or three cutoffs and the drift; the result
must be the undivided run's, bit for bit (canonical pair order in both),
temperature fields and recomputed wall normals included."""

import numpy as np
import pytest
import torch

from jaxsph_gb300 import cases, decompose, simulate

pytestmark = pytest.mark.gpu

KEYS = ("r", "u", "v", "rho", "p", "dudt", "dvdt", "drhodt")


def jittered_tgv3d(n_side=14, amp=0.2, seed=4):
    s = cases.tgv(dim=3, dx=2 * np.pi / n_side)
    rng = np.random.default_rng(seed)
    L = 2 * np.pi
    r = s.state["r"].double().numpy() + rng.uniform(-amp, amp, (s.n, 3)) * (L / n_side)
    s.state["r"] = torch.as_tensor(np.mod(r, L), dtype=torch.float32)
    return s


@pytest.mark.parametrize("make,parts", [
    (jittered_tgv3d, 2),
    (jittered_tgv3d, 3),
    (lambda: cases.tgv(dim=2, dx=1.0 / 48), 4),
    (lambda: cases.dam_break(dx=0.04), 3),
    (lambda: cases.lid_driven_cavity(dx=0.04), 2),
    # heat conduction (temperature fields exchanged and kept) and moving-lid
    # Riemann walls (normals recomputed per slab)
    (lambda: cases.heat_transfer(dx=0.04), 2),
    (lambda: cases.lid_driven_cavity(dx=0.04, solver_name="RIE"), 2),
])
def test_slabs_equal_the_undivided_run(make, parts):
    setup = make()
    steps = 25
    ref = simulate.Simulation(setup, canonical_order=True)
    ref.run(steps)
    want = ref.state()[0]
    slabs = decompose.VirtualSlabs(setup, parts)
    slabs.step(steps)
    assert len(slabs.last_sizes) == parts
    assert sum(o for o, _ in slabs.last_sizes) == setup.n
    assert all(n < setup.n for _, n in slabs.last_sizes) or parts == 2
    keys = KEYS + (("T", "dTdt") if "T" in want else ()) + (
        ("nw",) if setup.nw_fn is not None else ())
    for k in keys:
        assert torch.equal(slabs.state[k], want[k]), k
