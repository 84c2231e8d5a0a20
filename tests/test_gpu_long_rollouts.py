"""Rollouts at the configured step counts, on the GPU against the float64
oracle from identical float32 inputs:

* the 3D transport-velocity Taylor-Green vortex (WC2K, Re = 1600) over 500
  steps, the length of the 3D TGV configuration;
* the Riemann dam break (QSK, gravity, 3 wall layers) over 2,000 steps, the
  length of the dam-break configuration.

The particle counts are reduced (32^3 = 32,768 particles; dam break at
dx = 0.02, 7,244 particles) so that the CPU oracle runs each rollout within
about a minute; the step counts are the configurations'. Over hundreds of
steps float32 rounding differences grow, so the bar is relative to what
float32 arithmetic of the same algorithm gives: the GPU's distance from the
float64 run is at most 10x the float32 oracle's own distance from it, or the
absolute floor (positions 1e-5 of the box, density 2e-4 rho_ref, velocity
1e-3 u_ref), whichever is larger; the same for the kinetic energy, a field
quantity that particle-level divergence leaves nearly unchanged (floor 1e-4
of its float64 value). The neighbour sets at the final GPU state are
bit-exact against the float32 oracle's.
"""

import numpy as np
import pytest
import torch

import oracle
from jaxsph_gb300 import cases, partition, simulate, space
from jaxsph_gb300.kernel import make_kernel
from oracle_setup import oracle_rollout

pytestmark = pytest.mark.gpu


def _err(a, b):
    return (a.detach().double().cpu() - b.detach().double().cpu()).abs().max().item()


def _sets_bit_exact(setup, r_dev):
    cutoff = make_kernel(setup.solver["kernel"], setup.dx, setup.dim).cutoff
    disp, _ = space.periodic(setup.box)
    nb = partition.neighbor_list(disp, setup.box, cutoff, mask_self=False).allocate(r_dev)
    ofns = oracle.partition.NeighborListFns(setup.box, cutoff, torch.float32, mask_self=False)
    ref = ofns.allocate(r_dev.detach().float().cpu())
    got = oracle.partition.canonical_edges(nb.idx.long().cpu(), setup.n)
    want = oracle.partition.canonical_edges(ref.idx, setup.n)
    return nb.occupancy == ref.occupancy and torch.equal(got, want)


def _check_rollout(setup, steps):
    sim = simulate.Simulation(setup)
    code = sim.run(steps, check_every=100)
    assert code & (0x4 | 0x8 | 0x800) == 0, code  # no cell-size, box or non-finite error
    got = sim.state()[0]
    ref = oracle_rollout(setup, steps, torch.float64)
    ref32 = oracle_rollout(setup, steps, torch.float32)
    side = torch.as_tensor(setup.box, dtype=torch.float64)
    box = float(np.max(setup.box))

    def drift(a):
        return oracle.space.periodic_displacement(
            side, a["r"].double().cpu() - ref["r"]).abs().max().item()

    rho0 = setup.eos.rho_ref
    fluid = ref["tag"] == cases.FLUID

    def ekin(a):
        m = a["mass"].double().cpu()[fluid]
        return float(0.5 * (m * (a["u"].double().cpu()[fluid] ** 2).sum(1)).sum())

    e64 = ekin(ref)
    res = {
        "E_kin": (abs(ekin(got) - e64), abs(ekin(ref32) - e64), 1e-4 * e64),
        "r": (drift(got), drift(ref32), 1e-5 * box),
        "rho": (_err(got["rho"], ref["rho"]), _err(ref32["rho"], ref["rho"]), 2e-4 * rho0),
        "u": (_err(got["u"], ref["u"]), _err(ref32["u"], ref["u"]), 1e-3 * setup.u_ref),
    }
    def mean_drift(a):
        return oracle.space.periodic_displacement(
            side, a["r"].double().cpu() - ref["r"]).norm(dim=1).mean().item()

    print({k: f"gpu {a:.2e} / float32 oracle {b:.2e}" for k, (a, b, _) in res.items()},
          f"mean |dr| gpu {mean_drift(got):.2e} / float32 oracle {mean_drift(ref32):.2e}",
          f"E_kin float64 {e64:.4e}")
    for k, (e_gpu, e_f32, floor) in res.items():
        assert e_gpu <= max(floor, 10 * e_f32), (k, e_gpu, e_f32, floor)
    assert _sets_bit_exact(setup, got["r"].cuda())


def test_tgv3d_500_steps_matches_float64():
    setup = cases.tgv(dim=3, dx=2 * np.pi / 32)
    assert setup.n == 32_768 and setup.tvf == 1.0
    _check_rollout(setup, 500)


def test_dam_break_2000_steps_matches_float64():
    setup = cases.dam_break(dx=0.02)
    _check_rollout(setup, 2000)
