"""Verlet candidate lists: the skin changes how often candidates are rebuilt,
never a neighbour set.

Every step filters its candidates with the reference's exact membership test.
With ``canonical_order`` the pair sums run in ascending original index, so a
rollout is then bit for bit the same whatever the skin (a neighbour missed
under a skin would show as a difference), whether the rebuild is decided on
the device (graph replay) or by the host (eager steps). In the default cell
order a rollout is deterministic and matches within float32 rounding.
"""

import numpy as np
import pytest
import torch

from jaxsph_gb300 import cases, simulate

pytestmark = pytest.mark.gpu

KEYS = ("r", "u", "v", "rho", "p", "dudt", "dvdt")


def jittered_tgv3d(n_side=16, amp=0.2, seed=0):
    s = cases.tgv(dim=3, dx=2 * np.pi / n_side)
    rng = np.random.default_rng(seed)
    L = 2 * np.pi
    r = s.state["r"].double().numpy() + rng.uniform(-amp, amp, (s.n, 3)) * (L / n_side)
    s.state["r"] = torch.as_tensor(np.mod(r, L), dtype=torch.float32)
    return s


def rollout(setup, steps, skin, eager=False, canonical=True, **kw):
    sim = simulate.Simulation(setup, skin=skin, canonical_order=canonical, **kw)
    if eager:
        sim.engine.profile(steps)  # eager steps: the host reads each rebuild decision
    else:
        sim.run(steps)
    return sim, sim.state()


@pytest.mark.parametrize("make", [jittered_tgv3d,
                                  lambda: cases.tgv(dim=2, dx=1.0 / 40),
                                  lambda: cases.dam_break(dx=0.02)])
def test_skin_does_not_change_results(make):
    setup = make()
    steps = 120
    sim0, ref = rollout(setup, steps, 0.0)
    n0, _ = sim0.engine.rebuild_stats()
    # without a skin every step that moves a particle rebuilds (a case that
    # starts at rest does not move in its first step)
    assert n0 >= steps - 1
    for skin in (0.1, 0.3):
        sim, got = rollout(setup, steps, skin)
        n, _ = sim.engine.rebuild_stats()
        assert n < n0
        for a, b in zip(ref, got):
            for k in KEYS:
                assert torch.equal(a[k], b[k]), (skin, k)


def test_graph_replay_equals_eager_steps():
    setup = jittered_tgv3d(12, seed=1)
    _, a = rollout(setup, 60, 0.2)
    _, b = rollout(setup, 60, 0.2, eager=True)
    for k in KEYS:
        assert torch.equal(a[0][k], b[0][k]), k


def test_rebuilds_follow_the_displacement():
    # a case at rest (lattice, no velocity) never moves far enough to need a
    # rebuild after the one that loading it made
    setup = cases.tgv(dim=2, dx=1.0 / 32)
    for k in ("u", "v"):
        setup.state[k] = torch.zeros_like(setup.state[k])
    sim = simulate.Simulation(setup, skin=0.1)
    sim.run(30)
    n, per = sim.engine.rebuild_stats()
    assert n <= 1 and per > 0


def test_cell_order_is_deterministic_and_close():
    setup = jittered_tgv3d(12, seed=2)
    _, a = rollout(setup, 60, 0.2, canonical=False)
    _, b = rollout(setup, 60, 0.2, canonical=False)
    _, c = rollout(setup, 60, 0.2, canonical=True)
    for k in KEYS:
        assert torch.equal(a[0][k], b[0][k]), k
    L = 2 * np.pi
    d = a[0]["r"] - c[0]["r"]
    d = d - L * torch.round(d / L)
    assert float(d.abs().max()) < 1e-5 * L
    assert float((a[0]["rho"] - c[0]["rho"]).abs().max()) < 1e-5
