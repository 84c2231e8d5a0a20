"""The batched form: many independent cavities/channels advanced as one batch.

Every instance of a batch must come out bit for bit equal to the same
instance run alone (the batch only changes indices, never arithmetic), the
launch shape picked by the autotuner must not change any result, and a batched
instance must match the float64 oracle like a plain run does.
"""

import pytest
import torch

from jaxsph_gb300 import autotune, cases, simulate
from oracle_setup import oracle_rollout

pytestmark = pytest.mark.gpu

KEYS = ("r", "u", "v", "rho", "p", "dudt", "dvdt")


def small_batch(n=6, seed=1):
    return cases.cavity_channel_batch(n, seed=seed, n_min=100, n_max=900, dx_min=0.02,
                                      dx_max=0.08)


def test_batch_equals_individual_runs_bitwise():
    # in canonical order a case's sums do not depend on when the batch
    # rebuilt its candidate lists
    batch = small_batch()
    sim = simulate.Simulation(batch, canonical_order=True)
    sim.run(15)
    got = sim.state()
    assert len(got) == len(batch)
    for setup, st in zip(batch, got):
        alone = simulate.Simulation(setup, canonical_order=True)
        alone.run(15)
        ref = alone.state()[0]
        for k in KEYS:
            assert torch.equal(st[k], ref[k]), k


def test_block_size_does_not_change_results(tmp_path, monkeypatch):
    monkeypatch.setenv("JAXSPH_GB300_CACHE", str(tmp_path))
    batch = small_batch(4, seed=2)
    a = simulate.Simulation(batch, block_size=64)
    a.run(10)
    b = simulate.Simulation(batch, autotune=True)
    assert b.block_size in autotune.CANDIDATES
    b.run(10)
    for sa, sb in zip(a.state(), b.state()):
        for k in KEYS:
            assert torch.equal(sa[k], sb[k]), k
    # the second tuning of the same shape comes from the cache
    c = simulate.Simulation(batch, autotune=True)
    assert c.block_size == b.block_size


def test_batched_instance_matches_float64_oracle():
    batch = small_batch(3, seed=3)
    sim = simulate.Simulation(batch)
    steps = 20
    sim.run(steps)
    got = sim.state()
    for setup, st in zip(batch, got):
        ref = oracle_rollout(setup, steps, torch.float64)
        F = setup.p_ref / setup.dx + max(abs(x) for x in setup.g_ext_fn.spec["g"])
        assert (st["rho"].double().cpu() - ref["rho"]).abs().max().item() <= 2e-5
        du = (st["u"].double().cpu() - ref["u"]).abs().max().item()
        assert du <= 1e-4 * (setup.u_ref + F * setup.dt)
