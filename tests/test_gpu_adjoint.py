"""The differentiable form: hand-written adjoint vs the float64 oracle.

Loss: mean squared minimum-image distance of the final positions to a target
rollout from another seed (the inverse problem of the reference's
notebooks/iclr24_inverse.ipynb); gradient w.r.t. the initial velocity.

* vs torch autograd through the float64 oracle rollout (neighbour list frozen
  per step, like jax.grad(..., allow_int=True)): relative L2 error <= 1e-4;
* vs float64 central finite differences of the oracle along seeded random
  directions: relative error of the directional derivatives <= 1e-3 (the FD
  truncation and the float32 forward set this floor).
"""

import pytest
import torch

import oracle
from jaxsph_gb300 import adjoint, cases
from oracle_setup import oracle_case

pytestmark = pytest.mark.gpu

N_SIDE, STEPS, K = 20, 12, 5


def setups():
    a = cases.tgv_perturbed(n_side=N_SIDE, seed=1)
    b = cases.tgv_perturbed(n_side=N_SIDE, seed=2)
    return a, b


def oracle_loss(setup, u0, target, frozen=None):
    """Float64 oracle rollout from u0; returns (loss, list of per-step lists)."""
    solver, fns, bc, st = oracle_case(setup, torch.float64)
    st = dict(st, u=u0, v=u0)
    nb = fns.allocate(st["r"].detach())
    lists = []
    side = torch.as_tensor(setup.box, dtype=torch.float64)
    for k in range(STEPS):
        st = dict(st)
        st["u"] = st["u"] + setup.dt * st["dudt"]
        st["v"] = st["u"] + 0.0 * st["dvdt"]
        st["r"] = oracle.space.periodic_shift(side, st["r"], setup.dt * st["v"])
        if frozen is None:
            nb = fns.update(st["r"].detach(), nb)
            idx = nb.idx
        else:
            idx = frozen[k]
        lists.append(idx)
        st = solver.forward(st, idx)
        st = bc(st)
    loss = adjoint.position_mse(st["r"], target, setup.box)
    return loss, lists


@pytest.fixture(scope="module")
def problem():
    a, b = setups()
    roll_b = adjoint.AdjointRollout(b, STEPS, K)
    target = roll_b.forward(b.state["u"].cuda()).double().cpu()
    return a, target


def test_adjoint_matches_float64_autograd(problem):
    a, target = problem
    roll = adjoint.AdjointRollout(a, STEPS, K)
    u0 = a.state["u"].cuda().clone().requires_grad_(True)
    r = adjoint.rollout(u0, roll)
    loss = adjoint.position_mse(r.double(), target.cuda(), a.box)
    (g,) = torch.autograd.grad(loss, u0)
    u64 = a.state["u"].double().clone().requires_grad_(True)
    loss64, _ = oracle_loss(a, u64, target)
    (g64,) = torch.autograd.grad(loss64, u64)
    rel = ((g.double().cpu() - g64).norm() / g64.norm()).item()
    assert abs(loss.item() - loss64.item()) <= 1e-5 * loss64.item()
    assert rel <= 1e-4, rel


def test_adjoint_matches_float64_finite_differences(problem):
    a, target = problem
    roll = adjoint.AdjointRollout(a, STEPS, K)
    u0 = a.state["u"].cuda().clone().requires_grad_(True)
    loss = adjoint.position_mse(adjoint.rollout(u0, roll).double(), target.cuda(), a.box)
    (g,) = torch.autograd.grad(loss, u0)
    g = g.double().cpu()
    u64 = a.state["u"].double()
    _, frozen = oracle_loss(a, u64, target)
    gen = torch.Generator().manual_seed(7)
    eps = 1e-6
    for _ in range(6):
        d = torch.randn(u64.shape, generator=gen, dtype=torch.float64)
        d /= d.norm()
        lp, _ = oracle_loss(a, u64 + eps * d, target, frozen)
        lm, _ = oracle_loss(a, u64 - eps * d, target, frozen)
        fd = (lp - lm).item() / (2 * eps)
        ad = (g * d).sum().item()
        assert abs(ad - fd) <= 1e-3 * max(abs(fd), 1e-12) + 1e-9 * g.norm().item(), (ad, fd)


def test_adjoint_checkpointing_is_exact(problem):
    """The reverse sweep recomputes segments forward; the gradient must not
    depend on the checkpoint interval."""
    a, target = problem
    grads = []
    for k in (1, 4, STEPS):
        roll = adjoint.AdjointRollout(a, STEPS, k)
        u0 = a.state["u"].cuda().clone().requires_grad_(True)
        loss = adjoint.position_mse(adjoint.rollout(u0, roll).double(), target.cuda(), a.box)
        (g,) = torch.autograd.grad(loss, u0)
        grads.append(g)
    assert torch.equal(grads[0], grads[1]) and torch.equal(grads[1], grads[2])


# ---------------------------------------------------------------- the full step
# The reference's own gradient check (notebooks/iclr24_grads.ipynb, cell 5):
# d/dr0 of 0.5 * sum(u_T^2) after a few si_euler steps, here against torch
# autograd through the float64 oracle rollout (frozen lists, like
# jax.grad(..., allow_int=True)): the transport-velocity TGV and the
# lid-driven cavity with the generalized wall BC and its moving lid. Bar:
# relative L2 error <= 1e-4, or within 10x the float32 oracle's own.

GRAD_STEPS = 5


def _gpu_state_after(setup, steps):
    """A float32 state a few steps in (lattice at rest is too symmetric)."""
    from jaxsph_gb300 import simulate

    sim = simulate.Simulation(setup)
    sim.run(steps)
    st = sim.state()[0]
    full = {k: v for k, v in setup.state.items()}
    full.update({k: st[k] for k in st})
    return {k: v.detach().clone().cuda() for k, v in full.items()}


def _oracle_grad(setup, state0, dtype=torch.float64):
    """Loss 0.5 sum(u_T^2) and its gradient w.r.t. the initial positions."""
    solver, fns, bc, st = oracle_case(setup, dtype, state=state0)
    r0 = st["r"].clone().requires_grad_(True)
    st = dict(st, r=r0)
    nb = fns.allocate(r0.detach())
    for _ in range(GRAD_STEPS):
        st, nb = oracle.sph.si_euler_advance(setup.dt, setup.tvf, st, nb, fns, solver, bc)
    loss = 0.5 * (st["u"] ** 2).sum()
    (g,) = torch.autograd.grad(loss, r0)
    return float(loss.detach()), g.double()


def _gpu_grad(setup, state0):
    roll = adjoint.AdjointRollout(setup, GRAD_STEPS, checkpoint_every=GRAD_STEPS)
    out = roll.run(state0)
    u = out["u"]
    loss = 0.5 * float((u.double() ** 2).sum())
    _, lr0 = roll.backward(torch.zeros_like(out["r"]), u.clone())
    return loss, lr0.double().cpu()


@pytest.mark.parametrize("name", ["tgv2d_tvf", "ldc_walls"])
def test_full_step_gradient_matches_float64_autograd(name):
    if name == "tgv2d_tvf":
        setup = cases.tgv(dim=2, dx=1.0 / 16, kernel="WC2K", tvf=1.0)
    else:  # the notebook's cavity: N = 20, viscosity 0.1
        setup = cases.lid_driven_cavity(dx=1.0 / 20, viscosity=0.1)
    state0 = _gpu_state_after(setup, 10)
    loss, g = _gpu_grad(setup, state0)
    host0 = {k: v.cpu() for k, v in state0.items()}
    loss64, g64 = _oracle_grad(setup, host0)
    _, g32 = _oracle_grad(setup, host0, torch.float32)
    rel = ((g - g64).norm() / g64.norm()).item()
    rel32 = ((g32 - g64).norm() / g64.norm()).item()
    print(f"{name}: loss {loss:.6e} vs {loss64:.6e}, gradient rel L2 {rel:.2e} "
          f"(float32 oracle {rel32:.2e})")
    assert abs(loss - loss64) <= 1e-5 * abs(loss64)
    # 1e-4, or as close as float32 arithmetic of the same algorithm gets
    assert rel <= max(1e-4, 10 * rel32), (rel, rel32)


# ---------------------------------------------------------------- snapshots
@pytest.mark.parametrize("canonical", [False, True])
def test_snapshot_restore_repeats_steps_bit_for_bit(canonical):
    """A device snapshot taken between two steps, restored after more steps,
    makes the following steps repeat the first run's bit for bit (candidate
    lists rebuilt in between included)."""
    from jaxsph_gb300 import simulate

    setup = cases.tgv_perturbed(n_side=24, seed=5)
    sim = simulate.Simulation(setup, canonical_order=canonical)
    sim.engine.snapshot_init(1)
    sim.run(3)
    sim.engine.snapshot_save(0)
    sim.run(12)
    first = sim.state()[0]
    sim.run(7)  # move on, rebuilding the candidate lists
    sim.engine.snapshot_restore(0)
    sim.run(12)
    again = sim.state()[0]
    for k in ("r", "u", "v", "dudt", "dvdt", "rho", "p"):
        assert torch.equal(first[k], again[k]), k


def test_snapshot_misuse_is_refused():
    """A snapshot is taken between two steps and restored only from a saved slot."""
    from jaxsph_gb300 import _lib, simulate

    setup = cases.tgv_perturbed(n_side=16, seed=6)
    sim = simulate.Simulation(setup)
    sim.engine.snapshot_init(2)
    with pytest.raises(_lib.SphError):
        sim.engine.snapshot_save(0)  # a freshly loaded state: no step taken yet
    with pytest.raises(_lib.SphError):
        sim.engine.snapshot_restore(1)  # nothing saved there
    sim.run(2)
    sim.engine.snapshot_save(1)
    with pytest.raises(_lib.SphError):
        sim.engine.snapshot_save(2)  # beyond the slots
    sim.engine.snapshot_restore(1)
    with pytest.raises(_lib.SphError):
        sim.engine.snapshot_init(1)  # once per handle
