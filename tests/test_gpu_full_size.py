"""Parity at the measured sizes: the 3D Taylor-Green vortex on the 64^3 lattice
(262,144 particles, the benchmark workload) and the dam break at dx = 0.005
(80,000 fluid + 8,874 wall particles).

The 64^3 lattice puts 6 senders of every particle exactly on the cutoff
sphere (cutoff 2h = 2 dx, jax_sph/kernel.py:82-83); membership there is the
reference's float32 test ``metric < cutoff**2``
(jax_sph/jax_md/partition.py:897). In the dam break the reference's cell is
the cutoff to within float32 rounding along y (2.13 / 142 = 0.015), so senders
at the cutoff distance sit at the edge of the reference's 3^d candidate cells.
Bars (float32 GPU vs the oracle on the same float32 inputs):

* neighbour sets: bit-exact -- the drop-in edge list (canonical sort) and the
  per-particle sizes of the sets the forward passes summed over equal the
  float32 oracle's, on the lattice and after steps;
* one forward pass: the tolerances of tests/test_gpu_physics.py (density
  2e-6 rho_ref, pressure 2e-6 rho_ref c^2, accelerations 1e-5 F with F =
  p_ref / (rho_ref h) + |g|, or within 10x the float32 oracle's own error);
* a 10-step rollout: positions 1e-6 of the box, density 2e-5, velocity
  1e-4 (u_ref + F dt), or within 10x the float32 oracle's own drift.
"""

import numpy as np
import pytest
import torch

import oracle
from jaxsph_gb300 import cases, partition, simulate, space
from oracle_setup import oracle_case, oracle_rollout

pytestmark = pytest.mark.gpu


def _err(a, b):
    return (a.detach().double().cpu() - b.detach().double().cpu()).abs().max().item()


def _scale_F(setup):
    g = max(abs(x) for x in setup.g_ext_fn.spec["g"])
    return setup.p_ref / setup.dx + g


def _cutoff(setup):
    from jaxsph_gb300.kernel import make_kernel

    return make_kernel(setup.solver["kernel"], setup.dx, setup.dim).cutoff


def _oracle_list(setup, r):
    fns = oracle.partition.NeighborListFns(setup.box, _cutoff(setup), torch.float32,
                                           mask_self=False)
    return fns.allocate(torch.as_tensor(r, dtype=torch.float32).cpu())


def _receiver_counts(idx, n):
    """Edges per receiver (row 0 of the reference's NeighborList.idx)."""
    rows = idx[0].long().cpu()
    return torch.bincount(rows[rows < n], minlength=n)


def _check_sets(setup, r_dev):
    """Drop-in edge list at r vs the float32 oracle: bit-exact sets."""
    n = setup.n
    disp, _ = space.periodic(setup.box)
    fns = partition.neighbor_list(disp, setup.box, _cutoff(setup), mask_self=False)
    nb = fns.allocate(r_dev)
    ref = _oracle_list(setup, r_dev)
    assert nb.occupancy == ref.occupancy
    assert nb.max_occupancy == ref.max_occupancy
    assert nb.cell_list_capacity == ref.cell_list_capacity
    got = oracle.partition.canonical_edges(nb.idx.long().cpu(), n)
    want = oracle.partition.canonical_edges(ref.idx, n)
    assert torch.equal(got, want)
    return ref


@pytest.fixture(scope="module")
def tgv64():
    return cases.tgv(dim=3, dx=2 * np.pi / 64)


def test_tgv3d_64_lattice_sets_bit_exact(tgv64):
    setup = tgv64
    r = setup.state["r"].cuda()
    ref = _check_sets(setup, r)
    counts = _receiver_counts(ref.idx, setup.n)
    # the lattice's own structure: 27 points closer than 2 dx (self included)
    # plus those of the 6 exact ties whose float32 metric falls below cutoff^2
    assert int(counts.min()) == 27 and int(counts.max()) == 33
    # the per-step sets of the forward passes (the resident engine's)
    sim = simulate.Simulation(setup)
    sim.engine.forward()
    got = sim.engine.neighbour_counts("cuda").cpu().long()
    assert torch.equal(got, counts)


def test_tgv3d_64_sets_after_steps(tgv64):
    setup = tgv64
    sim = simulate.Simulation(setup)
    sim.run(5)
    st = sim.state()[0]
    got = sim.engine.neighbour_counts("cuda").cpu().long()
    ref = _check_sets(setup, st["r"].cuda().contiguous())
    assert torch.equal(got, _receiver_counts(ref.idx, setup.n))


def _forward_parity(setup, st32):
    """One GPU forward pass vs the float64 and float32 oracle on float32 inputs."""
    wc = simulate.make_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    dev = {k: v.cuda() for k, v in st32.items()}
    nb = fns.allocate(dev["r"])
    out = wc.forward_wrapper()(dev, nb)
    res = {}
    for dt_ in (torch.float64, torch.float32):
        sol, ofns, _, ost = oracle_case(setup, dt_, state=st32)
        onb = ofns.allocate(ost["r"])
        res[dt_] = sol.forward(ost, onb.idx)
    r64, r32 = res[torch.float64], res[torch.float32]
    F = _scale_F(setup)
    prs = setup.c_ref ** 2
    for key, tol in (("rho", 2e-6), ("p", 2e-6 * prs), ("dudt", 1e-5 * F), ("dvdt", 1e-5 * F),
                     ("drhodt", 1e-5 * F)):
        e_gpu = _err(out[key], r64[key])
        e_f32 = _err(r32[key], r64[key])
        assert e_gpu <= max(tol, 10 * e_f32 + 1e-2 * tol), (key, e_gpu, e_f32, tol)


def test_tgv3d_64_forward_matches_float64(tgv64):
    setup = tgv64
    # a non-trivial float32 state: the GPU's own state after a few steps
    sim = simulate.Simulation(setup)
    sim.run(4)
    st = {k: v.cpu() for k, v in sim.state()[0].items()}
    _forward_parity(setup, st)


def test_tgv3d_64_rollout_matches_float64(tgv64):
    setup = tgv64
    steps = 10
    sim = simulate.Simulation(setup)
    assert sim.run(steps) & 0xC == 0
    got = sim.state()[0]
    ref = oracle_rollout(setup, steps, torch.float64)
    ref32 = oracle_rollout(setup, steps, torch.float32)
    side = torch.as_tensor(setup.box, dtype=torch.float64)

    def drift(a):
        return oracle.space.periodic_displacement(
            side, a["r"].double().cpu() - ref["r"]).abs().max().item()

    F = _scale_F(setup)
    box = float(np.max(setup.box))
    assert drift(got) <= max(1e-6 * box, 10 * drift(ref32))
    assert _err(got["rho"], ref["rho"]) <= max(2e-5, 10 * _err(ref32["rho"], ref["rho"]))
    assert _err(got["u"], ref["u"]) <= max(1e-4 * (setup.u_ref + F * setup.dt),
                                           10 * _err(ref32["u"], ref["u"]))


@pytest.fixture(scope="module")
def db005():
    return cases.dam_break(dx=0.005)


def test_dam_break_dx0005_sets_bit_exact(db005):
    setup = db005
    assert setup.n == 88_874
    _check_sets(setup, setup.state["r"].cuda())


def test_dam_break_dx0005_forward_matches_float64(db005):
    setup = db005
    # a float32 state two float64 oracle steps in (the column starts to fall)
    st = oracle_rollout(setup, 2, torch.float64)
    st32 = {k: (v.float() if v.is_floating_point() else v.int()) for k, v in st.items()}
    _check_sets(setup, st32["r"].cuda())
    _forward_parity(setup, st32)
