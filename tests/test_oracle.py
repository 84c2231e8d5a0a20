"""The CPU oracle pinned against the reference's own tests (no GPU needed).

* neighbour lists: the four golden edge lists of the reference's
  tests/test_neighbors.py:89-121, in float64 (the reference test enables x64)
  and float32, allocate == update, no one-sided padding, self-edge rules;
* kernels: tests/test_kernel.py:17-44 (1D half-integral 0.5, W >= 0, W' <= 0)
  plus 2D/3D normalisation;
* the product's closed-form kernel derivatives against the oracle's autograd.
"""

import json
import math
import os

import numpy as np
import pytest
import torch

import oracle
from jaxsph_gb300 import kernel as pk

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "neighbors_golden.json")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("case", range(4))
def test_golden_neighbor_lists(case, dtype):
    c = json.load(open(GOLDEN))["cases"][case]
    r = torch.tensor(c["r"], dtype=dtype)
    n = r.shape[0]
    fns = oracle.partition.NeighborListFns(c["box_size"], c["cutoff"], dtype,
                                           mask_self=c["mask_self"])
    nb = fns.allocate(r)
    nb2 = fns._build(r, nb.cell_list_capacity, nb.max_occupancy, 0)
    assert not nb.did_buffer_overflow and not nb2.did_buffer_overflow
    assert torch.equal(nb.idx, nb2.idx)
    assert torch.equal(nb.idx[0] == n, nb.idx[1] == n)
    real = nb.idx[:, nb.idx[0] < n]
    selfe = real[0] == real[1]
    if c["mask_self"]:
        assert int(selfe.sum()) == 0
    else:
        assert len(torch.unique(real[0][selfe])) == n
    assert oracle.partition.canonical_edges(nb.idx, n).tolist() == c["target"]


def test_golden_fixture_is_the_reference_data():
    d = json.load(open(GOLDEN))
    assert len(d["cases"]) == 4
    assert [c["mask_self"] for c in d["cases"]] == [False, True, False, True]


@pytest.mark.parametrize("name,dx_factor", [("QSK", 1.0), ("WC2K", 1.3)])
def test_kernel_1d_half_integral(name, dx_factor):
    """tests/test_kernel.py:17-44 of the reference."""
    N = 500
    for h in (1.0, 0.1, 0.01):
        k = oracle.sph.make_kernel(name, dx_factor * h, 1)
        dx = k.cutoff / N
        x = torch.linspace(dx / 2, k.cutoff + dx / 2, N, dtype=torch.float64)
        w = k.w(x)
        gw = oracle.sph.grad_w(k, x).detach()
        assert abs(dx * w.sum().item() - 0.5) < 1e-2
        assert (w >= 0).all() and (gw <= 0).all()


@pytest.mark.parametrize("name", ["QSK", "WC2K"])
@pytest.mark.parametrize("dim", [2, 3])
def test_kernel_normalisation(name, dim):
    k = oracle.sph.make_kernel(name, 1.0, dim)
    r = torch.linspace(0, k.cutoff, 200001, dtype=torch.float64)
    w = k.w(r)
    shell = 2 * math.pi * r if dim == 2 else 4 * math.pi * r ** 2
    integral = torch.trapezoid(w * shell, r).item()
    if name == "QSK" and dim == 3:
        # the reference's 3D quintic constant 3/(359 pi) (kernel.py:64) is 0.28 %
        # above the exact 1/(120 pi); parity keeps the reference's value
        assert abs(integral - 360.0 / 359.0) < 1e-6
    else:
        assert abs(integral - 1.0) < 1e-6


@pytest.mark.parametrize("name", ["QSK", "WC2K"])
@pytest.mark.parametrize("dim", [2, 3])
def test_product_kernel_formulas_match_oracle_autograd(name, dim):
    h = 0.037
    k_o = oracle.sph.make_kernel(name, h, dim)
    k_p = pk.make_kernel(name, h, dim)
    assert k_p.cutoff == pytest.approx(k_o.cutoff)
    r = torch.linspace(0, 1.1 * k_o.cutoff, 5001, dtype=torch.float64)
    assert torch.allclose(k_p.w(r), k_o.w(r), rtol=1e-12, atol=1e-12 * k_o.sigma)
    g_o = oracle.sph.grad_w(k_o, r).detach()
    assert torch.allclose(k_p.grad_w(r), g_o, rtol=1e-10, atol=1e-10 * k_o.sigma / h)


def test_jnp_mod_semantics():
    side = torch.tensor(1.0, dtype=torch.float32)
    x = torch.tensor([-1.5, -0.25, -0.0, 0.0, 0.25, 1.0, 1.75], dtype=torch.float32)
    got = oracle.space.jnp_mod(x, side)
    want = torch.tensor([0.5, 0.75, -0.0, 0.0, 0.25, 0.0, 0.75], dtype=torch.float32)
    assert torch.equal(got, want)
    # a value just below zero wraps to exactly the box length in float32
    tiny = torch.tensor([-1e-9], dtype=torch.float32)
    assert oracle.space.jnp_mod(tiny, side).item() == 1.0


@pytest.mark.parametrize("solver_name", ["SPH", "DELTA"])
def test_oracle_step_conserves_mass_and_momentum(solver_name):
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case

    setup = cases.tgv(dim=2, dx=0.05, solver_name=solver_name, diff_alpha=0.5)
    solver, fns, bc, st = oracle_case(setup, torch.float64)
    nb = fns.allocate(st["r"])
    for _ in range(3):
        st, nb = oracle.sph.si_euler_advance(setup.dt, 0.0, st, nb, fns, solver, bc)
    # pairwise antisymmetric forces: total momentum change vanishes
    mom_rate = (st["mass"][:, None] * st["dudt"]).sum(0)
    assert mom_rate.abs().max().item() < 1e-9 * setup.p_ref
    # density summation of a uniform lattice with periodic images is uniform
    assert (st["rho"] - st["rho"].mean()).abs().max().item() < 1e-2


def test_oracle_delta_diffusion_term():
    """The delta-SPH term vanishes with alpha = 0 and damps relative motion."""
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case

    def dudt(name, alpha):
        setup = cases.tgv(dim=2, dx=0.05, solver_name=name, diff_alpha=alpha)
        solver, fns, bc, st = oracle_case(setup, torch.float64)
        out = solver.forward(st, fns.allocate(st["r"]).idx)
        return out["dudt"], st

    base, st = dudt("SPH", 0.0)
    assert torch.equal(dudt("DELTA", 0.0)[0], base)
    diff = dudt("DELTA", 0.5)[0] - base
    # a viscous-like term: its power on the velocity field is dissipative
    assert (st["mass"][:, None] * st["u"] * diff).sum().item() < 0.0


def _delta_evol_rates(perturb, u_zero):
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case

    out = {}
    for name in ("SPH", "DELTA"):
        setup = cases.tgv(dim=2, dx=0.05, solver_name=name, density_evolution=True)
        solver, fns, bc, st = oracle_case(setup, torch.float64)
        st["rho"] = st["rho"] * (1 + perturb * torch.sin(2 * math.pi * st["r"][:, 0]))
        if u_zero:
            st["u"] = torch.zeros_like(st["u"])
        out[name] = solver.forward(st, fns.allocate(st["r"]).idx)["drhodt"], st
    return out


def test_oracle_delta_density_evolution():
    """rho_evol_fn_delta: with a uniform density only the continuity term
    remains (that of rho_evol_fn); with the fluid at rest the diffusion of a
    density wave reduces it."""
    r = _delta_evol_rates(0.0, False)
    assert torch.allclose(r["DELTA"][0], r["SPH"][0], rtol=0, atol=1e-12)
    r = _delta_evol_rates(1e-3, True)
    drhodt, st = r["DELTA"]
    assert r["SPH"][0].abs().max().item() == 0.0
    dev = st["rho"] - st["rho"].mean()
    assert (drhodt * dev).sum().item() < 0.0


def test_oracle_heat_conduction_conserves_energy():
    """Cleary's pair term is antisymmetric: on a periodic box without walls
    sum_i m_i Cp_i dT/dt_i vanishes, and heat flows from hot to cold."""
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case

    setup = cases.tgv(dim=2, dx=0.05, heat_conduction=True, kappa_ref=1.0, Cp_ref=2.0)
    solver, fns, _, st = oracle_case(setup, torch.float64)
    st["T"] = 1 + 0.1 * torch.sin(2 * math.pi * st["r"][:, 0])
    out = solver.forward(st, fns.allocate(st["r"]).idx)
    rate = out["dTdt"]
    assert abs(float((st["mass"] * st["Cp"] * rate).sum())) < 1e-12 * float(rate.abs().max())
    assert float((rate * (st["T"] - st["T"].mean())).sum()) < 0.0


def test_heat_conduction_decays_a_temperature_wave_at_the_analytic_rate():
    """Physics pin of Cleary's temperature equation (solver.py:591-610,
    :832-850): on a periodic lattice at rest a wave T = 1 + a sin(2 pi x)
    decays as exp(-kappa k^2 t / (rho Cp)), k = 2 pi (the reference's Poiseuille
    and Couette tests pin the momentum terms the same way). 400 steps, within
    1 % of the analytic decay."""
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case

    kappa, cp = 0.07, 1.0
    setup = cases.tgv(dim=2, dx=0.02, heat_conduction=True, kappa_ref=kappa, Cp_ref=cp)
    setup.state["u"] = torch.zeros_like(setup.state["u"])
    setup.state["v"] = torch.zeros_like(setup.state["v"])
    solver, fns, bc, st = oracle_case(setup, torch.float64)
    x = st["r"][:, 0]
    wave = torch.sin(2 * math.pi * x)
    st["T"] = 1.0 + 0.1 * wave

    def amplitude(T):
        return 2 * ((T - 1.0) * wave).mean().item()

    a0, steps = amplitude(st["T"]), 400
    nb = fns.allocate(st["r"])
    with torch.no_grad():
        for _ in range(steps):
            st, nb = oracle.sph.si_euler_advance(setup.dt, setup.tvf, st, nb, fns, solver, bc)
    alpha = kappa / (st["rho"].mean().item() * cp)
    want = math.exp(-alpha * (2 * math.pi) ** 2 * steps * setup.dt)
    assert abs(amplitude(st["T"]) / a0 - want) < 0.01 * want


def test_2d_tgv_decays_at_the_viscous_rate():
    """Physics pin of the viscous term on the reference's 2D TGV validation
    (validation/validate.py:181-195): u_max and the kinetic energy decay as
    exp(-8 pi^2 t / Re) and its square. From the unrelaxed lattice the
    analytic decay holds until the lattice disorders (about t = 0.1 at dx =
    0.02; the reference validates from a relaxed state for that reason), so
    the pin covers the first 200 steps: u_max within 0.5 % there (measured
    0.14 %), the kinetic energy within 1.5 % (measured 0.9 %: plain SPH's own
    dissipation). A viscosity 15 % high or low misses the u_max bound (by
    0.9 % and 1.2 %; the energy by 2.9 % and 1.2 %)."""
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case

    setup = cases.tgv(dim=2, dx=0.02)
    solver, fns, bc, st = oracle_case(setup, torch.float64)

    def measures(st):
        speed = st["u"].norm(dim=1)
        return speed.max().item(), (0.5 * st["mass"] * speed ** 2).sum().item()

    (u0, e0), steps = measures(st), 200
    nb = fns.allocate(st["r"])
    with torch.no_grad():
        for _ in range(steps):
            st, nb = oracle.sph.si_euler_advance(setup.dt, setup.tvf, st, nb, fns, solver, bc)
    u, e = measures(st)
    decay = math.exp(-8 * math.pi ** 2 * steps * setup.dt * setup.viscosity)
    assert abs(u / u0 - decay) < 5e-3 * decay
    assert abs(e / e0 - decay ** 2) < 1.5e-2 * decay ** 2


def test_heat_transfer_bc_matches_the_oracle():
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_bc

    setup = cases.heat_transfer(dx=0.04)
    g = torch.Generator().manual_seed(0)
    st = {k: v.clone() for k, v in setup.state.items()}
    for k in ("u", "v", "dudt", "dvdt", "T", "dTdt"):
        st[k] = torch.randn(st[k].shape, generator=g)
    st["r"][:, 0] = torch.rand(setup.n, generator=g)
    want = oracle_bc(setup)({k: v.double() if v.is_floating_point() else v
                             for k, v in st.items()})
    got = setup.bc_fn(st)
    for k in ("u", "v", "dudt", "dvdt", "T", "dTdt"):
        assert torch.equal(got[k], want[k].float()), k  # the values set are float32 here
    assert (got["T"][st["tag"] == 3] == 1.23).all()


def test_moving_wall_normals_match_the_oracle():
    """The nw_fn of a moving-lid case (compute_nws_jax_wrapper): the case's
    torch restatement equals the oracle's, and both equal the scipy normals
    of the initial state except where the nearest layer point is point 0
    (which the reference's recomputation never takes: its corner block)."""
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_nw_fn

    setup = cases.lid_driven_cavity(dx=0.04, solver_name="RIE")
    assert setup.nw_fn is not None
    r = setup.state["r"]
    got = setup.nw_fn(r)
    want = oracle_nw_fn(setup)(r.double())
    # float32 normals carry eps |r| / |dr| of rounding (|r| ~ 1, |dr| >= dx / 10)
    assert (got.double() - want).abs().max().item() < 1e-4
    moved = torch.remainder(r + torch.tensor([0.013, 0.0]), torch.as_tensor(setup.box).float())
    assert (setup.nw_fn(moved).double() - oracle_nw_fn(setup)(moved.double())).abs().max() < 1e-4
    # against scipy on the initial positions
    layer = setup.nw_fn.spec["layer"].astype(np.float64)
    wall = setup.nw_fn.wall
    p = r.double().numpy()[wall] - np.asarray(setup.nw_fn.spec["offset"][:2])
    d = np.linalg.norm(layer[None, :, :] - p[:, None, :], axis=-1)
    nearest0 = np.argmin(d, axis=1) == 0
    diff = (got - setup.state["nw"]).abs().max(1).values.numpy()[wall]
    assert (diff[~nearest0] < 1e-5).all() and nearest0.any()
    assert setup.state["nw"][~torch.as_tensor(wall)].abs().max() == 0
    # no moving walls or no normals needed: no recomputation
    assert cases.lid_driven_cavity(dx=0.04).nw_fn is None
    assert cases.poiseuille(dx=0.05, solver_name="RIE").nw_fn is None


def test_oracle_gradient_through_steps():
    """torch autograd through the float64 oracle (the gradient oracle of the adjoint)."""
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case

    setup = cases.tgv(dim=2, dx=0.1)
    solver, fns, bc, st = oracle_case(setup, torch.float64)
    nb = fns.allocate(st["r"])
    u0 = st["u"].clone().requires_grad_(True)
    s = dict(st, u=u0, v=u0)
    for _ in range(2):
        s, _ = oracle.sph.si_euler_advance(setup.dt, 0.0, s, nb, fns, solver, bc)
    loss = (0.5 * s["u"] ** 2).sum()
    (g,) = torch.autograd.grad(loss, u0)
    assert torch.isfinite(g).all() and g.abs().max() > 0
