"""GPU forward pass and si_euler steps vs the CPU oracle (float64 and float32).

Tolerances (GPU float32 vs the float64 oracle on identical float32 inputs):

* density:        |rho - rho64|          <= 2e-6 * rho_ref
* pressure:       |p - p64|              <= 2e-6 * rho_ref * c_ref^2
* accelerations:  |a - a64|_inf          <= 1e-5 * F,  F = p_ref/(rho_ref*h) + |g|
  (a pair's pressure term; lattice accelerations are residuals of cancelling
  pair terms, so their own magnitude is no scale)
* velocities:     |u - u64|_inf          <= 1e-5 * (u_ref + F*dt) after one step
* positions:      |r - r64|_inf          <= 1e-6 * box after the steps run here
and every error is also at most 10x the float32 oracle's own error (+ 1e-7 of
the scale), i.e. the GPU is as accurate as a float32 evaluation of the same
algorithm.
"""

import numpy as np
import pytest
import torch

from jaxsph_gb300 import cases, integrator, partition, simulate, solver
from oracle_setup import oracle_case, oracle_rollout
import oracle

pytestmark = pytest.mark.gpu


def small_cases():
    return {
        "tgv2d_sph": lambda: cases.tgv(dim=2, dx=0.02),
        "tgv3d_sph_tvf": lambda: cases.tgv(dim=3, dx=2 * np.pi / 20),
        # the other kernel in each dimension: quintic in 3D, Wendland C2 in 2D
        "tgv3d_qsk": lambda: cases.tgv(dim=3, dx=2 * np.pi / 16, kernel="QSK"),
        "tgv2d_wc2k_tvf": lambda: cases.tgv(dim=2, dx=0.02, kernel="WC2K", tvf=1.0),
        "tgv2d_rie": lambda: cases.tgv(dim=2, dx=0.04, solver_name="RIE"),
        "db_rie": lambda: cases.dam_break(dx=0.04),
        "db_rie_freeslip": lambda: cases.dam_break(dx=0.04, free_slip=True),
        "ldc_sph": lambda: cases.lid_driven_cavity(dx=0.04),
        "ldc_sph_tvf": lambda: cases.lid_driven_cavity(dx=0.04, tvf=1.0),
        "pf_sph": lambda: cases.poiseuille(dx=0.05),
        "pf_sph_evol": lambda: cases.poiseuille(dx=0.05, density_evolution=True),
        "ldc_sph_freeslip_av": lambda: cases.lid_driven_cavity(dx=0.04, free_slip=True,
                                                               artificial_alpha=0.1),
        # delta-SPH: the reference runs it with density summation (pf.yaml, cf.yaml)
        "tgv2d_delta": lambda: cases.tgv(dim=2, dx=0.02, solver_name="DELTA", diff_alpha=0.5),
        "pf_delta": lambda: cases.poiseuille(dx=0.05, solver_name="DELTA"),
        "ldc_delta_tvf": lambda: cases.lid_driven_cavity(dx=0.04, tvf=1.0,
                                                         solver_name="DELTA"),
        # delta-SPH density evolution (validation/db2d.sh's delta-SPH dam break)
        "pf_delta_evol": lambda: cases.poiseuille(dx=0.05, solver_name="DELTA",
                                                  density_evolution=True),
        "db_delta_evol": lambda: cases.dam_break(dx=0.04, solver_name="DELTA", gamma=7.0,
                                                 u_ref=1.95, viscosity=0.0, free_slip=True,
                                                 artificial_alpha=0.0),
        "tgv3d_delta_evol": lambda: cases.tgv(dim=3, dx=2 * np.pi / 16, solver_name="DELTA",
                                              density_evolution=True, diff_delta=0.5),
        # density renormalisation after each kind of density evolution
        "tgv2d_delta_evol_renorm": lambda: cases.tgv(dim=2, dx=0.02, solver_name="DELTA",
                                                     density_evolution=True, rho_renorm=True),
        "ldc_sph_evol_renorm": lambda: cases.lid_driven_cavity(dx=0.04, density_evolution=True,
                                                               rho_renorm=True),
        "db_rie_renorm": lambda: cases.dam_break(dx=0.04, rho_renorm=True),
        # heat conduction with the wall temperature BC (cases/ht.py)
        "ht_sph": lambda: cases.heat_transfer(dx=0.04),
        "ht_rie": lambda: cases.heat_transfer(dx=0.04, solver_name="RIE"),
        "ht_delta_evol": lambda: cases.heat_transfer(dx=0.04, solver_name="DELTA",
                                                     density_evolution=True),
        # moving lid with Riemann walls: normals recomputed every step
        "ldc_rie": lambda: cases.lid_driven_cavity(dx=0.04, solver_name="RIE"),
        "cw_sph_evol": lambda: cases.cube_of_water(),
        "rpf_sph": lambda: cases.reverse_poiseuille(dx=0.05),
        "rpf3d_sph": lambda: cases.reverse_poiseuille(dim=3, dx=0.1),
        "ut_sph_evol": lambda: cases.unit_cube(dx=0.04),
    }


def scales(setup):
    g = max(abs(x) for x in setup.g_ext_fn.spec["g"])
    F = setup.p_ref / (1.0 * setup.dx) + g
    return F


def err(a, b):
    a = a.detach().double().cpu()
    b = b.detach().double().cpu()
    return (a - b).abs().max().item()


def perturbed_state(setup, steps=3):
    """A non-trivial float32 state: a few float64 oracle steps, rounded to float32."""
    st = oracle_rollout(setup, steps, torch.float64)
    return {k: (v.float() if v.is_floating_point() else v.int()) for k, v in st.items()}


def gpu_solver(setup, kahan=False):
    return simulate.make_solver(setup, kahan=kahan)


@pytest.mark.parametrize("name", list(small_cases()))
def test_forward_matches_oracle(name):
    setup = small_cases()[name]()
    st32 = perturbed_state(setup)
    wc = gpu_solver(setup)
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
    F = scales(setup)
    prs = setup.c_ref ** 2
    checks = [("rho", 2e-6), ("p", 2e-6 * prs), ("dudt", 1e-5 * F), ("dvdt", 1e-5 * F),
              ("u", 1e-5), ("v", 1e-5), ("drhodt", 1e-5 * F)]
    if "T" in r64:
        dT = float(r64["dTdt"].detach().abs().max()) + 1.0
        checks += [("T", 1e-6), ("dTdt", 1e-5 * dT)]
    for key, tol in checks:
        e_gpu = err(out[key], r64[key])
        e_f32 = err(r32[key], r64[key])
        assert e_gpu <= max(tol, 10 * e_f32 + 1e-7 * tol * 1e5), (key, e_gpu, e_f32, tol)


@pytest.mark.parametrize("name", ["tgv2d_sph", "tgv3d_sph_tvf", "db_rie", "ldc_sph", "pf_sph",
                                  "db_delta_evol", "tgv2d_delta_evol_renorm", "ht_sph",
                                  "ldc_rie", "ldc_sph_freeslip_av"])
def test_rollout_matches_oracle(name):
    setup = small_cases()[name]()
    steps = 20
    sim = simulate.Simulation(setup)
    code = sim.run(steps)
    assert code & 0xF == 0
    got = sim.state()[0]
    ref = oracle_rollout(setup, steps, torch.float64)
    # the float32 oracle's own drift from float64 over the rollout bounds
    # what float32 rounding alone explains (a noisy initial state amplifies it)
    ref32 = oracle_rollout(setup, steps, torch.float32)
    box = float(np.max(setup.box))
    F = scales(setup)
    side = torch.as_tensor(setup.box, dtype=torch.float64)

    def drift(a):
        return oracle.space.periodic_displacement(side, a["r"].double().cpu() - ref["r"])

    assert drift(got).abs().max().item() <= max(1e-6 * box, 10 * drift(ref32).abs().max().item())
    assert err(got["rho"], ref["rho"]) <= max(2e-5, 10 * err(ref32["rho"], ref["rho"]))
    assert err(got["u"], ref["u"]) <= max(1e-4 * (setup.u_ref + F * setup.dt),
                                          10 * err(ref32["u"], ref["u"]))
    if "T" in ref:
        assert err(got["T"], ref["T"]) <= max(1e-5, 10 * err(ref32["T"], ref["T"]))
    if setup.nw_fn is not None:  # the recomputed normals of the moved walls
        assert err(got["nw"], ref["nw"]) <= max(1e-5, 10 * err(ref32["nw"], ref["nw"]))


def test_drop_in_advance_equals_resident_rollout():
    setup = cases.lid_driven_cavity(dx=0.04)
    wc = gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    disp, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    st = setup.to("cuda")
    nb = fns.allocate(st["r"])
    for _ in range(5):
        st, nb = adv(setup.dt, st, nb)
    # the same neighbour sets, pair sums possibly in another cell order
    # (the two paths rebuild their candidate lists at different steps)
    sim = simulate.Simulation(setup)
    sim.run(5)
    got = sim.state()[0]
    for k in ("r", "u", "v", "rho", "p", "dudt", "dvdt"):
        a, b = st[k].double(), got[k].double()
        scale = float(b.abs().max()) + 1e-30
        assert float((a - b).abs().max()) <= 1e-5 * scale, k


def test_drop_in_generic_callables_match_descriptors():
    """si_euler with a plain function of the positions as g_ext_fn (no GPU
    spec) composes the step like the reference (integrator.py:22-56) and
    matches the fused step with the descriptor, up to the summation order."""
    setup = cases.poiseuille(dx=0.05)  # body force on a band of y, walls (bc_fn)
    _, shift = setup.space()
    results = []
    for generic in (False, True):
        wc = gpu_solver(setup)
        if generic:
            desc = setup.g_ext_fn
            wc.g_ext_fn = lambda r: desc(r)  # a plain callable: no spec
        fns = simulate.make_neighbor_fns(setup, wc)
        adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
        st = setup.to("cuda")
        nb = fns.allocate(st["r"])
        for _ in range(5):
            st, nb = adv(setup.dt, st, nb)
        results.append(st)
    a, b = results
    assert float(a["dudt"][:, 0].abs().max()) > 0.0  # the body force acts
    for k in ("r", "u", "v", "rho", "p", "dudt", "dvdt"):
        x, y = a[k].double().cpu(), b[k].double().cpu()
        scale = float(x.abs().max()) + 1e-30
        assert float((x - y).abs().max()) <= 1e-5 * scale, k


def test_drop_in_advance_reports_overflow_lazily():
    from jaxsph_gb300.partition import NeighborList

    setup = cases.tgv(dim=2, dx=0.05)
    wc = gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    st = setup.to("cuda")
    nb = fns.allocate(st["r"])
    st1, nb1 = adv(setup.dt, st, nb)
    assert not nb1.did_buffer_overflow
    # a list whose edge capacity is far too small overflows on the next step
    small = NeighborList(fns, nb1.reference_position, 0, nb1.cell_list_capacity, 10)
    st2, nb2 = adv(setup.dt, st1, small)
    assert nb2.did_buffer_overflow
    # the state itself does not depend on the capacity (a fresh solver: the
    # same call sequence, so the same pair order)
    wc2 = gpu_solver(setup)
    adv2 = integrator.si_euler(setup.tvf, wc2.forward_wrapper(), shift, setup.bc_fn, None)
    s1, n1 = adv2(setup.dt, st, fns.allocate(st["r"]))
    st3, _ = adv2(setup.dt, s1, n1)
    for k in ("r", "u", "rho", "dudt"):
        assert torch.equal(st2[k], st3[k]), k


def test_drop_in_advance_keeps_reference_position_within_threshold():
    from jaxsph_gb300.partition import NeighborListFns, Sparse

    setup = cases.tgv(dim=2, dx=0.05)
    wc = gpu_solver(setup)
    cut = wc._kernel_fn.cutoff
    # a skin as in the reference's dr_threshold: rebuild only past half of it
    fns = NeighborListFns(setup.box, cut, 0.5 * cut, 1.25, False, Sparse)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    st = setup.to("cuda")
    nb = fns.allocate(st["r"])
    st1, nb1 = adv(setup.dt, st, nb)
    assert torch.equal(nb1.reference_position, nb.reference_position)
    fns0 = simulate.make_neighbor_fns(setup, wc)
    st_b, _ = adv(setup.dt, st, fns0.allocate(st["r"]))
    # pairs beyond the kernel support add nothing (W = 0 there): the same
    # state up to the summation order of another binning
    for k in ("r", "u", "rho"):
        assert torch.allclose(st1[k], st_b[k], rtol=1e-6, atol=1e-6), k


def test_deterministic_and_graph_equals_eager():
    setup = cases.tgv(dim=3, dx=2 * np.pi / 20)
    a = simulate.Simulation(setup)
    a.run(9)  # eager + graph replays
    b = simulate.Simulation(setup)
    for _ in range(9):
        b.run(1)  # eager only
    sa, sb = a.state()[0], b.state()[0]
    for k in ("r", "u", "v", "rho", "p", "dudt", "dvdt"):
        assert torch.equal(sa[k], sb[k]), k


def test_forward_rejects_stale_neighbour_list():
    setup = cases.tgv(dim=2, dx=0.05)
    wc = gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    st = setup.to("cuda")
    nb = fns.allocate(st["r"])
    st2 = dict(st)
    st2["r"] = (st["r"] + 1e-3).contiguous()
    with pytest.raises(NotImplementedError):
        wc.forward_wrapper()(st2, nb)


def test_diagnostics_float64():
    setup = cases.dam_break(dx=0.04)
    sim = simulate.Simulation(setup)
    sim.run(10)
    st = sim.state()[0]
    d = sim.diagnostics()[0].cpu()
    fluid = st["tag"] == 0
    m = st["mass"].double()[fluid]
    u = st["u"].double()[fluid]
    v = st["v"].double()[fluid]
    assert abs(d[0].item() - m.sum().item()) <= 1e-12 * m.sum().item()
    mom = (m[:, None] * u).sum(0)
    assert torch.allclose(d[1:3], mom.cpu(), rtol=1e-9, atol=1e-12)
    ekin = 0.5 * (v ** 2).sum().item() * setup.dx ** 2
    assert abs(d[4].item() - ekin) <= 1e-6 * max(ekin, 1e-30) + 1e-15
    umax = st["u"].double().norm(dim=1).max().item()
    assert abs(d[5].item() - umax) <= 1e-7 * max(umax, 1e-30)


def test_drop_in_advance_on_pinned_host_state():
    # a pinned host state goes to the GPU and back inside the call: the
    # same result as on device tensors, bit for bit (each path its own
    # solver, so each engine sees its own call sequence)
    setup = cases.tgv(dim=3, dx=2 * np.pi / 12)
    wc, wcd = gpu_solver(setup), gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    advd = integrator.si_euler(setup.tvf, wcd.forward_wrapper(), shift, setup.bc_fn, None)
    keys = ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "mass", "eta", "nw")
    host = {k: setup.state[k].to(torch.int32 if k == "tag" else torch.float32)
            .contiguous().pin_memory() for k in keys}
    dev = {k: v.cuda() for k, v in host.items()}
    hs, hn = host, fns.allocate(host["r"])
    ds, dn = dev, fns.allocate(dev["r"])
    for _ in range(4):
        hs, hn = adv(setup.dt, hs, hn)
        ds, dn = advd(setup.dt, ds, dn)
    for k in ("r", "u", "v", "rho", "p", "dudt", "dvdt"):
        assert hs[k].device.type == "cpu" and hs[k].is_pinned(), k
        assert torch.equal(hs[k], ds[k].cpu()), k
    assert not hn.did_buffer_overflow


def test_summation_carries_drhodt_over():
    # density summation leaves drho/dt as the state had it (solver.py:794-796):
    # the forward pass, the drop-in step on device tensors and on pinned host
    # tensors all return the input's values
    setup = cases.tgv(dim=2, dx=0.05)
    g = torch.Generator().manual_seed(5)
    drhodt = torch.randn(setup.n, generator=g)
    keys = ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "mass", "eta", "nw")
    base = {k: setup.state[k].to(torch.int32 if k == "tag" else torch.float32).contiguous()
            for k in keys}
    base["drhodt"] = drhodt
    wc = gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    dev = {k: v.cuda() for k, v in base.items()}
    out = wc.forward_wrapper()(dev, fns.allocate(dev["r"]))
    assert torch.equal(out["drhodt"].cpu(), drhodt)
    _, shift = setup.space()
    for place in ("cuda", "pinned"):
        st = ({k: v.cuda() for k, v in base.items()} if place == "cuda"
              else {k: v.pin_memory() for k, v in base.items()})
        wc = gpu_solver(setup)
        adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
        nb = fns.allocate(st["r"])
        for _ in range(3):
            st, nb = adv(setup.dt, st, nb)
        assert torch.equal(st["drhodt"].cpu(), drhodt), place


def test_drop_in_heat_transfer_matches_the_resident_rollout():
    # the temperature fields go in and out of the drop-in step (pinned host
    # memory) like the others; T and dT/dt match the resident run
    setup = cases.heat_transfer(dx=0.04)
    wc = gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    st = {k: v.to(torch.int32 if k == "tag" else torch.float32).contiguous().pin_memory()
          for k, v in setup.state.items()}
    nb = fns.allocate(st["r"])
    for _ in range(5):
        st, nb = adv(setup.dt, st, nb)
    assert st["T"].is_pinned() and st["dTdt"].is_pinned()
    sim = simulate.Simulation(setup)
    sim.run(5)
    got = sim.state()[0]
    for k in ("r", "u", "rho", "T", "dTdt"):
        a, b = st[k].double(), got[k].double().cpu()
        assert float((a - b).abs().max()) <= 1e-5 * (float(b.abs().max()) + 1e-30), k


def test_drop_in_moving_wall_normals():
    # si_euler with the case's nw_fn: the drop-in step returns the recomputed
    # normals, and they follow the resident rollout
    setup = cases.lid_driven_cavity(dx=0.04, solver_name="RIE")
    wc = gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, setup.nw_fn)
    st = setup.to("cuda")
    nb = fns.allocate(st["r"])
    for _ in range(5):
        st, nb = adv(setup.dt, st, nb)
    want = setup.nw_fn(st["r"])
    assert float((st["nw"] - want).abs().max()) < 1e-5
    sim = simulate.Simulation(setup)
    sim.run(5)
    got = sim.state()[0]
    for k in ("r", "u", "nw"):
        a, b = st[k].double(), got[k].double()
        assert float((a - b).abs().max()) <= 1e-5 * (float(b.abs().max()) + 1e-30), k
    # a plain function as nw_fn (no GPU spec): the step is composed like the
    # reference's and returns the same normals
    nw_plain = setup.nw_fn.__call__
    adv2 = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, nw_plain)
    st2 = setup.to("cuda")
    nb2 = fns.allocate(st2["r"])
    for _ in range(5):
        st2, nb2 = adv2(setup.dt, st2, nb2)
    for k in ("r", "u", "nw"):
        a, b = st2[k].double().cpu(), st[k].double().cpu()
        assert float((a - b).abs().max()) <= 1e-5 * (float(b.abs().max()) + 1e-30), k


def test_drop_in_advance_rejects_pageable_host_arrays():
    setup = cases.tgv(dim=2, dx=0.05)
    wc = gpu_solver(setup)
    e = wc.engine(simulate.make_neighbor_fns(setup, wc), wc.sph_case(
        simulate.make_neighbor_fns(setup, wc), setup.n))
    keys = ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "mass", "eta", "nw")
    st = {k: setup.state[k].to(torch.int32 if k == "tag" else torch.float32).contiguous()
          for k in keys}
    out = {k: torch.empty_like(st[k]) for k in ("r", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p")}
    with pytest.raises(Exception, match="pinned"):
        e.advance(st, out)  # refused by the library, before any launch
    # the drop-in advance then falls back to device copies
    fns = simulate.make_neighbor_fns(setup, wc)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    res, _ = adv(setup.dt, st, fns.allocate(st["r"].cuda()))
    assert res["r"].is_cuda
    # the raw call, as a C caller makes it
    from jaxsph_gb300 import _lib
    import ctypes
    vin, vout = _lib.SphStateView(), _lib.SphStateView()
    vin.n = vout.n = setup.n
    for k in keys:
        setattr(vin, k, st[k].data_ptr())
    for k in out:
        setattr(vout, k, out[k].data_ptr())
    status = torch.zeros((), dtype=torch.int32, device="cuda")
    rc = e.lib.sph_advance(e.h, ctypes.byref(vin), ctypes.byref(vout), None, 0.0,
                           status.data_ptr(), None)
    assert rc & _lib.ERR_INVALID_ARG
    assert b"pinned" in e.lib.sph_last_error()


def test_drop_in_advance_with_a_foreign_state():
    # a state that is not the engine's last result (positions differ from
    # the ones it holds) makes the step rebuild: the result equals a fresh
    # engine's, bit for bit (the sort is stable by original index)
    setup = cases.tgv(dim=3, dx=2 * np.pi / 12)
    wc, wc2 = gpu_solver(setup), gpu_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    adv2 = integrator.si_euler(setup.tvf, wc2.forward_wrapper(), shift, setup.bc_fn, None)
    st = setup.to("cuda")
    nb = fns.allocate(st["r"])
    s = st
    for _ in range(3):
        s, nb = adv(setup.dt, s, nb)
    got, _ = adv(setup.dt, st, fns.allocate(st["r"]))  # back to the initial state
    want, _ = adv2(setup.dt, st, fns.allocate(st["r"]))
    for k in ("r", "u", "v", "rho", "p", "dudt", "dvdt"):
        assert torch.equal(got[k], want[k]), k
