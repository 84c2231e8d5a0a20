"""Host-side case construction against the reference's setup code (no GPU)."""

import numpy as np
import pytest
import torch

import oracle
from jaxsph_gb300 import _lib, cases, partition
from oracle_setup import oracle_bc, oracle_g


def test_tgv2d_lattice_layout():
    s = cases.tgv(dim=2)
    r = s.state["r"]
    assert s.n == 2500 and r.dtype == torch.float32
    # x fastest (meshgrid indexing="xy"), cell centres (i + 1/2) dx rounded in float32
    assert r[1, 0] > r[0, 0] and r[1, 1] == r[0, 1]
    assert r[0, 0].item() == np.float32(np.float32(0.5) * np.float32(0.02))
    assert s.dt == pytest.approx(0.25 * 0.02 / 11)
    assert s.p_ref == 100.0 and s.p_bg == 0.0


def test_tgv3d_lattice_layout():
    s = cases.tgv(dim=3)
    r = s.state["r"]
    assert s.n == 64 ** 3
    # meshgrid(range(nx), range(ny), range(nz), indexing="xy"): z fastest, then x, then y
    assert r[1, 2] > r[0, 2] and r[1, 0] == r[0, 0] and r[1, 1] == r[0, 1]
    assert r[64, 0] > r[0, 0] and r[64, 1] == r[0, 1]
    assert r[64 * 64, 1] > r[0, 1]
    assert s.solver["kernel"] == "WC2K" and s.tvf == 1.0
    assert s.viscosity == pytest.approx(1 / 1600)


def test_dam_break_geometry():
    s = cases.dam_break()
    tag = s.state["tag"]
    assert s.n == 88874 and int((tag == 1).sum()) == 8874 and int((tag == 0).sum()) == 80000
    assert (tag[:8874] == 1).all()  # walls first in memory
    assert np.allclose(s.box, [5.496, 2.13])
    assert s.dt == pytest.approx(0.25 * 0.005 / (10 * np.sqrt(2) + np.sqrt(2)))
    nw = s.state["nw"]
    wall = tag == 1
    assert torch.allclose(nw[wall].norm(dim=1), torch.ones(8874), atol=1e-5)
    assert (nw[~wall] == 0).all()
    assert (s.state["p"][wall] == 0).all()


def test_lid_driven_cavity_tags():
    s = cases.lid_driven_cavity()
    tag = s.state["tag"]
    assert s.n == 3136 and int((tag == 2).sum()) == 168 and int((tag == 0).sum()) == 2500
    lid = s.state["u"][tag == 2]
    assert torch.all(lid[:, 0] == 1.0)  # bc_fn applied at initialisation


def test_poiseuille_band_force():
    s = cases.poiseuille()
    g = s.g_ext_fn(s.state["r"])
    fluid = s.state["tag"] == 0
    assert torch.all(g[fluid, 0] == 1000.0) and torch.all(g[~fluid, 0] == 0.0)


def test_couette_geometry_and_wall_speed():
    # cases/cf.py: the Poiseuille channel, top wall layers moving at 1.25
    s = cases.couette(dx=0.0333333)
    tag = s.state["tag"]
    assert s.n == 432 and int((tag == 0).sum()) == 360
    assert int((tag == 1).sum()) == 36 and int((tag == 2).sum()) == 36
    assert torch.all(s.state["r"][tag == 2][:, 1] > s.state["r"][tag == 0][:, 1].max())
    assert torch.all(s.state["u"][tag == 2][:, 0] == 1.25)
    assert torch.all(s.g_ext_fn(s.state["r"]) == 0.0)


def test_cavity_channel_batch_shapes():
    batch = cases.cavity_channel_batch(8, seed=0)
    ns = [s.n for s in batch]
    assert [s.name for s in batch] == ["ldc", "pf"] * 4
    assert min(ns) > 500 and max(ns) < 60000
    for s in batch:
        assert 0.004 - 1e-12 <= s.dx <= 0.02 + 1e-12
    pf = batch[1]
    eta = pf.viscosity
    assert pf.g_ext_fn.spec["g"][0] == pytest.approx(8 * eta * 1.25)


def test_cube_of_water_layout():
    # cases/cw.py + cw.yaml: walls of the unit box first, the 0.3 cube at (0.5, 0.5)
    s = cases.cube_of_water()
    tag, r, u = s.state["tag"], s.state["r"], s.state["u"]
    assert s.n == 312 and int((tag == 1).sum()) == 276 and (tag[:276] == 1).all()
    f = tag == 0
    assert torch.allclose(r[f].min(0).values, torch.tensor([0.675, 0.675]))
    assert torch.all(u[f] == torch.tensor([0.0, -0.5])) and torch.all(u[~f] == 0.0)
    assert (s.state["p"][~f] == 0).all()  # bc_fn at initialisation
    assert s.solver["is_rho_evol"] and s.solver["is_bc_trick"]


def test_reverse_poiseuille_force_flips_at_y1():
    # cases/rpf.py: +g in x for y <= 1, -g above; no walls
    s = cases.reverse_poiseuille()
    assert s.n == 3200 and bool((s.state["tag"] == 0).all()) and s.dt == 0.0005
    r = torch.tensor([[0.5, 0.5], [0.5, 1.0], [0.5, 1.0001], [0.5, 1.9]])
    assert s.g_ext_fn(r)[:, 0].tolist() == [1.0, 1.0, -1.0, -1.0]
    assert s.p_bg == pytest.approx(0.05 * 100.0)
    assert cases.reverse_poiseuille(dim=3, dx=0.05).n == 20 * 40 * 10


def test_unit_cube_layout():
    # cases/ut.py + ut.yaml: a 0.5 cube of fluid at 0.25 in a periodic unit box
    s = cases.unit_cube()
    r = s.state["r"]
    assert s.n == 625 and torch.allclose(r.min(0).values, torch.tensor([0.26, 0.26]))
    assert torch.allclose(r.max(0).values, torch.tensor([0.74, 0.74]))
    assert s.solver["is_rho_evol"] and not s.solver["is_bc_trick"]


@pytest.mark.parametrize("make", [lambda: cases.dam_break(dx=0.05),
                                  lambda: cases.lid_driven_cavity(dx=0.05),
                                  lambda: cases.poiseuille(dx=0.05),
                                  lambda: cases.couette(dx=0.05),
                                  lambda: cases.heat_transfer(dx=0.05),
                                  lambda: cases.cube_of_water(),
                                  lambda: cases.reverse_poiseuille(dx=0.05),
                                  lambda: cases.unit_cube(dx=0.05)])
def test_descriptors_match_oracle_callbacks(make):
    s = make()
    g = torch.Generator().manual_seed(0)
    st = {k: (v + torch.randn(v.shape, generator=g) if v.is_floating_point() else v)
          for k, v in s.state.items()}
    st64 = {k: (v.double() if v.is_floating_point() else v.long()) for k, v in st.items()}
    ours = s.bc_fn({k: v.double() if v.is_floating_point() else v for k, v in st.items()})
    ref = oracle_bc(s)(st64)
    for k in ("u", "v", "dudt", "dvdt", "p"):
        assert torch.equal(ours[k], ref[k]), k
    assert torch.equal(s.g_ext_fn(st64["r"]), oracle_g(s)(st64["r"]))


def test_heat_transfer_layout():
    """cases/ht.py: a 1 x 0.2 fluid layer between two 3-layer walls, the hot
    Dirichlet part of the bottom wall within 0.25 of the middle, the
    temperature fields of case_setup.py:298-306, noise on the fluid only."""
    dx = 0.02
    s = cases.heat_transfer(dx=dx, r0_noise_factor=0.0)
    tag = s.state["tag"].numpy()
    assert (tag == 0).sum() == 50 * 10 and (tag > 0).sum() == 2 * 50 * 3
    hot = s.state["r"][torch.as_tensor(tag == 3)].double()
    assert len(hot) == 24 * 3 and (hot[:, 1] < 3 * dx).all()
    assert ((hot[:, 0] - 0.5).abs() < 0.25).all()
    for k, v in (("T", 1.0), ("kappa", 7.313), ("Cp", 305.27)):
        assert torch.allclose(s.state[k][torch.as_tensor(tag != 3)], torch.tensor(v))
    assert (s.state["T"][torch.as_tensor(tag == 3)] == np.float32(1.23)).all()
    assert s.solver["is_heat_conduction"] and s.solver["is_bc_trick"]
    noisy = cases.heat_transfer(dx=dx, seed=3)
    moved = (noisy.state["r"] - s.state["r"]).abs().sum(1) > 0
    assert moved[torch.as_tensor(tag == 0)].all() and not moved[torch.as_tensor(tag > 0)].any()


def test_moving_wall_normals_only_where_the_reference_recomputes():
    # case_setup.py:209-218: moving walls with the Riemann solver or free slip
    assert cases.lid_driven_cavity(dx=0.05, solver_name="RIE").nw_fn is not None
    assert cases.lid_driven_cavity(dx=0.05, free_slip=True).nw_fn is not None
    assert cases.couette(dx=0.05, solver_name="RIE").nw_fn is not None
    assert cases.lid_driven_cavity(dx=0.05).nw_fn is None
    assert cases.dam_break(dx=0.05).nw_fn is None  # walls at rest
    s = cases.lid_driven_cavity(dx=0.05, solver_name="RIE")
    wall = torch.as_tensor(s.nw_fn.wall)
    assert s.state["nw"][wall].norm(dim=1).min() > 0.99
    assert s.state["nw"][~wall].abs().max() == 0


def test_matscipy_backend_arguments():
    from jaxsph_gb300 import space

    disp, _ = space.periodic(np.ones(2))
    fns = partition.neighbor_list(disp, np.ones(2), 0.1, backend="matscipy",
                                  num_particles_max=100, pbc=np.array([True, True]))
    assert fns.matscipy and fns.num_particles_max == 100
    assert fns.config().nl_backend == _lib.NL_MATSCIPY
    assert fns.case(10).r_cutoff == 0.1  # the cutoff as matscipy gets it
    with pytest.raises(NotImplementedError):
        partition.neighbor_list(disp, np.ones(2), 0.1, backend="matscipy",
                                pbc=np.array([True, False]))
    with pytest.raises(NotImplementedError):
        partition.neighbor_list(disp, np.ones(2), 0.1, backend="unknown")


def test_fourier_perturbation_is_divergence_free_periodic_and_scaled():
    """The adjoint workload's initial perturbation: u = (dpsi/dy, -dpsi/dx)
    has zero divergence, the unit period of the box and RMS speed sigma."""
    rng = np.random.default_rng(5)
    pts = rng.uniform(0.0, 1.0, (64, 2))
    eps = 1e-5
    # one call for every probe: the field is scaled by its RMS over the points
    # it is given, so all probes must share that scale
    probes = [pts + [eps, 0.0], pts - [eps, 0.0], pts + [0.0, eps], pts - [0.0, eps], pts,
              pts + [1.0, -1.0]]
    u_all = cases.fourier_perturbation(np.concatenate(probes), 0.1, 8, 1).reshape(6, -1, 2)
    div = (u_all[0, :, 0] - u_all[1, :, 0] + u_all[2, :, 1] - u_all[3, :, 1]) / (2 * eps)
    # velocity gradients are ~ 2 pi kmax |u|; central differences leave ~eps^2 of them
    grad_scale = 2 * np.pi * 8 * np.abs(u_all[4]).max()
    assert np.abs(div).max() < 1e-6 * grad_scale
    np.testing.assert_allclose(u_all[5], u_all[4], atol=1e-9)
    grid = (np.stack(np.meshgrid(np.arange(32), np.arange(32)), -1).reshape(-1, 2) + 0.5) / 32
    whole = cases.fourier_perturbation(grid, 0.1, 8, 1)
    assert abs(np.sqrt((whole ** 2).sum(1).mean()) - 0.1) < 1e-12
    assert not np.allclose(whole, cases.fourier_perturbation(grid, 0.1, 8, 2))


@pytest.mark.parametrize("mask_self", [False, True])
@pytest.mark.parametrize("cap_factor", [0.6, 1.0, 1.5])
def test_matscipy_edge_order_truncation_and_padding(mask_self, cap_factor):
    """The host ordering of the matscipy backend's list (self edges first, then
    pairs by first index), truncated to the capacity or padded, equals the
    oracle's restatement for edges arriving in any order."""
    rng = np.random.default_rng(3)
    n = 60
    r = torch.as_tensor(rng.uniform(0.0, 1.0, (n, 2)), dtype=torch.float32)
    edges = oracle.partition.matscipy_edges(r, n, [1.0, 1.0], 0.2, mask_self)
    cap = int(edges.shape[1] * cap_factor)
    want, overflow = oracle.partition.matscipy_idx(edges, cap, n)
    shuffled = edges[:, torch.as_tensor(rng.permutation(edges.shape[1]))].to(torch.int32)
    got = partition.NeighborListFns._matscipy_order(None, shuffled, cap, n)
    assert got.dtype == torch.int32 and got.shape == (2, cap)
    assert torch.equal(got.long(), want)
    assert overflow == (cap_factor < 1.0)


@pytest.mark.parametrize("gamma", [1.0, 7.0])
def test_product_eos_matches_the_oracle_and_inverts(gamma):
    from jaxsph_gb300 import eos

    rho = torch.linspace(0.9, 1.1, 41, dtype=torch.float64)
    pairs = [(eos.TaitEoS(100.0, 1.0, 3.0, gamma), oracle.sph.TaitEoS(100.0, 1.0, 3.0, gamma)),
             (eos.RIEMANNEoS(1.0, 2.0, 1.4142), oracle.sph.RIEMANNEoS(1.0, 2.0, 1.4142))]
    for prod, ref in pairs:
        p = prod.p_fn(rho)
        torch.testing.assert_close(p, ref.p_fn(rho), rtol=1e-15, atol=1e-12)
        torch.testing.assert_close(prod.rho_fn(p), ref.rho_fn(p), rtol=1e-15, atol=0)
        torch.testing.assert_close(prod.rho_fn(p), rho, rtol=1e-13, atol=0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_product_periodic_space_matches_the_oracle_bitwise(dtype):
    """space.periodic's displacement and shift (jax_md/space.py:170-209) on the
    host equal the oracle's jnp.mod restatement bit for bit, including values on
    and just beyond the box faces."""
    from jaxsph_gb300 import space

    side_np = np.array([1.0, 2.0 * np.pi])
    side = torch.as_tensor(side_np, dtype=dtype)
    rng = np.random.default_rng(11)
    a = torch.as_tensor(rng.uniform(-0.2, 1.2, (500, 2)) * side_np, dtype=dtype)
    b = torch.as_tensor(rng.uniform(0.0, 1.0, (500, 2)) * side_np, dtype=dtype)
    edge = torch.tensor([[0.0, 0.0], [1.0, 2 * np.pi], [-0.5, -np.pi], [0.5, np.pi]], dtype=dtype)
    a = torch.cat([a, edge, torch.nextafter(edge, edge + 1), torch.nextafter(edge, edge - 1)])
    b = torch.cat([b, torch.zeros_like(edge).repeat(3, 1)])
    disp, shift = space.periodic(side_np)
    got = disp(a, b)
    want = oracle.space.periodic_displacement(side, a - b)
    assert got.dtype == dtype and torch.equal(got, want)
    dr = torch.as_tensor(rng.normal(0.0, 0.05, a.shape), dtype=dtype)
    assert torch.equal(shift(b, dr), oracle.space.periodic_shift(side, b, dr))
    assert torch.equal(shift(a, dr), oracle.space.periodic_shift(side, a, dr))
