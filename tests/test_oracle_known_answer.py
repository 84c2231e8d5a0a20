"""Known-answer check of the oracle's forward pass on a handful of particles.

The reference's tests hold no per-particle density or acceleration values, so
this test computes them a second, independent way: scalar Python loops over
particle pairs written straight from the reference's formulas, with the kernel
derivatives in closed form instead of autograd --

* kernels (jax_sph/kernel.py:51-103): quintic W = s (q3^5 - 6 q2^5 + 15 q1^5),
  dW/dr = s/h (-5 q3^4 + 30 q2^4 - 75 q1^4); Wendland C2 W = s (1-q/2)^4 (2q+1),
  dW/dr = -5 s q (1-q/2)^3 / h;
* summation density rho_i = m_i sum_j W_ij over every j within the cutoff,
  self included (solver.py:176-178), Tait p = p_ref ((rho/rho0)^g - 1) + p_bg
  (eos.py:20-37);
* the standard acceleration with transport-velocity stress and the TVF term
  (solver.py:199-256), r_ij = r_i - r_j the minimum-image displacement
  (jax_md/space.py:170-181), EPS = 2.22e-16 (solver.py:21);
* the Riemann solver's acceleration with the wall mirror states, the
  Shepard wall velocity and the limiter (solver.py:316-401, :533-588), on
  fluid particles above a row of wall particles under gravity;
* the generalized wall BC, no-slip and free-slip (solver.py:431-530: Shepard
  wall velocity and pressure with the gravity term, inverse EOS for every
  particle) and Monaghan's artificial viscosity (:404-428);
* one si_euler step (integrator.py:22-56) with SPH continuity (solver.py:24-30)
  and a particle drifting through a periodic face, and the Riemann continuity
  with wall mirror states (solver.py:108-164);
* delta-SPH: Marrone's density evolution with both renormalised gradient
  terms and the diffusive acceleration (solver.py:33-105, :259-313), the
  density renormalisation (:167-173) and Cleary's temperature equation
  (:591-610, :832-850).

One pair sits across a periodic face, so a wrong image or sign shows. The
vectorised oracle (gather / index_add over the edge list, gradients by
autograd) must agree to float64 rounding.
"""

import math

import pytest
import torch

import oracle

EPS = 2.220446049250313e-16


def _sigma(name, dim, h):
    if name == "QSK":
        return (7.0 / 478.0 / math.pi / h**2) if dim == 2 else (3.0 / 359.0 / math.pi / h**3)
    return (7.0 / 4.0 / math.pi / h**2) if dim == 2 else (21.0 / 16.0 / math.pi / h**3)


def _w_dw(name, dim, h, r):
    s = _sigma(name, dim, h)
    q = r / h
    if name == "QSK":
        q1, q2, q3 = max(0.0, 1 - q), max(0.0, 2 - q), max(0.0, 3 - q)
        w = s * (q3**5 - 6 * q2**5 + 15 * q1**5)
        dw = s / h * (-5 * q3**4 + 30 * q2**4 - 75 * q1**4)
    else:
        q1 = max(0.0, 1 - 0.5 * q)
        w = s * q1**4 * (2 * q + 1)
        dw = -5 * s * q * q1**3 / h
    return w, dw


def _min_image(a, b, box):
    d = [a[k] - b[k] for k in range(len(a))]
    return [x - box[k] * round(x / box[k]) for k, x in enumerate(d)]


def _scalar_forward(name, st, box, h, cutoff, p_ref, rho0, p_bg, gamma):
    r, m, eta = st["r"], st["mass"], st["eta"]
    u, v = st["u"], st["v"]
    n, dim = len(r), len(r[0])
    pairs = []
    for i in range(n):
        for j in range(n):
            rij = _min_image(r[i], r[j], box)
            d = math.sqrt(sum(x * x for x in rij))
            if d < cutoff:
                pairs.append((i, j, rij, d))
    rho = [0.0] * n
    for i, j, rij, d in pairs:
        rho[i] += _w_dw(name, dim, h, d)[0]
    rho = [m[i] * rho[i] for i in range(n)]
    p = [p_ref * ((x / rho0) ** gamma - 1) + p_bg for x in rho]
    p_bg_tvf = p_ref * ((0.0 / rho0) ** gamma - 1) + p_bg
    dudt = [[0.0] * dim for _ in range(n)]
    dvdt = [[0.0] * dim for _ in range(n)]
    for i, j, rij, d in pairs:
        dw = _w_dw(name, dim, h, d)[1]
        c = ((m[i] / rho[i]) ** 2 + (m[j] / rho[j]) ** 2) / m[i] * dw / (d + EPS)
        eta_ij = 2 * eta[i] * eta[j] / (eta[i] + eta[j] + EPS)
        p_ij = (rho[j] * p[i] + rho[i] * p[j]) / (rho[i] + rho[j])
        si = sum((v[i][k] - u[i][k]) * rij[k] for k in range(dim))
        sj = sum((v[j][k] - u[j][k]) * rij[k] for k in range(dim))
        for k in range(dim):
            a_r = 0.5 * (rho[i] * u[i][k] * si + rho[j] * u[j][k] * sj)
            dudt[i][k] += c * (-p_ij * rij[k] + a_r + eta_ij * (u[i][k] - u[j][k]))
            dvdt[i][k] += c * p_bg_tvf * rij[k]
    return rho, p, dudt, dvdt, len(pairs)


POSITIONS = {
    2: [[0.50, 0.50], [0.57, 0.53], [0.44, 0.58], [0.52, 0.40], [0.02, 0.50], [0.96, 0.52],
        [0.30, 0.30]],
    3: [[0.50, 0.50, 0.50], [0.58, 0.53, 0.49], [0.45, 0.60, 0.52], [0.51, 0.43, 0.57],
        [0.02, 0.50, 0.50], [0.95, 0.52, 0.47], [0.20, 0.20, 0.20]],
}


@pytest.mark.parametrize("name,dim", [("QSK", 2), ("WC2K", 3), ("WC2K", 2), ("QSK", 3)])
def test_oracle_forward_matches_hand_computed_pair_sums(name, dim):
    g = torch.Generator().manual_seed(7 + dim)
    r = torch.tensor(POSITIONS[dim], dtype=torch.float64)
    n = r.shape[0]
    dx = 0.05
    h = dx
    box = [1.0] * dim
    cutoff = (3.0 if name == "QSK" else 2.0) * h
    p_ref, rho0, p_bg, gamma = 100.0, 1.0, 3.0, 1.0
    st = {
        "r": r,
        "tag": torch.zeros(n, dtype=torch.int32),
        "mass": 1e-3 * (1.0 + 0.3 * torch.rand(n, generator=g, dtype=torch.float64)),
        "eta": 0.01 * (1.0 + torch.rand(n, generator=g, dtype=torch.float64)),
        "u": torch.randn(n, dim, generator=g, dtype=torch.float64),
        "v": torch.randn(n, dim, generator=g, dtype=torch.float64),
        "dudt": torch.zeros(n, dim, dtype=torch.float64),
        "dvdt": torch.zeros(n, dim, dtype=torch.float64),
        "rho": torch.ones(n, dtype=torch.float64),
        "drhodt": torch.zeros(n, dtype=torch.float64),
        "p": torch.zeros(n, dtype=torch.float64),
        "nw": torch.zeros(n, dim, dtype=torch.float64),
    }
    fns = oracle.partition.NeighborListFns(box, cutoff, torch.float64, mask_self=False)
    nb = fns.allocate(r)
    solver = oracle.sph.WCSPH(box, oracle.sph.TaitEoS(p_ref, rho0, p_bg, gamma),
                              oracle.sph.g_ext_zero, dx, dim, 1e-4, 10.0, kernel=name)
    out = solver.forward(st, nb.idx)

    plain = {k: v.tolist() for k, v in st.items()}
    rho, p, dudt, dvdt, n_pairs = _scalar_forward(name, plain, box, h, cutoff, p_ref, rho0,
                                                  p_bg, gamma)
    assert int((nb.idx[0] < n).sum()) == n_pairs
    # the configuration has real pairs, one of them (4, 5) through the periodic face
    assert n_pairs > n + 4
    edges = set(map(tuple, nb.idx.t().tolist()))
    assert (4, 5) in edges and (5, 4) in edges
    torch.testing.assert_close(out["rho"], torch.tensor(rho, dtype=torch.float64),
                               rtol=1e-12, atol=0)
    torch.testing.assert_close(out["p"], torch.tensor(p, dtype=torch.float64),
                               rtol=1e-12, atol=1e-12)
    scale = max(abs(x) for row in dudt for x in row)
    torch.testing.assert_close(out["dudt"], torch.tensor(dudt, dtype=torch.float64),
                               rtol=0, atol=1e-12 * scale)
    scale = max(abs(x) for row in dvdt for x in row)
    torch.testing.assert_close(out["dvdt"], torch.tensor(dvdt, dtype=torch.float64),
                               rtol=0, atol=1e-12 * scale)
    # the isolated particle sees only itself
    assert abs(out["rho"][-1].item() - st["mass"][-1].item() * _w_dw(name, dim, h, 0.0)[0]) \
        < 1e-12 * out["rho"][-1].item()


def _scalar_riemann(name, st, box, h, cutoff, u_ref, rho0, p_bg, c_ref, eta_limiter, g):
    """Riemann SPH (solver.py:316-401, :533-588, :741-744, :886-921) with the
    generalized wall BC on: SOLID_WALL senders mirror the receiver's state
    through their normal, their viscous velocity is 2 u_j - u_tilde_j."""
    r, m, eta, tag, nw = st["r"], st["mass"], st["eta"], st["tag"], st["nw"]
    u = st["u"]
    n, dim = len(r), len(r[0])
    pairs = []
    for i in range(n):
        for j in range(n):
            rij = _min_image(r[i], r[j], box)
            d = math.sqrt(sum(x * x for x in rij))
            if d < cutoff:
                pairs.append((i, j, rij, d))
    rho = list(st["rho"])
    summ = [0.0] * n
    for i, j, rij, d in pairs:
        summ[i] += _w_dw(name, dim, h, d)[0]
    rho = [m[i] * summ[i] if tag[i] == 0 else rho[i] for i in range(n)]

    def eos_p(x):
        return 100 * u_ref**2 * (x - rho0) + p_bg

    def eos_rho(x):
        return (x - p_bg) / (100 * u_ref**2) + rho0

    p = [eos_p(x) for x in rho]
    # Shepard average of the fluid velocities around every particle
    num = [[0.0] * dim for _ in range(n)]
    den = [0.0] * n
    for i, j, rij, d in pairs:
        if tag[j] == 0:
            w = _w_dw(name, dim, h, d)[0]
            den[i] += w
            for k in range(dim):
                num[i][k] += w * u[j][k]
    ut = [[num[i][k] / (den[i] + EPS) for k in range(dim)] for i in range(n)]
    gvec = [0.0, -g] + [0.0] * (dim - 2)
    dudt = [list(gvec) for _ in range(n)]

    def dot(a, b):
        return sum(a[k] * b[k] for k in range(dim))

    for i, j, rij, d in pairs:
        dw = _w_dw(name, dim, h, d)[1]
        e = [x / (d + EPS) for x in rij]
        wall = tag[j] != 0
        if wall:
            u_l = -dot(u[i], nw[j])
            u_r = -u_l + 2 * dot(u[j], nw[j])
            p_r = p[i] + rho[i] * (-dot(gvec, rij))
            rho_r = eos_rho(p_r)
        else:
            u_l, u_r = -dot(u[i], e), -dot(u[j], e)
            p_r, rho_r = p[j], rho[j]
        beta = min(eta_limiter * max(u_l - u_r, 0.0), c_ref)
        p_star = (p[i] + p_r) / 2 + 0.5 * (rho[i] + rho_r) / 2 * (u_l - u_r) * beta
        eta_ij = 2 * eta[i] * eta[j] / (eta[i] + eta[j] + EPS)
        for k in range(dim):
            u_d = 2 * u[j][k] - ut[j][k]
            v_ij = u[i][k] - u_d if wall else u[i][k] - u[j][k]
            eq9 = -2 * m[j] * (p_star / (rho[i] * rho[j])) * dw * e[k]
            eq6 = 2 * m[j] * eta_ij / (rho[i] * rho[j]) * v_ij / (d + EPS) * dw
            dudt[i][k] += eq9 + eq6
    return rho, p, dudt, len(pairs)


def test_oracle_riemann_forward_with_walls_matches_hand_computed_sums():
    name, dim = "QSK", 2
    g = torch.Generator().manual_seed(11)
    dx = h = 0.05
    box = [1.0, 1.0]
    cutoff = 3 * h
    # a fluid cluster above a row of SOLID_WALL particles with upward normals
    fluid = [[0.50, 0.50], [0.56, 0.52], [0.45, 0.55], [0.52, 0.44], [0.47, 0.47]]
    walls = [[0.42 + 0.05 * k, 0.40] for k in range(5)]
    r = torch.tensor(fluid + walls, dtype=torch.float64)
    n = r.shape[0]
    tag = torch.tensor([0] * len(fluid) + [1] * len(walls), dtype=torch.int32)
    nw = torch.zeros(n, dim, dtype=torch.float64)
    nw[len(fluid):, 1] = 1.0
    u_ref, rho0, p_bg, c_ref, eta_limiter, grav = 1.0, 1.0, 0.0, 10.0, 3, 1.0
    u = 0.3 * torch.randn(n, dim, generator=g, dtype=torch.float64)
    u[len(fluid):] = 0.0
    st = {
        "r": r, "tag": tag, "nw": nw, "u": u, "v": u.clone(),
        "mass": dx * dx * (1.0 + 0.1 * torch.rand(n, generator=g, dtype=torch.float64)),
        "eta": 0.01 * (1.0 + torch.rand(n, generator=g, dtype=torch.float64)),
        "dudt": torch.zeros(n, dim, dtype=torch.float64),
        "dvdt": torch.zeros(n, dim, dtype=torch.float64),
        "rho": 1.0 + 0.01 * torch.rand(n, generator=g, dtype=torch.float64),
        "drhodt": torch.zeros(n, dtype=torch.float64),
        "p": torch.zeros(n, dtype=torch.float64),
    }
    fns = oracle.partition.NeighborListFns(box, cutoff, torch.float64, mask_self=False)
    nb = fns.allocate(r)
    solver = oracle.sph.WCSPH(box, oracle.sph.RIEMANNEoS(rho0, p_bg, u_ref),
                              oracle.sph.make_g_ext_db(grav), dx, dim, 1e-4, c_ref,
                              eta_limiter=eta_limiter, solver="RIE", kernel=name,
                              is_bc_trick=True)
    out = solver.forward(st, nb.idx)
    plain = {k: v.tolist() for k, v in st.items()}
    rho, p, dudt, n_pairs = _scalar_riemann(name, plain, box, h, cutoff, u_ref, rho0, p_bg,
                                            c_ref, eta_limiter, grav)
    assert int((nb.idx[0] < n).sum()) == n_pairs
    # fluid particles see the wall
    assert any(a < len(fluid) <= b for a, b in nb.idx.t().tolist() if b < n)
    torch.testing.assert_close(out["rho"], torch.tensor(rho, dtype=torch.float64),
                               rtol=1e-12, atol=0)
    torch.testing.assert_close(out["p"], torch.tensor(p, dtype=torch.float64),
                               rtol=0, atol=1e-10)
    scale = max(abs(x) for row in dudt for x in row)
    torch.testing.assert_close(out["dudt"], torch.tensor(dudt, dtype=torch.float64),
                               rtol=0, atol=1e-12 * scale)


def _scalar_sph_walls(name, st, box, h, dx, cutoff, p_ref, rho0, p_bg, gamma, g, alpha,
                      free_slip):
    """Standard SPH with the generalized wall BC (solver.py:431-530, order of
    :796-821) and Monaghan's artificial viscosity (:404-428, c_ab = 10)."""
    r, m, eta, tag, nw = st["r"], st["mass"], st["eta"], st["tag"], st["nw"]
    u, v = [list(x) for x in st["u"]], [list(x) for x in st["v"]]
    n, dim = len(r), len(r[0])

    def dot(a, b):
        return sum(a[k] * b[k] for k in range(dim))

    pairs = []
    for i in range(n):
        for j in range(n):
            rij = _min_image(r[i], r[j], box)
            d = math.sqrt(sum(x * x for x in rij))
            if d < cutoff:
                pairs.append((i, j, rij, d))
    summ = [0.0] * n
    for i, j, rij, d in pairs:
        summ[i] += _w_dw(name, dim, h, d)[0]
    rho = [m[i] * summ[i] if tag[i] == 0 else st["rho"][i] for i in range(n)]
    p = [p_ref * ((x / rho0) ** gamma - 1) + p_bg for x in rho]
    p_bg_tvf = p_ref * (0.0 - 1) + p_bg
    gvec = [0.0, -g] + [0.0] * (dim - 2)
    # wall particles: Shepard sums over their fluid neighbours
    wsum = [0.0] * n
    uw = [[0.0] * dim for _ in range(n)]
    vw = [[0.0] * dim for _ in range(n)]
    pw = [0.0] * n
    rwf = [[0.0] * dim for _ in range(n)]
    for i, j, rij, d in pairs:
        if tag[j] != 0:
            continue
        w = _w_dw(name, dim, h, d)[0]
        wsum[i] += w
        pw[i] += w * p[j]
        for k in range(dim):
            uw[i][k] += w * u[j][k]
            vw[i][k] += w * v[j][k]
            rwf[i][k] += rho[j] * w * rij[k]
    for i in range(n):
        if tag[i] == 0:
            continue
        xu = [x / (wsum[i] + EPS) for x in uw[i]]
        xv = [x / (wsum[i] + EPS) for x in vw[i]]
        if free_slip:
            nn = [-x for x in nw[i]]
            xu = [nn[k] * dot(xu, nn) for k in range(dim)]
            xv = [nn[k] * dot(xv, nn) for k in range(dim)]
        u[i] = [2 * u[i][k] - xu[k] for k in range(dim)]
        v[i] = [2 * v[i][k] - xv[k] for k in range(dim)]
        p[i] = (pw[i] + dot(gvec, rwf[i])) / (wsum[i] + EPS)
    rho = [rho0 * ((x + p_ref - p_bg) / p_ref) ** (1 / gamma) for x in p]
    dudt = [list(gvec) for _ in range(n)]
    dvdt = [[0.0] * dim for _ in range(n)]
    for i, j, rij, d in pairs:
        dw = _w_dw(name, dim, h, d)[1]
        e = [x / (d + EPS) for x in rij]
        c = ((m[i] / rho[i]) ** 2 + (m[j] / rho[j]) ** 2) / m[i] * dw / (d + EPS)
        eta_ij = 2 * eta[i] * eta[j] / (eta[i] + eta[j] + EPS)
        p_ij = (rho[j] * p[i] + rho[i] * p[j]) / (rho[i] + rho[j])
        si = dot([v[i][k] - u[i][k] for k in range(dim)], rij)
        sj = dot([v[j][k] - u[j][k] for k in range(dim)], rij)
        both_fluid = tag[i] == 0 and tag[j] == 0
        av = 0.0
        if both_fluid:
            av = m[j] * alpha * dx * 10.0 * dot([u[i][k] - u[j][k] for k in range(dim)], rij) \
                / ((rho[i] + rho[j]) / 2 * (d * d + 0.01 * dx * dx))
        for k in range(dim):
            a_r = 0.5 * (rho[i] * u[i][k] * si + rho[j] * u[j][k] * sj)
            dudt[i][k] += c * (-p_ij * rij[k] + a_r + eta_ij * (u[i][k] - u[j][k]))
            dudt[i][k] += av * dw * e[k]
            dvdt[i][k] += c * p_bg_tvf * rij[k]
    return rho, p, u, v, dudt, dvdt


@pytest.mark.parametrize("free_slip", [False, True])
def test_oracle_wall_bc_forward_matches_hand_computed_sums(free_slip):
    name, dim = "QSK", 2
    g = torch.Generator().manual_seed(13)
    dx = h = 0.05
    box = [1.0, 1.0]
    cutoff = 3 * h
    fluid = [[0.50, 0.50], [0.56, 0.52], [0.45, 0.55], [0.52, 0.44], [0.47, 0.47]]
    walls = [[0.42 + 0.05 * k, 0.40] for k in range(5)] + [[0.44 + 0.05 * k, 0.36]
                                                          for k in range(4)]
    r = torch.tensor(fluid + walls, dtype=torch.float64)
    n, nf = r.shape[0], len(fluid)
    tag = torch.tensor([0] * nf + [1] * (n - nf), dtype=torch.int32)
    tag[-1] = 2  # one MOVING_WALL
    nw = torch.zeros(n, dim, dtype=torch.float64)
    nw[nf:, 1] = 1.0
    p_ref, rho0, p_bg, gamma, grav, alpha = 100.0, 1.0, 2.0, 1.0, 1.0, 0.1
    u = 0.3 * torch.randn(n, dim, generator=g, dtype=torch.float64)
    u[nf:] = 0.0
    u[-1, 0] = 1.0
    st = {
        "r": r, "tag": tag, "nw": nw, "u": u,
        "v": u + 0.05 * torch.randn(n, dim, generator=g, dtype=torch.float64),
        "mass": dx * dx * (1.0 + 0.1 * torch.rand(n, generator=g, dtype=torch.float64)),
        "eta": 0.01 * (1.0 + torch.rand(n, generator=g, dtype=torch.float64)),
        "dudt": torch.zeros(n, dim, dtype=torch.float64),
        "dvdt": torch.zeros(n, dim, dtype=torch.float64),
        "rho": 1.0 + 0.01 * torch.rand(n, generator=g, dtype=torch.float64),
        "drhodt": torch.zeros(n, dtype=torch.float64),
        "p": torch.zeros(n, dtype=torch.float64),
    }
    fns = oracle.partition.NeighborListFns(box, cutoff, torch.float64, mask_self=False)
    nb = fns.allocate(r)
    solver = oracle.sph.WCSPH(box, oracle.sph.TaitEoS(p_ref, rho0, p_bg, gamma),
                              oracle.sph.make_g_ext_db(grav), dx, dim, 1e-4, 10.0,
                              kernel=name, is_bc_trick=True, artificial_alpha=alpha,
                              is_free_slip=free_slip)
    out = solver.forward(st, nb.idx)
    plain = {k: v.tolist() for k, v in st.items()}
    rho, p, uu, vv, dudt, dvdt = _scalar_sph_walls(name, plain, box, h, dx, cutoff, p_ref, rho0,
                                                   p_bg, gamma, grav, alpha, free_slip)
    f64 = torch.float64
    torch.testing.assert_close(out["p"], torch.tensor(p, dtype=f64), rtol=0, atol=1e-10)
    torch.testing.assert_close(out["rho"], torch.tensor(rho, dtype=f64), rtol=1e-12, atol=0)
    torch.testing.assert_close(out["u"], torch.tensor(uu, dtype=f64), rtol=0, atol=1e-13)
    torch.testing.assert_close(out["v"], torch.tensor(vv, dtype=f64), rtol=0, atol=1e-13)
    for key, want in (("dudt", dudt), ("dvdt", dvdt)):
        scale = max(abs(x) for row in want for x in row)
        torch.testing.assert_close(out[key], torch.tensor(want, dtype=f64), rtol=0,
                                   atol=1e-12 * scale)
    # the walls really took the BC: a wall velocity differs from its input
    assert (out["u"][nf:] - st["u"][nf:]).abs().max() > 1e-3


def _pairs(r, box, cutoff):
    out = []
    for i in range(len(r)):
        for j in range(len(r)):
            rij = _min_image(r[i], r[j], box)
            d = math.sqrt(sum(x * x for x in rij))
            if d < cutoff:
                out.append((i, j, rij, d))
    return out


def test_oracle_si_euler_step_with_continuity_matches_hand_computed_values():
    """si_euler (integrator.py:22-56): u += dt dudt, v = u + tvf dt/2 dvdt,
    r = (r + dt v) mod L, then SPH continuity (solver.py:24-30) from the
    state's density and the standard + TVF accelerations on the new density."""
    name, dim = "WC2K", 3
    g = torch.Generator().manual_seed(17)
    dx = h = 0.05
    box = [1.0, 1.0, 1.0]
    cutoff = 2 * h
    r = torch.tensor(POSITIONS[3], dtype=torch.float64)
    r[4, 0] = 0.001  # drifts across the lower face
    n = r.shape[0]
    p_ref, rho0, p_bg, gamma, tvf, dt = 100.0, 1.0, 0.0, 1.0, 1.0, 2e-3
    st = {
        "r": r, "tag": torch.zeros(n, dtype=torch.int32),
        "mass": 1e-4 * (1.0 + 0.3 * torch.rand(n, generator=g, dtype=torch.float64)),
        "eta": 0.01 * (1.0 + torch.rand(n, generator=g, dtype=torch.float64)),
        "u": torch.randn(n, dim, generator=g, dtype=torch.float64),
        "v": torch.zeros(n, dim, dtype=torch.float64),
        "dudt": torch.randn(n, dim, generator=g, dtype=torch.float64),
        "dvdt": torch.randn(n, dim, generator=g, dtype=torch.float64),
        "rho": 1.0 + 0.02 * torch.rand(n, generator=g, dtype=torch.float64),
        "drhodt": torch.zeros(n, dtype=torch.float64),
        "p": torch.zeros(n, dtype=torch.float64),
        "nw": torch.zeros(n, dim, dtype=torch.float64),
    }
    st["u"][4, 0] = -2.0  # 4 moves by about -4e-3: through x = 0
    st["dudt"][4, 0] = 0.0
    # room for particle 4 in its new cell: the update keeps the allocated capacities
    fns = oracle.partition.NeighborListFns(box, cutoff, torch.float64, mask_self=False,
                                           capacity_multiplier=4.0)
    nb = fns.allocate(r)
    solver = oracle.sph.WCSPH(box, oracle.sph.TaitEoS(p_ref, rho0, p_bg, gamma),
                              oracle.sph.g_ext_zero, dx, dim, dt, 10.0, kernel=name,
                              is_rho_evol=True)
    out, nb = oracle.sph.si_euler_advance(dt, tvf, st, nb, fns, solver, oracle.sph.bc_identity)
    assert not nb.did_buffer_overflow

    s = {k: v.tolist() for k, v in st.items()}
    u = [[s["u"][i][k] + dt * s["dudt"][i][k] for k in range(dim)] for i in range(n)]
    v = [[u[i][k] + tvf * 0.5 * dt * s["dvdt"][i][k] for k in range(dim)] for i in range(n)]
    rr = [[(s["r"][i][k] + dt * v[i][k]) % box[k] for k in range(dim)] for i in range(n)]
    assert rr[4][0] > 0.99  # wrapped
    m, eta, rho_in = s["mass"], s["eta"], s["rho"]
    pairs = _pairs(rr, box, cutoff)
    drho = [0.0] * n
    for i, j, rij, d in pairs:
        dw = _w_dw(name, dim, h, d)[1]
        gradw = [dw * x / (d + EPS) for x in rij]
        drho[i] += m[j] / rho_in[j] * sum((u[i][k] - u[j][k]) * gradw[k] for k in range(dim))
    drho = [rho_in[i] * drho[i] for i in range(n)]
    rho = [rho_in[i] + dt * drho[i] for i in range(n)]
    p = [p_ref * ((x / rho0) ** gamma - 1) + p_bg for x in rho]
    p_bg_tvf = p_ref * (0.0 - 1) + p_bg
    dudt = [[0.0] * dim for _ in range(n)]
    dvdt = [[0.0] * dim for _ in range(n)]
    for i, j, rij, d in pairs:
        dw = _w_dw(name, dim, h, d)[1]
        c = ((m[i] / rho[i]) ** 2 + (m[j] / rho[j]) ** 2) / m[i] * dw / (d + EPS)
        eta_ij = 2 * eta[i] * eta[j] / (eta[i] + eta[j] + EPS)
        p_ij = (rho[j] * p[i] + rho[i] * p[j]) / (rho[i] + rho[j])
        si = sum((v[i][k] - u[i][k]) * rij[k] for k in range(dim))
        sj = sum((v[j][k] - u[j][k]) * rij[k] for k in range(dim))
        for k in range(dim):
            a_r = 0.5 * (rho[i] * u[i][k] * si + rho[j] * u[j][k] * sj)
            dudt[i][k] += c * (-p_ij * rij[k] + a_r + eta_ij * (u[i][k] - u[j][k]))
            dvdt[i][k] += c * p_bg_tvf * rij[k]

    f64 = torch.float64
    assert any(i == 4 and j == 5 for i, j, _, _ in pairs)
    torch.testing.assert_close(out["r"], torch.tensor(rr, dtype=f64), rtol=0, atol=1e-15)
    torch.testing.assert_close(out["u"], torch.tensor(u, dtype=f64), rtol=0, atol=1e-15)
    torch.testing.assert_close(out["v"], torch.tensor(v, dtype=f64), rtol=0, atol=1e-15)
    torch.testing.assert_close(out["drhodt"], torch.tensor(drho, dtype=f64), rtol=0,
                               atol=1e-12 * max(map(abs, drho)))
    torch.testing.assert_close(out["rho"], torch.tensor(rho, dtype=f64), rtol=1e-13, atol=0)
    for key, want in (("dudt", dudt), ("dvdt", dvdt)):
        scale = max(abs(x) for row in want for x in row)
        torch.testing.assert_close(out[key], torch.tensor(want, dtype=f64), rtol=0,
                                   atol=1e-12 * scale)


def test_oracle_riemann_continuity_matches_hand_computed_values():
    """Riemann continuity (solver.py:108-164, applied :772-790): the linear
    Riemann mass flux, wall senders mirrored through their normals, fluid
    receivers only."""
    name, dim = "QSK", 2
    g = torch.Generator().manual_seed(19)
    dx = h = 0.05
    box = [1.0, 1.0]
    cutoff = 3 * h
    fluid = [[0.50, 0.50], [0.56, 0.52], [0.45, 0.55], [0.52, 0.44], [0.47, 0.47]]
    walls = [[0.42 + 0.05 * k, 0.40] for k in range(5)]
    r = torch.tensor(fluid + walls, dtype=torch.float64)
    n, nf = r.shape[0], len(fluid)
    tag = torch.tensor([0] * nf + [1] * (n - nf), dtype=torch.int32)
    nw = torch.zeros(n, dim, dtype=torch.float64)
    nw[nf:, 1] = 1.0
    u_ref, rho0, p_bg, c_ref, grav, dt = 1.0, 1.0, 0.0, 10.0, 1.0, 1e-4
    u = 0.3 * torch.randn(n, dim, generator=g, dtype=torch.float64)
    u[nf:] = 0.0
    rho_in = 1.0 + 0.01 * torch.rand(n, generator=g, dtype=torch.float64)
    st = {
        "r": r, "tag": tag, "nw": nw, "u": u, "v": u.clone(),
        "mass": dx * dx * (1.0 + 0.1 * torch.rand(n, generator=g, dtype=torch.float64)),
        "eta": 0.01 * (1.0 + torch.rand(n, generator=g, dtype=torch.float64)),
        "dudt": torch.zeros(n, dim, dtype=torch.float64),
        "dvdt": torch.zeros(n, dim, dtype=torch.float64),
        "rho": rho_in,
        "drhodt": torch.zeros(n, dtype=torch.float64),
        "p": 100 * u_ref**2 * (rho_in - rho0) + p_bg,
    }
    fns = oracle.partition.NeighborListFns(box, cutoff, torch.float64, mask_self=False)
    nb = fns.allocate(r)
    solver = oracle.sph.WCSPH(box, oracle.sph.RIEMANNEoS(rho0, p_bg, u_ref),
                              oracle.sph.make_g_ext_db(grav), dx, dim, dt, c_ref,
                              solver="RIE", kernel=name, is_bc_trick=True, is_rho_evol=True)
    out = solver.forward(st, nb.idx)

    s = {k: v.tolist() for k, v in st.items()}
    m, rho, p, uu, nws = s["mass"], s["rho"], s["p"], s["u"], s["nw"]
    gvec = [0.0, -grav]

    def dot(a, b):
        return a[0] * b[0] + a[1] * b[1]

    drho = [0.0] * n
    for i, j, rij, d in _pairs(s["r"], box, cutoff):
        dw = _w_dw(name, dim, h, d)[1]
        e = [x / (d + EPS) for x in rij]
        gradw = [dw * x for x in e]
        if s["tag"][j] != 0:
            u_l = -dot(uu[i], nws[j])
            u_r = -u_l + 2 * dot(uu[j], nws[j])
            p_r = p[i] + rho[i] * (-dot(gvec, rij))
            rho_r = (p_r - p_bg) / (100 * u_ref**2) + rho0
        else:
            u_l, u_r = -dot(uu[i], e), -dot(uu[j], e)
            p_r, rho_r = p[j], rho[j]
        u_avg = (u_l + u_r) / 2
        rho_avg = (rho[i] + rho_r) / 2
        u_star = u_avg + 0.5 * (p[i] - p_r) / (rho_avg * c_ref)
        v_star = [u_star * (-e[k]) + ((uu[i][k] + uu[j][k]) / 2 - u_avg * (-e[k]))
                  for k in range(dim)]
        drho[i] += 2 * rho[i] * m[j] / rho[j] * dot([uu[i][k] - v_star[k] for k in range(dim)],
                                                  gradw)
    drho = [drho[i] if s["tag"][i] == 0 else 0.0 for i in range(n)]
    want_rho = [rho[i] + dt * drho[i] for i in range(n)]
    f64 = torch.float64
    torch.testing.assert_close(out["drhodt"], torch.tensor(drho, dtype=f64), rtol=0,
                               atol=1e-12 * max(map(abs, drho)))
    torch.testing.assert_close(out["rho"], torch.tensor(want_rho, dtype=f64), rtol=1e-14,
                               atol=0)
    assert max(map(abs, drho[:nf])) > 0


def _inv2(a):
    det = a[0][0] * a[1][1] - a[0][1] * a[1][0]
    return [[a[1][1] / det, -a[0][1] / det], [-a[1][0] / det, a[0][0] / det]]


@pytest.mark.parametrize("renorm", [False, True])
def test_oracle_delta_sph_and_heat_match_hand_computed_values(renorm):
    """delta-SPH density evolution with both renormalised gradient terms
    (solver.py:33-105, the sender-side term summed over receivers as the
    reference does), the optional renormalisation (:167-173), the delta-SPH
    acceleration (:259-313) and Cleary's temperature equation (:591-610,
    :832-850), on a jittered periodic 8 x 8 lattice."""
    name, dim = "QSK", 2
    g = torch.Generator().manual_seed(23)
    dx = h = 0.05
    side = 8
    box = [side * dx, side * dx]
    cutoff = 3 * h
    ij = torch.stack(torch.meshgrid(torch.arange(side), torch.arange(side), indexing="xy"),
                     -1).reshape(-1, 2).to(torch.float64)
    r = (ij + 0.5) * dx + 0.1 * dx * torch.randn(side * side, 2, generator=g,
                                                 dtype=torch.float64)
    r = torch.remainder(r, box[0])
    n = r.shape[0]
    p_ref, rho0, p_bg, gamma, c_ref, dt = 100.0, 1.0, 0.0, 1.0, 10.0, 1e-4
    alpha, delta = 0.1, 0.02
    st = {
        "r": r, "tag": torch.zeros(n, dtype=torch.int32),
        "mass": dx * dx * (1.0 + 0.1 * torch.rand(n, generator=g, dtype=torch.float64)),
        "eta": 0.01 * (1.0 + torch.rand(n, generator=g, dtype=torch.float64)),
        "u": 0.5 * torch.randn(n, dim, generator=g, dtype=torch.float64),
        "dudt": torch.zeros(n, dim, dtype=torch.float64),
        "dvdt": torch.zeros(n, dim, dtype=torch.float64),
        "rho": 1.0 + 0.02 * torch.rand(n, generator=g, dtype=torch.float64),
        "drhodt": torch.zeros(n, dtype=torch.float64),
        "p": torch.zeros(n, dtype=torch.float64),
        "nw": torch.zeros(n, dim, dtype=torch.float64),
        "T": 1.0 + torch.rand(n, generator=g, dtype=torch.float64),
        "dTdt": torch.randn(n, generator=g, dtype=torch.float64),
        "kappa": 0.5 + torch.rand(n, generator=g, dtype=torch.float64),
        "Cp": 1.0 + torch.rand(n, generator=g, dtype=torch.float64),
    }
    st["v"] = st["u"] + 0.05 * torch.randn(n, dim, generator=g, dtype=torch.float64)
    fns = oracle.partition.NeighborListFns(box, cutoff, torch.float64, mask_self=False)
    nb = fns.allocate(r)
    solver = oracle.sph.WCSPH(box, oracle.sph.TaitEoS(p_ref, rho0, p_bg, gamma),
                              oracle.sph.g_ext_zero, dx, dim, dt, c_ref, kernel=name,
                              solver="DELTA", is_rho_evol=True, diff_alpha=alpha,
                              diff_delta=delta, is_rho_renorm=renorm,
                              is_heat_conduction=True)
    out = solver.forward(st, nb.idx)

    s = {k: v.tolist() for k, v in st.items()}
    m, rho, u, v, eta = s["mass"], s["rho"], s["u"], s["v"], s["eta"]
    pairs = _pairs(s["r"], box, cutoff)
    assert int((nb.idx[0] < n).sum()) == len(pairs)

    def dot(a, b):
        return a[0] * b[0] + a[1] * b[1]

    def grad(rij, d):
        dw = _w_dw(name, dim, h, d)[1]
        return [dw * x / (d + EPS) for x in rij]

    vol = [m[i] / rho[i] for i in range(n)]
    # M_i = sum over receiver i of outer(-r_ij, gradW_ij V_j); the sender-side
    # matrix sums outer(r_ij, gradW_ij V_i) over the sender j
    mi = [[[0.0, 0.0], [0.0, 0.0]] for _ in range(n)]
    mj = [[[0.0, 0.0], [0.0, 0.0]] for _ in range(n)]
    for i, j, rij, d in pairs:
        gw = grad(rij, d)
        for a in range(2):
            for b in range(2):
                mi[i][a][b] += -rij[a] * gw[b] * vol[j]
                mj[j][a][b] += rij[a] * gw[b] * vol[i]
    li = [_inv2(x) for x in mi]
    lj = [_inv2(x) for x in mj]
    gi = [[0.0, 0.0] for _ in range(n)]
    gj = [[0.0, 0.0] for _ in range(n)]
    for i, j, rij, d in pairs:
        gw = grad(rij, d)
        for a in range(2):
            gi[i][a] += (rho[j] - rho[i]) * sum(li[i][a][b] * gw[b] * vol[j] for b in range(2))
            gj[i][a] += (rho[i] - rho[j]) * sum(lj[j][a][b] * (-gw[b]) * vol[i]
                                                for b in range(2))
    cont = [0.0] * n
    diff = [0.0] * n
    for i, j, rij, d in pairs:
        gw = grad(rij, d)
        cont[i] += dot([u[i][k] - u[j][k] for k in range(2)], gw) * vol[j]
        psi = [2 * (rho[j] - rho[i]) * (-rij[k]) / (d + EPS) ** 2 - gi[i][k] - gj[j][k]
               for k in range(2)]
        diff[i] += dot(psi, gw) * vol[j]
    drho = [rho[i] * cont[i] + c_ref * delta * h * diff[i] for i in range(n)]
    rho_new = [rho[i] + dt * drho[i] for i in range(n)]
    if renorm:
        num = [0.0] * n
        den = [0.0] * n
        for i, j, rij, d in pairs:
            w = _w_dw(name, dim, h, d)[0]
            num[i] += m[j] * w
            den[i] += m[j] / rho_new[j] * w
        rho_new = [num[i] / min(den[i], 1.0) for i in range(n)]
    rho = rho_new
    p = [p_ref * ((x / rho0) ** gamma - 1) + p_bg for x in rho]
    temp = [s["T"][i] + dt * s["dTdt"][i] for i in range(n)]
    kap, cp = s["kappa"], s["Cp"]
    dTdt = [0.0] * n
    dudt = [[0.0, 0.0] for _ in range(n)]
    for i, j, rij, d in pairs:
        gw = grad(rij, d)
        dw = _w_dw(name, dim, h, d)[1]
        f_ab = dot(rij, gw) / (d * d + EPS)
        keff = kap[i] * kap[j] / (kap[i] + kap[j])
        dTdt[i] += 4 * m[j] * keff * (temp[i] - temp[j]) * f_ab / (cp[i] * rho[i] * rho[j])
        c = ((m[i] / rho[i]) ** 2 + (m[j] / rho[j]) ** 2) / m[i] * dw / (d + EPS)
        eta_ij = 2 * eta[i] * eta[j] / (eta[i] + eta[j] + EPS)
        p_ij = (rho[j] * p[i] + rho[i] * p[j]) / (rho[i] + rho[j])
        si = dot([v[i][k] - u[i][k] for k in range(2)], rij)
        sj = dot([v[j][k] - u[j][k] for k in range(2)], rij)
        pi_ij = dot([u[j][k] - u[i][k] for k in range(2)], [-x for x in rij]) / (d + EPS) ** 2
        for k in range(2):
            a_r = 0.5 * (rho[i] * u[i][k] * si + rho[j] * u[j][k] * sj)
            dudt[i][k] += c * (-p_ij * rij[k] + a_r + eta_ij * (u[i][k] - u[j][k]))
            dudt[i][k] += (m[j] / rho[j]) * pi_ij * gw[k] * alpha * h * c_ref * rho0 / rho[i]

    f64 = torch.float64
    torch.testing.assert_close(out["drhodt"], torch.tensor(drho, dtype=f64), rtol=0,
                               atol=1e-11 * max(map(abs, drho)))
    torch.testing.assert_close(out["rho"], torch.tensor(rho, dtype=f64), rtol=1e-13, atol=0)
    torch.testing.assert_close(out["T"], torch.tensor(temp, dtype=f64), rtol=1e-15, atol=0)
    torch.testing.assert_close(out["dTdt"], torch.tensor(dTdt, dtype=f64), rtol=0,
                               atol=1e-12 * max(map(abs, dTdt)))
    scale = max(abs(x) for row in dudt for x in row)
    torch.testing.assert_close(out["dudt"], torch.tensor(dudt, dtype=f64), rtol=0,
                               atol=1e-11 * scale)
    # the diffusion term is really exercised
    assert max(map(abs, diff)) * c_ref * delta * h > 1e-3 * max(map(abs, drho))
