"""Initial states of the four cases on the hot path (host-side, one-off).

Restates ``SimulationSetup.initialize`` (``jax_sph/case_setup.py:44-231``)
for Taylor-Green vortex (``cases/tgv.py``), dam break (``cases/db.py``),
lid-driven cavity (``cases/ldc.py``) and Poiseuille flow (``cases/pf.py``)
with their YAML defaults, so that synthetic inputs have exactly the
reference's shapes, particle order (walls first, lattice ``meshgrid`` order)
and float32 rounding. Each ``g_ext_fn``/``bc_fn`` is a callable that also
carries a ``spec`` the GPU engine evaluates inside its kernels.
"""

from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .eos import RIEMANNEoS, TaitEoS
from .space import periodic

EPS = 2.220446049250313e-16  # jnp.finfo(float).eps (case_setup.py:26)
FLUID, SOLID_WALL, MOVING_WALL, DIRICHLET_WALL = 0, 1, 2, 3  # utils.py:22-29


# ------------------------------------------------------------ lattices (utils.py:35-77)
def _grid(box, dx, dtype):
    n = np.array(np.round(np.asarray(box, dtype=np.float64) / dx), dtype=int)
    grid = np.meshgrid(*[np.arange(k) for k in n], indexing="xy")
    idx = np.vstack([g.ravel() for g in grid]).T
    if dtype == np.float32:
        return (idx.astype(np.float32) + np.float32(0.5)) * np.float32(dx)
    return (idx.astype(np.float64) + 0.5) * dx


def pos_init_cartesian_2d(box, dx, dtype=np.float32):
    """Particles at cell centres of a Cartesian grid, x fastest (utils.py:35-45)."""
    return _grid(box, dx, dtype)


def pos_init_cartesian_3d(box, dx, dtype=np.float32):
    """3D grid in ``meshgrid(..., indexing="xy")`` order (utils.py:48-53)."""
    return _grid(box, dx, dtype)


def _add(r, offset, dtype):
    return (r + np.asarray(offset, dtype=np.float64).astype(dtype)).astype(dtype)


def pos_box_2d(fluid_box, dx, n_walls=3, dtype=np.float32):
    """Wall layers around a 2D box: left, bottom, right, top (utils.py:56-77)."""
    dxn = n_walls * dx
    vertical = pos_init_cartesian_2d(np.array([dxn, fluid_box[1] + 2 * dxn]), dx, dtype)
    horiz = pos_init_cartesian_2d(np.array([fluid_box[0], dxn]), dx, dtype)
    wall_l = vertical.copy()
    wall_b = _add(horiz, [dxn, 0.0], dtype)
    wall_r = _add(vertical, [fluid_box[0] + dxn, 0.0], dtype)
    wall_t = _add(horiz, [dxn, fluid_box[1] + dxn], dtype)
    return np.concatenate([wall_l, wall_b, wall_r, wall_t])


# ------------------------------------------------------------ g_ext / bc descriptors
class GExt:
    """External acceleration ``g_ext_fn(r)`` with a GPU spec (kind, vector, band)."""

    def __init__(self, kind, g=(0.0, 0.0, 0.0), band=(0.0, 0.0)):
        self.spec = dict(kind=kind, g=tuple(float(x) for x in g), band=tuple(band))

    def __call__(self, r):
        res = torch.zeros_like(r)
        k, g, (lo, hi) = self.spec["kind"], self.spec["g"], self.spec["band"]
        if k == _lib.GEXT_CONST:
            for d in range(r.shape[1]):
                res[:, d] = g[d]
        elif k == _lib.GEXT_BAND_X:
            band = (r[:, 1] < hi) & (r[:, 1] > lo)
            res[:, 0] = torch.where(band, torch.full_like(r[:, 0], g[0]), torch.zeros_like(r[:, 0]))
        elif k == _lib.GEXT_REVERSE_X:
            res[:, 0] = torch.where(r[:, 1] > hi, torch.full_like(r[:, 0], -g[0]),
                                    torch.full_like(r[:, 0], g[0]))
        return res


class BC:
    """Boundary condition ``bc_fn(state)`` with a GPU spec (kind, lid velocity;
    heat transfer: reference / hot-wall temperature ``T`` and the inflow /
    outflow bounds ``x``)."""

    def __init__(self, kind, u_lid=(0.0, 0.0, 0.0), T=(0.0, 0.0), x=(0.0, 0.0)):
        self.spec = dict(kind=kind, u_lid=tuple(float(v) for v in u_lid),
                         T=tuple(float(v) for v in T), x=tuple(float(v) for v in x))

    def __call__(self, state):
        k = self.spec["kind"]
        if k == _lib.BC_NONE:
            return state
        if k == _lib.BC_HT:
            return self._heat_transfer(dict(state))
        st = dict(state)
        tag = st["tag"]
        solid = (tag == SOLID_WALL)[:, None]
        lid = (tag == MOVING_WALL)[:, None]
        for key in ("u", "v"):
            x = torch.where(solid, torch.zeros_like(st[key]), st[key])
            if k == _lib.BC_LID:
                ul = torch.as_tensor(self.spec["u_lid"][:x.shape[1]], dtype=x.dtype, device=x.device)
                x = torch.where(lid, ul.expand_as(x), x)
            st[key] = x
        for key in ("dudt", "dvdt"):
            m = solid | lid if k == _lib.BC_LID else solid
            st[key] = torch.where(m, torch.zeros_like(st[key]), st[key])
        if k == _lib.BC_SOLID_ZERO_P:
            st["p"] = torch.where(solid[:, 0], torch.zeros_like(st["p"]), st["p"])
        return st

    def _heat_transfer(self, st):
        # HT._boundary_conditions_fn (cases/ht.py:176-211)
        tag, x = st["tag"], st["r"][:, 0]
        (t_ref, t_hot), (x_in, x_out) = self.spec["T"], self.spec["x"]
        fluid = tag == FLUID
        hot, solid = tag == DIRICHLET_WALL, tag == SOLID_WALL
        if "T" in st:
            T, dT = st["T"], st["dTdt"]
            inflow = fluid & (x < x_in)
            for m, val in ((inflow, t_ref), (hot, t_hot), (solid, t_ref)):
                T = torch.where(m, torch.full_like(T, val), T)
                dT = torch.where(m, torch.zeros_like(dT), dT)
            dT = torch.where(fluid & (x > x_out), torch.zeros_like(dT), dT)
            st["T"], st["dTdt"] = T, dT
        static = (hot | solid)[:, None]
        for key in ("u", "v", "dudt", "dvdt"):
            st[key] = torch.where(static, torch.zeros_like(st[key]), st[key])
        return st


# ------------------------------------------------------------ setup container
@dataclass
class CaseSetup:
    """Everything ``SimulationSetup.initialize`` returns, plus solver settings."""

    name: str
    dim: int
    dx: float
    box: np.ndarray
    state: dict
    dt: float
    sequence_length: int
    c_ref: float
    p_ref: float
    p_bg: float
    u_ref: float
    viscosity: float
    eos: object
    g_ext_fn: GExt
    bc_fn: BC
    solver: dict = field(default_factory=dict)  # WCSPH keyword arguments
    tvf: float = 0.0
    nw_fn: object = None  # WallNormals when moving walls need recomputed normals

    @property
    def n(self):
        return int(self.state["r"].shape[0])

    def space(self):
        return periodic(self.box)

    def to(self, device):
        st = {k: v.to(device) for k, v in self.state.items()}
        return st

    def load_state0(self, path, keys=("r",)):
        """Take ``keys`` of the fluid particles from a saved .h5 state
        (``case.state0_path`` / ``case.state0_keys``, case_setup.py:184-194);
        every key restarts a run."""
        from .io_state import apply_state0

        apply_state0(self.state, path, keys, fluid_tag=FLUID)
        return self


def _finish(name, dim, dx, box, r, tag, v, *, rho_ref=1.0, viscosity=0.01, u_ref=1.0,
            c_ref_factor=10.0, gamma=1.0, p_bg_factor=0.0, g_ext_magnitude=0.0, cfl=0.25,
            dt=None, t_end=1.0, solver_name="SPH", kernel="QSK", h_fac=1.0, tvf=0.0,
            is_bc_trick=False, density_evolution=False, artificial_alpha=0.0,
            free_slip=False, eta_limiter=3, g_ext=None, bc=None, nw=None, dtype=np.float32,
            diff_alpha=0.01, diff_delta=0.1, rho_renorm=False, heat_conduction=False,
            T_ref=1.0, kappa_ref=0.0, Cp_ref=0.0, wall_layer=None):
    """The common part of ``initialize`` (case_setup.py:71-231)."""
    c_ref = c_ref_factor * u_ref
    p_ref = rho_ref * c_ref ** 2 / gamma
    p_bg = p_bg_factor * p_ref
    h = dx
    mass_ref = h ** dim * rho_ref
    dt_convective = cfl * h / (c_ref + u_ref)
    dt_viscous = cfl * h ** 2 * rho_ref / (viscosity + EPS)
    dt_body_force = cfl * (h / (g_ext_magnitude + EPS)) ** 0.5
    dt_cfl = float(np.amin([dt_convective, dt_viscous, dt_body_force]))
    dt = dt_cfl if dt is None else dt
    sequence_length = int(t_end / dt)
    if solver_name == "RIE":
        eos = RIEMANNEoS(rho_ref, p_bg, u_ref)
    else:
        eos = TaitEoS(p_ref, rho_ref, p_bg, gamma)
    n = r.shape[0]
    t = torch.float32 if dtype == np.float32 else torch.float64
    rho = torch.full((n,), rho_ref, dtype=t)
    state = {
        "r": torch.as_tensor(r, dtype=t),
        "tag": torch.as_tensor(tag, dtype=torch.int32),
        "u": torch.as_tensor(v, dtype=t),
        "v": torch.as_tensor(v, dtype=t),
        "dudt": torch.zeros((n, dim), dtype=t),
        "dvdt": torch.zeros((n, dim), dtype=t),
        "drhodt": torch.zeros((n,), dtype=t),
        "rho": rho,
        "p": eos.p_fn(rho),
        "mass": torch.full((n,), mass_ref, dtype=t),
        "eta": torch.full((n,), viscosity, dtype=t),
        "nw": torch.as_tensor(nw if nw is not None else np.zeros((n, dim)), dtype=t),
    }
    if heat_conduction:  # case_setup.py:298-306
        state.update(T=torch.full((n,), T_ref, dtype=t), dTdt=torch.zeros((n,), dtype=t),
                     kappa=torch.full((n,), kappa_ref, dtype=t),
                     Cp=torch.full((n,), Cp_ref, dtype=t))
    g_ext = g_ext or GExt(_lib.GEXT_ZERO)
    bc = bc or BC(_lib.BC_NONE)
    state = bc(state)  # case_setup.py:203
    solver = dict(solver=solver_name, kernel=kernel, h_fac=h_fac, is_bc_trick=is_bc_trick,
                  is_rho_evol=density_evolution, is_rho_renorm=rho_renorm,
                  is_heat_conduction=heat_conduction,
                  artificial_alpha=artificial_alpha,
                  is_free_slip=free_slip, eta_limiter=eta_limiter,
                  diff_alpha=diff_alpha, diff_delta=diff_delta)  # defaults.py:96-99
    setup = CaseSetup(name, dim, dx, np.asarray(box, dtype=np.float64), state, dt,
                      sequence_length, c_ref, p_ref, p_bg, u_ref, viscosity, eos, g_ext, bc,
                      solver, tvf)
    if wall_layer is not None and (tag == MOVING_WALL).any() and (
            (solver_name == "RIE" or free_slip) and is_bc_trick):
        # case_setup.py:209-218: moving walls recompute their normals each step
        setup.nw_fn = WallNormals(*wall_layer, box=box, wall=np.isin(
            tag, [SOLID_WALL, MOVING_WALL, DIRICHLET_WALL]))
    return setup


# ------------------------------------------------------------ cases
def tgv(dim=2, dx=None, viscosity=None, solver_name="SPH", tvf=None, kernel=None,
        dtype=np.float32, t_end=5.0, **kw):
    """Taylor-Green vortex (cases/tgv.py, cases/tgv.yaml).

    2D: unit box, u = -cos(2 pi x) sin(2 pi y), v = sin(2 pi x) cos(2 pi y).
    3D: box (2 pi)^3, u = sin x cos y cos z, v = -cos x sin y cos z, w = 0.
    """
    if dim == 2:
        dx = 0.02 if dx is None else dx
        box = np.array([1.0, 1.0])
        r = pos_init_cartesian_2d(box, dx, dtype)
        x, y = r[:, 0].astype(np.float64), r[:, 1].astype(np.float64)
        v = np.stack([-np.cos(2 * np.pi * x) * np.sin(2 * np.pi * y),
                      np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)], 1)
        viscosity = 0.01 if viscosity is None else viscosity
        kernel = kernel or "QSK"
        tvf = 0.0 if tvf is None else tvf
    else:
        box = 2 * np.pi * np.array([1.0, 1.0, 1.0])
        dx = 2 * np.pi / 64 if dx is None else dx
        r = pos_init_cartesian_3d(box, dx, dtype)
        x, y, z = (r[:, k].astype(np.float64) for k in range(3))
        v = np.stack([np.sin(x) * np.cos(y) * np.cos(z), -np.cos(x) * np.sin(y) * np.cos(z),
                      np.zeros_like(x)], 1)
        viscosity = 1.0 / 1600.0 if viscosity is None else viscosity
        kernel = kernel or "WC2K"
        tvf = 1.0 if tvf is None else tvf
    tag = np.full(r.shape[0], FLUID)
    kw.setdefault("density_evolution", solver_name == "RIE")
    return _finish(f"tgv{dim}d", dim, dx, box, r, tag, v, viscosity=viscosity,
                   solver_name=solver_name, kernel=kernel, tvf=tvf, t_end=t_end, dtype=dtype,
                   **kw)


class WallNormals:
    """The integrator's ``nw_fn`` for moving walls (compute_nws_jax_wrapper,
    utils.py:197-275) with a GPU spec: every wall particle's normal is the
    normalised displacement from ``r - offset`` to its nearest point of a
    static wall layer discretised 5x finer, searched within ``cutoff``
    (layer point 0 never counts, as in the reference; ties go to the lowest
    index); fluid normals are zero."""

    def __init__(self, layer, offset, cutoff, box, wall):
        self.spec = dict(layer=np.ascontiguousarray(layer, dtype=np.float32),
                         offset=tuple(float(x) for x in offset), cutoff=float(cutoff))
        self.box = np.asarray(box, dtype=np.float64)
        self.wall = np.asarray(wall, dtype=bool)

    def __call__(self, r):
        from .space import periodic

        disp, _ = periodic(self.box)
        wall = torch.as_tensor(self.wall, device=r.device)
        off = torch.as_tensor(self.spec["offset"][:r.shape[1]], dtype=torch.float32,
                              device=r.device)
        layer = torch.as_tensor(self.spec["layer"], device=r.device)
        p = r[wall].float() - off
        d_in = disp(p[:, None, :], layer[None, :, :])  # membership: metric(wall, layer)
        ok = (d_in * d_in).sum(-1) < np.float32(self.spec["cutoff"] ** 2)
        ok[:, 0] = False
        dr = disp(layer[None, :, :], p[:, None, :])
        dist = torch.sqrt((dr * dr).sum(-1))
        dist = torch.where(ok, dist, torch.full_like(dist, float("inf")))
        k = torch.argmin(dist, dim=1)  # the first of equally near points
        rows = torch.arange(p.shape[0], device=r.device)
        best = dist[rows, k]
        nw_w = dr[rows, k] / (best[:, None] + EPS)
        nw_w = torch.where(torch.isfinite(best)[:, None], nw_w, torch.zeros_like(nw_w))
        nw = torch.zeros_like(r, dtype=torch.float32)
        nw[wall] = nw_w
        return nw


def _wall_layer(dx, n_walls, offset_vec, wall_part_fn, dtype):
    """The fine layer of compute_nws (utils.py:214-217), in float32 like the
    reference, with the offset and the search radius."""
    off = np.asarray(offset_vec, dtype=np.float64)
    layer = (wall_part_fn(dx / 5, 1).astype(dtype) - (off / n_walls / 5).astype(dtype))
    return layer.astype(dtype), off.astype(dtype), dx * n_walls * 2.0 ** 0.5 * 1.01


def _nws_scipy(r, tag, dx, n_walls, offset_vec, wall_part_fn, dtype):
    """Wall normals by nearest point of a 5x finer wall layer (utils.py:169-194)."""
    from scipy.spatial import KDTree

    wall = np.isin(tag, [SOLID_WALL, MOVING_WALL, DIRICHLET_WALL])
    r_aligned = r[wall].astype(np.float64) - offset_vec
    layer = wall_part_fn(dx / 5, 1).astype(np.float64) - offset_vec / n_walls / 5
    dist, match = KDTree(layer).query(r_aligned, k=1)
    dr = layer[match] - r_aligned
    nw = np.zeros(r.shape, dtype=np.float64)
    nw[wall] = dr / (dist[:, None] + EPS)
    return nw.astype(dtype)


def dam_break(dx=0.005, n_walls=3, dtype=np.float32, t_end=12.0, dt=None, **kw):
    """2D dam break with Riemann SPH (cases/db.py, cases/db.yaml).

    Tank 5.366 x 2.0 with 3 wall layers, water column 2 x 1, box offset 0.1.
    ``dt`` defaults to the CFL step (db.yaml's 3e-4 violates CFL at dx=0.005).
    """
    L_wall, H_wall, L, H, box_offset = 5.366, 2.0, 2.0, 1.0, 0.1
    g = 1.0
    u_ref = 1.4142135623730951
    box = np.array([L_wall + 2 * n_walls * dx + box_offset, H_wall + 2 * n_walls * dx + box_offset])
    r_f = (pos_init_cartesian_2d(np.array([L, H]), dx, dtype) + dtype(n_walls * dx)).astype(dtype)

    def walls(ddx, nw_):
        return pos_box_2d(np.array([L_wall, H_wall]), ddx, nw_, dtype)

    r_w = walls(dx, n_walls)
    r = np.concatenate([r_w, r_f])
    tag = np.concatenate([np.full(len(r_w), SOLID_WALL), np.full(len(r_f), FLUID)])
    offset_vec = np.ones(2) * n_walls * dx
    nw = _nws_scipy(r, tag, dx, n_walls, offset_vec, walls, dtype)
    v = np.zeros_like(r, dtype=np.float64)
    # db.yaml's settings; keywords override them (e.g. the delta-SPH validation
    # run of validation/db2d.sh: solver_name="DELTA", gamma=7, u_ref=1.95,
    # viscosity=0, free_slip=True, artificial_alpha=0)
    opts = dict(viscosity=0.00005, u_ref=u_ref, solver_name="RIE", kernel="QSK",
                is_bc_trick=True, density_evolution=True, artificial_alpha=0.1)
    opts.update(kw)
    return _finish("db", 2, dx, box, r, tag, v, g_ext_magnitude=g, t_end=t_end, dt=dt,
                   g_ext=GExt(_lib.GEXT_CONST, (0.0, -g, 0.0)), bc=BC(_lib.BC_SOLID_ZERO_P),
                   nw=nw, dtype=dtype, **opts)


def lid_driven_cavity(dx=0.02, n_walls=3, viscosity=0.01, u_lid=1.0, dtype=np.float32,
                      t_end=5.0, dt=None, **kw):
    """2D lid-driven cavity (cases/ldc.py, cases/ldc.yaml): SPH with the wall BC."""
    box = np.ones(2) + 2 * n_walls * dx
    r_f = (pos_init_cartesian_2d(np.ones(2), dx, dtype) + dtype(n_walls * dx)).astype(dtype)
    r_w = pos_box_2d(np.ones(2), dx, n_walls, dtype)
    r = np.concatenate([r_w, r_f])
    tag = np.concatenate([np.full(len(r_w), SOLID_WALL), np.full(len(r_f), FLUID)])
    tag = np.where(r[:, 1].astype(np.float64) > box[1] - n_walls * dx, MOVING_WALL, tag)
    v = np.zeros_like(r, dtype=np.float64)

    def walls(ddx, nw_):  # LDC._init_walls_2d (cases/ldc.py:49-51)
        return pos_box_2d(np.ones(2), ddx, nw_, dtype)

    offset_vec = np.ones(2) * n_walls * dx  # LDC._offset_vec (cases/ldc.py:103-108)
    nw = None
    if kw.get("solver_name") == "RIE" or kw.get("free_slip"):
        nw = _nws_scipy(r, tag, dx, n_walls, offset_vec, walls, dtype)
    return _finish("ldc", 2, dx, box, r, tag, v, viscosity=viscosity, p_bg_factor=0.01,
                   is_bc_trick=True, t_end=t_end, dt=dt,
                   bc=BC(_lib.BC_LID, (u_lid, 0.0, 0.0)), nw=nw, dtype=dtype,
                   wall_layer=_wall_layer(dx, n_walls, offset_vec, walls, dtype), **kw)


def poiseuille(dx=0.0166666, n_walls=3, viscosity=100.0, u_ref=1.25, g_ext_magnitude=1000.0,
               dtype=np.float32, t_end=0.01, dt=None, **kw):
    """2D Poiseuille flow (cases/pf.py, cases/pf.yaml): channel L=0.4, H=1, body force."""
    L, H = 0.4, 1.0
    dxn = n_walls * dx
    box = np.array([L, H + 2 * dxn])
    r_f = _add(pos_init_cartesian_2d(np.array([L, H]), dx, dtype), [0.0, dxn], dtype)

    def walls(ddx, nw_):  # PF._init_walls_2d (cases/pf.py:43-57)
        hz = pos_init_cartesian_2d(np.array([L, ddx * nw_]), ddx, dtype)
        return np.concatenate([hz, _add(hz, [0.0, H + ddx * nw_], dtype)])

    r_w = walls(dx, n_walls)
    r = np.concatenate([r_w, r_f])
    tag = np.concatenate([np.full(len(r_w), SOLID_WALL), np.full(len(r_f), FLUID)])
    v = np.zeros_like(r, dtype=np.float64)
    nw = None
    if kw.get("solver_name") == "RIE" or kw.get("free_slip"):
        nw = _nws_scipy(r, tag, dx, n_walls, np.array([0.0, dxn]), walls, dtype)
    g = GExt(_lib.GEXT_BAND_X, (g_ext_magnitude, 0.0, 0.0), (dxn, box[1] - dxn))
    return _finish("pf", 2, dx, box, r, tag, v, viscosity=viscosity, u_ref=u_ref,
                   g_ext_magnitude=g_ext_magnitude, is_bc_trick=True, t_end=t_end, dt=dt,
                   g_ext=g, bc=BC(_lib.BC_SOLID_ZERO), nw=nw, dtype=dtype, **kw)


def heat_transfer(dx=0.02, n_walls=3, dtype=np.float32, t_end=1.5, dt=None,
                  r0_noise_factor=0.05, seed=0, hot_wall_temperature=1.23,
                  hot_wall_half_width=0.25, **kw):
    """2D heat transfer over a flat plate (cases/ht.py, cases/ht.yaml).

    A fluid layer L=1 x H=0.2 between two 3-layer walls, periodic along x,
    driven by a body force on the fluid band; the bottom wall within
    hot_wall_half_width of the middle is a hot Dirichlet wall. Fluid
    positions get Gaussian noise of r0_noise_factor*dx (seeded here; the
    reference draws it from its JAX key), wrapped into the box.
    """
    L, H = 1.0, 0.2
    dxn = n_walls * dx
    box = np.array([L, H + 2 * dxn])
    r_f = _add(pos_init_cartesian_2d(np.array([L, H]), dx, dtype), [0.0, dxn], dtype)

    def walls(ddx, nw_):  # HT._init_walls_2d (cases/ht.py:40-54)
        hz = pos_init_cartesian_2d(np.array([L, ddx * nw_]), ddx, dtype)
        return np.concatenate([hz, _add(hz, [0.0, H + ddx * nw_], dtype)])

    r_w = walls(dx, n_walls)
    r = np.concatenate([r_w, r_f])
    tag = np.concatenate([np.full(len(r_w), SOLID_WALL), np.full(len(r_f), FLUID)])
    x, y = r[:, 0].astype(np.float64), r[:, 1].astype(np.float64)
    hot = (y < dxn) & (x < L / 2 + hot_wall_half_width) & (x > L / 2 - hot_wall_half_width)
    tag = np.where(hot, DIRICHLET_WALL, tag)
    if r0_noise_factor:
        # case_setup.py:138-144: noise on the fluid, then the periodic shift
        rng = np.random.default_rng(seed)
        noise = rng.normal(0.0, r0_noise_factor * dx, r.shape) * (tag == FLUID)[:, None]
        r = np.mod(r.astype(np.float64) + noise, box).astype(dtype)
    v = np.zeros_like(r, dtype=np.float64)
    nw = None
    if kw.get("solver_name") == "RIE" or kw.get("free_slip"):
        nw = _nws_scipy(r, tag, dx, n_walls, np.array([0.0, dxn]), walls, dtype)
    g_mag = 2.3
    g = GExt(_lib.GEXT_BAND_X, (g_mag, 0.0, 0.0), (dxn, box[1] - dxn))
    bc = BC(_lib.BC_HT, T=(1.0, hot_wall_temperature), x=(dxn, L - dxn))
    opts = dict(g_ext_magnitude=g_mag, is_bc_trick=True, p_bg_factor=0.05,
                heat_conduction=True, T_ref=1.0, kappa_ref=7.313, Cp_ref=305.27)
    opts.update(kw)
    return _finish("ht", 2, dx, box, r, tag, v, t_end=t_end, dt=dt, g_ext=g, bc=bc, nw=nw,
                   dtype=dtype, **opts)


def couette(dx=0.0166666, n_walls=3, viscosity=100.0, u_ref=1.25, u_x_wall=1.25,
            dtype=np.float32, t_end=0.01, dt=None, **kw):
    """2D Couette flow (cases/cf.py, cases/cf.yaml): the Poiseuille channel
    L=0.4, H=1 without body force, its top wall moving at u_x_wall."""
    L, H = 0.4, 1.0
    dxn = n_walls * dx
    box = np.array([L, H + 2 * dxn])
    r_f = _add(pos_init_cartesian_2d(np.array([L, H]), dx, dtype), [0.0, dxn], dtype)

    def walls(ddx, nw_):  # CF._init_walls_2d (cases/cf.py:50-63)
        hz = pos_init_cartesian_2d(np.array([L, ddx * nw_]), ddx, dtype)
        return np.concatenate([hz, _add(hz, [0.0, H + ddx * nw_], dtype)])

    r_w = walls(dx, n_walls)
    r = np.concatenate([r_w, r_f])
    tag = np.concatenate([np.full(len(r_w), SOLID_WALL), np.full(len(r_f), FLUID)])
    # the top wall moves (cases/cf.py:101-104)
    tag = np.where(r[:, 1].astype(np.float64) > box[1] - n_walls * dx, MOVING_WALL, tag)
    v = np.zeros_like(r, dtype=np.float64)
    nw = None
    if kw.get("solver_name") == "RIE" or kw.get("free_slip"):
        nw = _nws_scipy(r, tag, dx, n_walls, np.array([0.0, dxn]), walls, dtype)
    # walls at rest, the moving wall at u_wall, no wall acceleration
    # (cases/cf.py:156-171): the lid boundary condition
    return _finish("cf", 2, dx, box, r, tag, v, viscosity=viscosity, u_ref=u_ref,
                   is_bc_trick=True, t_end=t_end, dt=dt,
                   bc=BC(_lib.BC_LID, (u_x_wall, 0.0, 0.0)), nw=nw, dtype=dtype,
                   wall_layer=_wall_layer(dx, n_walls, np.array([0.0, dxn]), walls, dtype),
                   **kw)


def cube_of_water(dx=0.05, n_walls=3, dtype=np.float32, t_end=1.0, dt=None, **kw):
    """2D cube of water falling in a walled box (cases/cw.py, cases/cw.yaml): SPH with
    the generalized wall BC and density evolution, gravity -1 in y, the fluid's
    initial velocity (0, -0.5)."""
    L_wall, H_wall, L, H = 1.0, 1.0, 0.3, 0.3
    cube_offset = np.array([0.5, 0.5])
    dxn = n_walls * dx
    box = np.array([L_wall, H_wall]) + 2 * dxn
    r_w = pos_box_2d(np.array([L_wall, H_wall]), dx, n_walls, dtype)
    r_f = _add(pos_init_cartesian_2d(np.array([L, H]), dx, dtype), dxn + cube_offset, dtype)
    r = np.concatenate([r_w, r_f])
    tag = np.concatenate([np.full(len(r_w), SOLID_WALL), np.full(len(r_f), FLUID)])
    # CW._init_velocity2D: every particle u_init; bc_fn then zeroes the walls
    v = np.tile(np.array([0.0, -0.5]), (len(r), 1))
    g = 1.0
    opts = dict(is_bc_trick=True, density_evolution=True)
    opts.update(kw)
    return _finish("cw", 2, dx, box, r, tag, v, g_ext_magnitude=g, t_end=t_end, dt=dt,
                   g_ext=GExt(_lib.GEXT_CONST, (0.0, -g, 0.0)), bc=BC(_lib.BC_SOLID_ZERO_P),
                   dtype=dtype, **opts)


def reverse_poiseuille(dim=2, dx=0.025, dtype=np.float32, t_end=100.0, dt=0.0005, **kw):
    """Reverse Poiseuille flow (cases/rpf.py, cases/rpf.yaml): a periodic box
    [1, 2] (3D: [1, 2, 0.5]) filled with fluid at rest, body force +1 in x
    below y = 1 and -1 above; viscosity 0.1, background pressure 0.05 p_ref."""
    box = np.array([1.0, 2.0]) if dim == 2 else np.array([1.0, 2.0, 0.5])
    r = _grid(box, dx, dtype)
    tag = np.full(len(r), FLUID)
    v = np.zeros_like(r, dtype=np.float64)
    g = 1.0
    opts = dict(viscosity=0.1, p_bg_factor=0.05)
    opts.update(kw)
    return _finish("rpf", dim, dx, box, r, tag, v, g_ext_magnitude=g, t_end=t_end, dt=dt,
                   g_ext=GExt(_lib.GEXT_REVERSE_X, (g, 0.0, 0.0), (1.0, 1.0)),
                   dtype=dtype, **opts)


def unit_cube(dim=2, dx=0.02, dtype=np.float32, t_end=1.0, dt=None, **kw):
    """The reference's unit-test case (cases/ut.py, cases/ut.yaml): a cube of
    water (0.5 on a side) falling under gravity -1 in y through a periodic box
    1 on a side, SPH with density evolution, no walls."""
    L_wall, L, H = 1.0, 0.5, 0.5
    cube_offset = np.full(dim, 0.25)
    box = np.full(dim, L_wall)
    cube = np.array([L, H]) if dim == 2 else np.array([L, L, H])
    r = _add(_grid(cube, dx, dtype), cube_offset, dtype)
    tag = np.full(len(r), FLUID)
    v = np.zeros_like(r, dtype=np.float64)
    g = 1.0
    gv = (0.0, -g, 0.0)
    opts = dict(density_evolution=True)
    opts.update(kw)
    return _finish("ut", dim, dx, box, r, tag, v, g_ext_magnitude=g, t_end=t_end, dt=dt,
                   g_ext=GExt(_lib.GEXT_CONST, gv), dtype=dtype, **opts)


def fourier_perturbation(r, sigma=0.1, kmax=8, seed=1):
    """Divergence-free random velocity field on the periodic unit square.

    Stream function psi = sum over integer wave vectors 0 < |k| <= kmax of
    Gaussian coefficients times cos/sin(2 pi k.x); u = (d psi/dy, -d psi/dx),
    scaled to an RMS speed of ``sigma`` over the given points.
    """
    rng = np.random.default_rng(seed)
    x = np.asarray(r, dtype=np.float64)
    u = np.zeros_like(x)
    for kx in range(-kmax, kmax + 1):
        for ky in range(0, kmax + 1):
            if (kx, ky) == (0, 0) or kx * kx + ky * ky > kmax * kmax:
                continue
            if ky == 0 and kx < 0:
                continue
            a, b = rng.normal(size=2)
            ph = 2 * np.pi * (kx * x[:, 0] + ky * x[:, 1])
            dpsi = 2 * np.pi * (-a * np.sin(ph) + b * np.cos(ph))  # d psi / d phase
            u[:, 0] += dpsi * ky
            u[:, 1] -= dpsi * kx
    rms = np.sqrt((u ** 2).sum(1).mean())
    return u * (sigma / rms)


def tgv_perturbed(n_side=128, sigma=0.1, kmax=8, seed=1, dtype=np.float32, **kw):
    """2D periodic TGV (SPH, tvf = 0, QSK) whose initial velocity is the TGV field
    plus a seeded divergence-free random Fourier perturbation: the workload of
    the differentiable form (inverse problems on initial velocities)."""
    s = tgv(dim=2, dx=1.0 / n_side, dtype=dtype, **kw)
    r = s.state["r"].numpy()
    pert = fourier_perturbation(r, sigma, kmax, seed)
    u = s.state["u"].double().numpy() + pert
    t = s.state["u"].dtype
    s.state["u"] = torch.as_tensor(u, dtype=t)
    s.state["v"] = s.state["u"].clone()
    s.name = f"tgv2d_perturbed_seed{seed}"
    return s


def cavity_channel_batch(n_instances=256, seed=0, n_min=1000, n_max=40000, re_min=10.0,
                         re_max=1000.0, dx_min=0.004, dx_max=0.02, dtype=np.float32, t_end=1.0):
    """Independent lid-driven cavities and Poiseuille channels for the batched form.

    Instances alternate LDC / PF. Fluid particle counts are drawn log-uniform
    in [n_min, n_max] and set the lattice spacing (cavity: (1/dx)^2 fluid
    particles, channel: 0.4/dx^2), clamped to [dx_min, dx_max]; Reynolds
    numbers are uniform in [re_min, re_max]. Cavity: eta = u_lid/Re (lid
    speed 1, side 1). Channel: u_max = 1.25, eta = u_max/Re and the Morris
    body force g = 8 eta u_max / H^2 (H = 1). Every instance uses its own CFL
    time step; all share the SPH solver, QSK kernel and the wall BC.
    """
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_instances):
        n_target = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        re = float(rng.uniform(re_min, re_max))
        if k % 2 == 0:
            dx = float(np.clip(1.0 / np.sqrt(n_target), dx_min, dx_max))
            out.append(lid_driven_cavity(dx=dx, viscosity=1.0 / re, dtype=dtype, t_end=t_end))
        else:
            dx = float(np.clip(np.sqrt(0.4 / n_target), dx_min, dx_max))
            u_max = 1.25
            eta = u_max / re
            out.append(poiseuille(dx=dx, viscosity=eta, u_ref=u_max,
                                  g_ext_magnitude=8.0 * eta * u_max, dtype=dtype, t_end=t_end))
    return out


CASES = {"tgv": tgv, "db": dam_break, "ldc": lid_driven_cavity, "pf": poiseuille}
