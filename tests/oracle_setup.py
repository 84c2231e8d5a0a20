"""Map a ``jaxsph_gb300.cases.CaseSetup`` onto the CPU oracle (test helper)."""

import torch

import oracle
from jaxsph_gb300 import _lib


def oracle_eos(setup):
    e = setup.eos
    if e.kind == _lib.EOS_RIEMANN:
        return oracle.sph.RIEMANNEoS(e.rho_ref, e.p_bg, e.u_ref)
    return oracle.sph.TaitEoS(e.p_ref, e.rho_ref, e.p_bg, e.gamma)


def oracle_g(setup):
    spec = setup.g_ext_fn.spec
    if spec["kind"] == _lib.GEXT_CONST:
        g = spec["g"]

        def f(r):
            res = torch.zeros_like(r)
            for d in range(r.shape[1]):
                res[:, d] = g[d]
            return res
        return f
    if spec["kind"] == _lib.GEXT_BAND_X:
        return _band(spec)
    if spec["kind"] == _lib.GEXT_REVERSE_X:
        return _reverse(spec)
    return oracle.sph.g_ext_zero


def _reverse(spec):
    # RPF._external_acceleration_fn (cases/rpf.py:58-63)
    y0 = spec["band"][1]
    g = spec["g"][0]

    def f(r):
        res = torch.zeros_like(r)
        res[:, 0] = torch.where(r[:, 1] > y0, -torch.ones_like(r[:, 0]), torch.ones_like(r[:, 0]))
        return res * g
    return f


def _band(spec):
    lo, hi = spec["band"]
    g = spec["g"][0]

    def f(r):
        res = torch.zeros_like(r)
        band = (r[:, 1] < hi) & (r[:, 1] > lo)
        res[:, 0] = torch.where(band, torch.ones_like(r[:, 0]), torch.zeros_like(r[:, 0]))
        return res * g
    return f


def oracle_bc(setup):
    spec = setup.bc_fn.spec
    k = spec["kind"]
    if k == _lib.BC_SOLID_ZERO:
        return oracle.sph.bc_solid_zero
    if k == _lib.BC_SOLID_ZERO_P:
        return lambda s: oracle.sph.bc_solid_zero(s, zero_p=True)
    if k == _lib.BC_LID:
        return oracle.sph.make_bc_ldc(spec["u_lid"][:setup.dim])
    if k == _lib.BC_HT:
        return oracle.sph.make_bc_ht(*spec["T"], *spec["x"])
    return oracle.sph.bc_identity


def oracle_case(setup, dtype=torch.float64, mask_self=False, state=None):
    s = setup.solver
    solver = oracle.sph.WCSPH(setup.box, oracle_eos(setup), oracle_g(setup), setup.dx, setup.dim,
                              setup.dt, setup.c_ref, eta_limiter=s["eta_limiter"],
                              solver=s["solver"], kernel=s["kernel"], h_fac=s["h_fac"],
                              is_bc_trick=s["is_bc_trick"], is_rho_evol=s["is_rho_evol"],
                              artificial_alpha=s["artificial_alpha"],
                              is_free_slip=s["is_free_slip"],
                              diff_alpha=s.get("diff_alpha", 0.01),
                              diff_delta=s.get("diff_delta", 0.1),
                              is_rho_renorm=s.get("is_rho_renorm", False),
                              is_heat_conduction=s.get("is_heat_conduction", False))
    fns = oracle.partition.NeighborListFns(setup.box, solver.kernel.cutoff, dtype,
                                           mask_self=mask_self)
    src = setup.state if state is None else state
    st = {k: (v.detach().cpu().to(dtype) if v.is_floating_point() else v.detach().cpu().long())
          for k, v in src.items()}
    return solver, fns, oracle_bc(setup), st


def oracle_nw_fn(setup):
    """The oracle's moving-wall normals for a case with a WallNormals nw_fn."""
    if setup.nw_fn is None:
        return None
    spec = setup.nw_fn.spec
    return oracle.sph.make_wall_normals(spec["layer"], spec["offset"][:setup.dim],
                                        spec["cutoff"], setup.box, setup.nw_fn.wall)


def oracle_rollout(setup, steps, dtype=torch.float64, state=None):
    solver, fns, bc, st = oracle_case(setup, dtype, state=state)
    nw_fn = oracle_nw_fn(setup)
    nb = fns.allocate(st["r"])
    for _ in range(steps):
        st_, nb_ = oracle.sph.si_euler_advance(setup.dt, setup.tvf, st, nb, fns, solver, bc,
                                               nw_fn)
        if nb_.did_buffer_overflow:  # simulate.py:120-128: re-allocate and redo the step
            nb = fns.allocate(st["r"])
            st, nb = oracle.sph.si_euler_advance(setup.dt, setup.tvf, st, nb, fns, solver, bc,
                                                 nw_fn)
        else:
            st, nb = st_, nb_
    return st
