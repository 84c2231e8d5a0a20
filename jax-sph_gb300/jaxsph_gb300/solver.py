"""WCSPH forward pass: drop-in for ``jax_sph.solver.WCSPH`` (solver.py:613-951).

``WCSPH(...).forward_wrapper()`` returns ``forward(state, neighbors) -> state``
with the reference's state-dict contract. The computation runs in
``libsph_gb300`` (density passes, generalized wall BC pass, heat pass, force
pass; see ``csrc/sph_forward.cu`` and ``csrc/sph_delta.cu``) in float32 on the
GPU. The branches on the hot path are the SPH, Riemann and delta-SPH solvers
with density summation or evolution (continuity, Riemann, Marrone's delta-SPH)
and renormalisation, the generalized wall boundary condition (no-slip and
free-slip) with the wall temperature, heat conduction, transport velocity and
artificial viscosity, over the quintic and Wendland C2 kernels.
"""

import numpy as np
import torch

from . import _lib
from .kernel import make_kernel

STATE_KEYS = ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "mass", "eta", "nw")
HEAT_KEYS = ("T", "dTdt", "kappa", "Cp")  # with heat conduction (case_setup.py:164-181)
_VEC = ("r", "u", "v", "dudt", "dvdt", "nw")


def prepare_state(state, dim, device="cuda", heat=False):
    """Contiguous float32 / int32 CUDA copies of the fields the kernels read."""
    n = int(state["r"].shape[0])
    out = {}
    for k in STATE_KEYS + (HEAT_KEYS if heat else ()):
        x = state.get(k)
        if x is None:
            if k == "nw":
                continue
            if k in ("drhodt", "dTdt"):
                x = torch.zeros(n)
            else:
                raise KeyError(f"state is missing '{k}'")
        t = torch.as_tensor(x)
        want = torch.int32 if k == "tag" else torch.float32
        t = t.to(device=device, dtype=want).contiguous()
        if k in _VEC and (t.ndim != 2 or t.shape[1] != dim):
            raise ValueError(f"state['{k}'] must have shape (N, {dim})")
        out[k] = t
    return out


OUT_KEYS = ("r", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p")
OUT_KEYS_SUMMATION = ("r", "u", "v", "dudt", "dvdt", "rho", "p")
HEAT_OUT_KEYS = ("T", "dTdt")


def empty_outputs(st, heat=False):
    return {k: torch.empty_like(st[k]) for k in OUT_KEYS + (HEAT_OUT_KEYS if heat else ())}


def host_state(state, dim, need_nw, heat=False):
    """The state's own tensors when every field is a contiguous host tensor of
    the kernels' dtype (float32, int32 tags) and shape; else None. (Whether
    they are pinned the library checks itself, before any work.)"""
    out = {}
    for k in STATE_KEYS + (HEAT_KEYS if heat else ()):
        t = state.get(k)
        if t is None:
            if k == "nw" and not need_nw:
                continue
            return None
        if not isinstance(t, torch.Tensor) or t.device.type != "cpu":
            return None
        if t.dtype != (torch.int32 if k == "tag" else torch.float32) or not t.is_contiguous():
            return None
        if k in _VEC and (t.ndim != 2 or t.shape[1] != dim):
            return None
        out[k] = t
    return out


class WCSPH:
    """Weakly compressible SPH solver with transport velocity formulation."""

    def __init__(self, displacement_fn, eos, g_ext_fn, dx, dim, dt, c_ref, eta_limiter=3,
                 diff_delta=0.02, diff_alpha=0.1, solver="SPH", kernel="QSK", h_fac=1.0,
                 is_bc_trick=False, is_rho_evol=False, artificial_alpha=0.0,
                 is_free_slip=False, is_rho_renorm=False, is_heat_conduction=False,
                 kahan=False):
        if solver not in _lib.SOLVERS:
            raise NotImplementedError(
                f"solver {solver!r}: the GPU hot path implements SPH, RIE and DELTA")
        self.displacement_fn = displacement_fn
        self.eos = eos
        self.g_ext_fn = g_ext_fn
        self.dx, self.dim, self.dt, self.c_ref = float(dx), int(dim), float(dt), float(c_ref)
        self.eta_limiter = float(eta_limiter)
        self.diff_delta, self.diff_alpha = float(diff_delta), float(diff_alpha)
        self.solver = solver
        self.kernel = kernel
        self._kernel_fn = make_kernel(kernel, h_fac * dx, dim)
        self.is_bc_trick = bool(is_bc_trick)
        self.is_rho_evol = bool(is_rho_evol)
        self.is_rho_renorm = bool(is_rho_renorm)
        self.is_heat_conduction = bool(is_heat_conduction)
        self.artificial_alpha = float(artificial_alpha)
        self.is_free_slip = bool(is_free_slip)
        self.kahan = bool(kahan)
        self._engines = {}
        self._step_cases = {}
        self._last_host = None

    # ---------------------------------------------------------------- engine
    def solver_flags(self):
        return dict(kernel=_lib.KERNELS[self.kernel], solver=_lib.SOLVERS[self.solver],
                    is_rho_evol=self.is_rho_evol, is_rho_renorm=self.is_rho_renorm,
                    is_heat_conduction=self.is_heat_conduction, is_bc_trick=self.is_bc_trick,
                    is_free_slip=self.is_free_slip, kahan=self.kahan)

    def g_spec(self):
        spec = getattr(self.g_ext_fn, "spec", None)
        if spec is None:
            return dict(kind=_lib.GEXT_ARRAY, g=(0.0, 0.0, 0.0), band=(0.0, 0.0))
        return spec

    def sph_case(self, nl_fns, n, dt=0.0, tvf=0.0, bc=None):
        s = nl_fns.case(n)
        s.dx = self.dx
        s.h = self._kernel_fn.h
        s.dt = float(dt)
        s.dt_solver = self.dt
        s.tvf = float(tvf)
        s.c_ref = self.c_ref
        s.eos = self.eos.kind
        s.p_ref = float(self.eos.p_ref)
        s.rho_ref = float(self.eos.rho_ref)
        s.p_bg = float(self.eos.p_bg)
        s.gamma = float(self.eos.gamma)
        s.u_ref = float(self.eos.u_ref)
        s.eta_limiter = self.eta_limiter
        s.artificial_alpha = self.artificial_alpha
        s.diff_alpha = self.diff_alpha
        s.diff_delta = self.diff_delta
        g = self.g_spec()
        s.g_kind = g["kind"]
        for d in range(3):
            s.g[d] = g["g"][d]
        s.g_band_lo, s.g_band_hi = g["band"]
        bc = bc or dict(kind=_lib.BC_NONE, u_lid=(0.0, 0.0, 0.0))
        s.bc_kind = bc["kind"]
        for d in range(3):
            s.u_lid[d] = bc["u_lid"][d]
        for k in range(2):
            s.bc_T[k] = bc.get("T", (0.0, 0.0))[k]
            s.bc_x[k] = bc.get("x", (0.0, 0.0))[k]
        return s

    def engine(self, nl_fns, case):
        key = (id(nl_fns), int(case.n))
        e = self._engines.get(key)
        if e is None:
            if abs(nl_fns.r_cutoff - self._kernel_fn.cutoff) > 1e-12 * max(1.0, nl_fns.r_cutoff):
                raise ValueError("neighbour-list cutoff differs from the kernel cutoff")
            # a skin lets consecutive drop-in steps keep their candidate lists
            # (the neighbour set of every step is exact either way)
            e = _lib.Engine(nl_fns.config(**self.solver_flags(), verlet_skin=0.1), [case])
            self._engines = {key: e}
        elif e.cases[0] is not case and bytes(e.cases[0]) != bytes(case):
            e.update_cases([case])
        return e

    @staticmethod
    def _wall_layer(e, nw_fn):
        """Give the engine the moving walls' layer once (it keeps it)."""
        if getattr(e, "_nw_fn", None) is not nw_fn:
            spec = nw_fn.spec
            e.set_wall_layer(spec["layer"], spec["offset"], spec["cutoff"])
            e._nw_fn = nw_fn

    def _load(self, state, neighbors, case, load=True):
        nl_fns = neighbors._fns
        st = prepare_state(state, self.dim, heat=self.is_heat_conduction)
        if self.g_spec()["kind"] == _lib.GEXT_ARRAY:
            st["g_ext"] = torch.as_tensor(self.g_ext_fn(st["r"])).to(
                device=st["r"].device, dtype=torch.float32).contiguous()
        if (self.solver == "RIE" or self.is_free_slip) and "nw" not in st:
            st["nw"] = torch.zeros_like(st["r"])
        e = self.engine(nl_fns, case)
        if load:
            e.set_state(st)
        cap = neighbors.cell_list_capacity
        e.nl_set_capacity(cap if cap is not None else 2 ** 31 - 1, neighbors.max_occupancy)
        return e, st

    @staticmethod
    def _result(state, out):
        res = dict(state)
        for k, v in out.items():
            res[k] = v
        for k in ("tag", "mass", "eta"):
            res[k] = state[k]
        return res

    # ---------------------------------------------------------------- API
    def forward_wrapper(self):
        """``forward(state, neighbors) -> state`` (solver.py:702-951)."""

        def forward(state, neighbors):
            nl_fns = neighbors._fns
            r = torch.as_tensor(state["r"])
            ref = torch.as_tensor(neighbors.reference_position).to(r.device, r.dtype)
            if nl_fns.dr_threshold == 0.0 and not torch.equal(r, ref):
                raise NotImplementedError(
                    "forward with a neighbour list built on other positions: update the list first")
            case = self.sph_case(nl_fns, r.shape[0])
            e, st = self._load(state, neighbors, case)
            e.forward()
            out = empty_outputs(st, self.is_heat_conduction)
            e.get_state(out)
            return self._result(state, out)

        forward.__wcsph__ = self
        return forward

    def advance(self, dt, tvf, state, neighbors, bc_fn, nw_fn=None):
        """One fused si_euler step on the GPU (integrator.py:22-56).

        A state of pinned (page-locked) host tensors is copied to the GPU and
        its result back inside the one library call (DMA, one copy per
        field), and the call returns once the result is in host memory. Any
        other state goes to the GPU first and stays there.
        """
        nl_fns = neighbors._fns
        bc_spec = getattr(bc_fn, "spec", None)
        # the step's parameters, built once per (list, size, dt, tvf, bc)
        key = (id(nl_fns), int(state["r"].shape[0]), float(dt), float(tvf), id(bc_spec))
        hit = self._step_cases.get(key)
        case = hit[0] if hit else None
        if case is None:
            if self.g_spec()["kind"] == _lib.GEXT_ARRAY:
                raise NotImplementedError(
                    "si_euler needs a g_ext_fn with a GPU spec (e.g. jaxsph_gb300.cases.GExt)")
            case = self.sph_case(nl_fns, key[1], dt=dt, tvf=tvf, bc=bc_spec)
            if len(self._step_cases) > 16:
                self._step_cases.clear()
            # the entry holds the list functions and the bc spec, so their ids
            # in the key cannot be reused by other objects
            self._step_cases[key] = (case, nl_fns, bc_spec)
        # the state returned by the last host-buffer step, passed back as it was:
        # its fields are known to be valid and its view is already built
        last = self._last_host
        vin = None
        eng = self.engine(nl_fns, case)
        if (last is not None and last[0] is state and last[3] is eng
                and all(state.get(k) is t for k, t in last[1].items())):
            st, vin = last[1], last[2]
        else:
            st = host_state(state, self.dim, self.solver == "RIE" or self.is_free_slip,
                            self.is_heat_conduction)
        self._last_host = None
        thr = nl_fns.threshold_sq
        ref = torch.as_tensor(neighbors.reference_position) if thr > 0.0 else None
        status = None
        host = st is not None
        if nw_fn is not None:
            self._wall_layer(eng, nw_fn)
        if host:
            e = eng
            cap = neighbors.cell_list_capacity
            e.nl_set_capacity(cap if cap is not None else 2 ** 31 - 1, neighbors.max_occupancy)
            # a summation carries drho/dt over unchanged (solver.py:794-796):
            # the result keeps the input's tensor, nothing is copied
            keys = OUT_KEYS if self.is_rho_evol else OUT_KEYS_SUMMATION
            if self.is_heat_conduction:
                keys = keys + HEAT_OUT_KEYS
            if nw_fn is not None:
                keys = keys + ("nw",)  # recomputed after the drift (integrator.py:33-34)
            # results and the status word in one pinned block: the status is
            # host memory, read without a device synchronisation
            out, status_h, vout = _lib.host_outputs(key[1], self.dim, keys)
            if thr > 0.0 and not (ref.device.type == "cpu" and ref.is_pinned()):
                ref = ref.to(torch.float32).contiguous().pin_memory()
            try:
                # returns once the results are in host memory
                status = e.advance(st, out, ref if thr > 0.0 else None, thr, vin=vin,
                                   vout=vout, status=status_h)
            except _lib.SphError as err:
                if "pinned" not in str(err):
                    raise
                host = False  # pageable host arrays: go through device copies instead
        if not host:
            e, st = self._load(state, neighbors, case, load=False)
            out = empty_outputs(st, self.is_heat_conduction)
            if nw_fn is not None:
                out["nw"] = torch.empty_like(st["nw"])
            if thr > 0.0:
                ref = ref.to(device=st["r"].device, dtype=torch.float32).contiguous()
            # one fused call: load, step, read back; the status stays a device
            # value inside the returned list's error code until the caller
            # tests it (host-side failures raise from the call)
            status = e.advance(st, out, ref if thr > 0.0 else None, thr)
        res = self._result(state, out)
        if host:
            fields = {k: res[k] for k in STATE_KEYS + HEAT_KEYS if res.get(k) is not None}
            self._last_host = (res, fields, e.next_view(), e)
        if bc_fn is not None and bc_spec is None:
            res = bc_fn(res)
        from .partition import NeighborList

        if thr > 0.0:
            # the reference rebuilds inside the step only when a particle
            # moved beyond the threshold (jax_md/partition.py:1010-1018)
            if host:
                moved = bool(int(status.item()) & _lib.INFO_MOVED)
                nbrs = NeighborList(nl_fns, res["r"] if moved else ref,
                                    neighbors.error.update(int(status.item()) & 0xFF, moved),
                                    neighbors.cell_list_capacity, neighbors.max_occupancy)
            else:
                mv = (status & _lib.INFO_MOVED) != 0
                nbrs = NeighborList(nl_fns, torch.where(mv, res["r"], ref),
                                    neighbors.error.merged(status & 0xFF, mv),
                                    neighbors.cell_list_capacity, neighbors.max_occupancy)
        else:
            # threshold 0: a list not rebuilt is one at unchanged positions,
            # whose reference position and overflow bits equal the new ones
            nbrs = NeighborList(nl_fns, res["r"], neighbors.error.merged(status),
                                neighbors.cell_list_capacity, neighbors.max_occupancy)
        if nl_fns.matscipy:
            # the particles that count are the unpadded ones (integrator.py:47)
            nbrs._num_particles = (res["tag"] != _lib.TAG_PAD).sum()
            nbrs._pad = int(nl_fns.num_particles_max or key[1])
        return res, nbrs
