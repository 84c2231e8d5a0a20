"""Resident GPU rollouts: the fast path behind ``jax_sph.simulate.simulate``.

``Simulation`` keeps one or many cases resident on the GPU in cell-sorted
order and advances them with ``sph_step`` (a CUDA graph of whole si_euler
steps, no host work between steps). Many cases sharing one configuration
(e.g. lid-driven cavities and Poiseuille channels of different resolutions)
run as one concatenated batch: one cell list with per-case offsets, one launch
per pass for the whole batch.

``simulate`` reproduces the reference driver loop (``jax_sph/simulate.py:
110-134``): a discarded warm-up ``advance(0.0)``, ``sequence_length + 2``
steps and the overflow protocol. The status word is polled every
``check_every`` steps instead of every step; results never depend on the
capacities (nothing is truncated on the GPU), so an overflow only triggers a
re-allocation of the capacities, without re-running steps.
"""

import torch

from . import _lib
from .partition import NeighborListFns, Sparse
from .solver import WCSPH, prepare_state


def make_solver(setup, kahan=False):
    """The ``WCSPH`` instance ``simulate`` builds for a case (simulate.py:49-69)."""
    disp, _ = setup.space()
    s = setup.solver
    return WCSPH(disp, setup.eos, setup.g_ext_fn, setup.dx, setup.dim, setup.dt, setup.c_ref,
                 eta_limiter=s.get("eta_limiter", 3), diff_delta=s.get("diff_delta", 0.1),
                 diff_alpha=s.get("diff_alpha", 0.01), solver=s["solver"], kernel=s["kernel"],
                 h_fac=s.get("h_fac", 1.0), is_bc_trick=s["is_bc_trick"],
                 is_rho_evol=s["is_rho_evol"], artificial_alpha=s["artificial_alpha"],
                 is_free_slip=s["is_free_slip"], is_rho_renorm=s.get("is_rho_renorm", False),
                 is_heat_conduction=s.get("is_heat_conduction", False), kahan=kahan)


def make_neighbor_fns(setup, solver, mask_self=False, capacity_multiplier=1.25):
    """``partition.neighbor_list`` as ``simulate`` calls it (simulate.py:75-86)."""
    return NeighborListFns(setup.box, solver._kernel_fn.cutoff, 0.0, capacity_multiplier,
                           mask_self, Sparse)


class Simulation:
    """One or more cases advanced together on the GPU.

    ``setups`` is a ``CaseSetup`` or a list of them sharing dimension, kernel,
    solver and boundary treatment. States are given and returned per case in
    the reference's particle order. ``skin`` (a fraction of the cutoff) sets
    how far particles may move before the candidate lists are rebuilt; the
    neighbour set of every step is the reference's whatever its value. Pair
    sums run in cell order (deterministic for a given run); with
    ``canonical_order`` they run in ascending original index, so that results
    are bit for bit independent of the skin, the batching and checkpoint
    restores.
    """

    def __init__(self, setups, kahan=False, mask_self=False, capacity_multiplier=1.25,
                 device="cuda", autotune=False, block_size=None, fp64_positions=False,
                 skin=0.1, canonical_order=False):
        if not isinstance(setups, (list, tuple)):
            setups = [setups]
        _lib.require_cuda()
        self.setups = list(setups)
        self.device = torch.device(device)
        self.solvers = [make_solver(s, kahan) for s in self.setups]
        self.nl = [make_neighbor_fns(s, v, mask_self, capacity_multiplier)
                   for s, v in zip(self.setups, self.solvers)]
        flags = self.solvers[0].solver_flags()
        for v in self.solvers[1:]:
            if v.solver_flags() != flags or v.dim != self.solvers[0].dim:
                raise ValueError("batched cases must share dimension, kernel, solver and BC treatment")
        cfg = self.nl[0].config(**flags, fp64_positions=fp64_positions, verlet_skin=skin,
                                canonical_order=canonical_order)
        self.cases = [v.sph_case(nl, s.n, dt=s.dt, tvf=s.tvf, bc=s.bc_fn.spec)
                      for s, v, nl in zip(self.setups, self.solvers, self.nl)]
        for v in self.solvers:
            if v.g_spec()["kind"] == _lib.GEXT_ARRAY:
                raise NotImplementedError("resident rollouts need g_ext_fn with a GPU spec")
        self.engine = _lib.Engine(cfg, self.cases)
        self.wall_normals = any(s.nw_fn is not None for s in self.setups)
        if self.wall_normals:
            if len(self.setups) > 1:
                raise NotImplementedError("moving-wall normals need a single case")
            spec = self.setups[0].nw_fn.spec
            self.engine.set_wall_layer(spec["layer"], spec["offset"], spec["cutoff"])
        self.sizes = [s.n for s in self.setups]
        self.dim = self.setups[0].dim
        self.steps_done = 0
        self.block_size = 256
        self.load([s.state for s in self.setups])
        if block_size is not None:
            self.engine.set_block_size(block_size)
            self.block_size = int(block_size)
        elif autotune:
            from . import autotune as _at

            self.block_size, self.tuning = _at.tune(self.engine)
            self.load([s.state for s in self.setups])  # tuning ran steps: start over

    def load(self, states):
        heat = self.solvers[0].is_heat_conduction
        parts = [prepare_state(st, self.dim, self.device, heat=heat) for st in states]
        full = {k: torch.cat([p[k] for p in parts]).contiguous() for k in parts[0]}
        if "nw" not in full:
            full["nw"] = torch.zeros_like(full["r"])
        self._full = full
        self.engine.set_state(full)
        self.capacity = self.engine.nl_allocate()
        self.engine.read_status(clear=True)

    def restore(self, full):
        """Reload a state saved with ``state(split=False)`` from this simulation,
        keeping the capacities (no host synchronisation)."""
        self._full = full
        self.engine.set_state(full)

    def run(self, nsteps, check_every=None):
        """Advance every case by ``nsteps`` si_euler steps. Returns the status bits seen."""
        seen = 0
        check_every = check_every or nsteps
        left = int(nsteps)
        while left > 0:
            k = min(left, check_every)
            self.engine.step(k)
            left -= k
            self.steps_done += k
            seen |= self._poll()  # once after every batch of steps
        return seen if nsteps > 0 else self._poll()

    def _poll(self):
        code = self.engine.read_status(clear=True)
        if code & (_lib.ERR_INVALID_ARG | _lib.ERR_CUDA):
            raise _lib.SphError(code, "GPU step failed")
        if code & (_lib.NEIGHBOR_LIST_OVERFLOW | _lib.CELL_LIST_OVERFLOW):
            # simulate.py:120-128: re-allocate at the current positions
            self.capacity = self.engine.nl_allocate()
            self.engine.read_status(clear=True)
        return code

    def state(self, split=True):
        """Current state(s) in the original particle order (device tensors)."""
        full = self._full
        keys = ("r", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p")
        if "T" in full:
            keys = keys + ("T", "dTdt")
        if self.wall_normals:
            keys = keys + ("nw",)  # recomputed every step
        out = {k: torch.empty_like(full[k]) for k in keys}
        self.engine.get_state(out)
        for k in ("tag", "mass", "eta", "nw", "kappa", "Cp"):
            if k in full and k not in out:
                out[k] = full[k]
        if not split:
            return out
        res, o = [], 0
        for n in self.sizes:
            res.append({k: v[o:o + n] for k, v in out.items()})
            o += n
        return res

    def diagnostics(self):
        """Per-case float64 (mass, momentum xyz, E_kin, u_max, rho_min, rho_max) from the GPU."""
        return self.engine.diagnostics(self.device)


def simulate(setup, steps=None, check_every=100, kahan=False, data_path=None, write_every=1):
    """The reference driver loop on the GPU (simulate.py:110-134); returns the final state.

    With ``data_path``, writes ``traj_<k>.h5`` every ``write_every`` files like
    the reference: file k holds the state after k + 1 steps (the loop writes
    before each step, skipping the initial state, simulate.py:114-115).
    """
    sim = Simulation(setup, kahan=kahan)
    steps = setup.sequence_length + 2 if steps is None else steps
    # warm-up advance(0.0, ...) of the reference: its result is discarded
    if data_path is None:
        sim.run(steps, check_every=check_every)
        return sim.state()[0]
    import os

    from .io_state import write_state

    os.makedirs(data_path, exist_ok=True)
    seq = setup.sequence_length
    done = 0
    for k in range(0, steps - 1, int(write_every)):
        # file k: the state after k + 1 steps
        sim.run(k + 1 - done, check_every=check_every)
        done = k + 1
        write_state(k, sim.state()[0], data_path, seq, write_every)
    if steps > done:
        sim.run(steps - done, check_every=check_every)
    return sim.state()[0]
