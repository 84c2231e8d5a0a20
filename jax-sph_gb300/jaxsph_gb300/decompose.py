"""Spatial domain decomposition of one case into slabs: the multi-GPU mode.

The step is local in space: a particle's new state depends on the particles
within the cutoff after the drift, and their densities on the particles
within the cutoff of those -- two levels; with the generalized wall boundary
condition of the SPH solver a wall neighbour's pressure is a Shepard sum of
its fluid neighbours' pressures, a third level. So the box is cut into slabs
along its longest axis, each slab is advanced by its own engine on the
particles it owns plus a halo of every particle within ``levels * cutoff +
2 * drift`` of the slab (drift: the most any particle moves in the step), and
each slab keeps the results of the particles it owns. The halo carries everything the owned particles'
neighbours need, so a step needs one exchange before it (halo and migrated
particles: point-to-point, no collective) and none inside it.

Local states keep the particles in ascending global index and the engines sum
pairs in canonical (original-index) order, so every owned particle's result
is bit for bit the one of the undivided run.

``VirtualSlabs`` runs all slabs in one process on one GPU (one engine per
slab); ``DistributedSlabs`` runs one slab per rank of a ``torch.distributed``
group, exchanging halos and migrants with point-to-point sends.
"""

import numpy as np
import torch

from . import _lib
from .simulate import make_neighbor_fns, make_solver
from .solver import prepare_state

STATE_FIELDS = ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "mass", "eta", "nw")
OUT_FIELDS = ("r", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p")
HEAT_FIELDS = ("T", "dTdt", "kappa", "Cp")
_VECTOR = ("r", "u", "v", "dudt", "dvdt", "nw")


def state_fields(setup):
    """The fields a slab exchanges and keeps: with heat conduction the
    temperature fields too."""
    heat = setup.solver.get("is_heat_conduction", False)
    return STATE_FIELDS + (HEAT_FIELDS if heat else ())


def out_fields(setup):
    """The fields a step changes: with heat conduction T and dT/dt, with
    moving walls the recomputed normals."""
    out = OUT_FIELDS
    if setup.solver.get("is_heat_conduction", False):
        out = out + ("T", "dTdt")
    if setup.nw_fn is not None:
        out = out + ("nw",)
    return out


def longest_axis(box):
    return int(np.argmax(np.asarray(box, dtype=np.float64)))


def slab_of(x, length, n_parts):
    """Slab index of coordinates x in [0, length): floor(x n / length), clamped."""
    k = torch.floor(x.double() * (n_parts / length)).long()
    return k.clamp_(0, n_parts - 1)


def near_slab(x, k, n_parts, length, width):
    """Whether x lies within ``width`` of slab k (periodic), inside it included."""
    half = 0.5 * length / n_parts
    centre = (k + 0.5) * length / n_parts
    d = x.double() - centre
    d = d - length * torch.round(d / length)
    return d.abs() <= half + width


def step_drift(state, dt, cv):
    """An upper bound of how far any particle moves in the coming si_euler
    step: |u + dt dudt + cv dvdt| dt, maximised component-wise (cv =
    tvf dt / 2, integrator.py:26-30)."""
    u, a, b = state["u"].double(), state["dudt"].double(), state["dvdt"].double()
    v = u.abs() + dt * a.abs() + abs(cv) * b.abs()
    return float(dt * torch.linalg.vector_norm(v, dim=1).max()) if v.numel() else 0.0


def halo_width(cutoff, drift, levels=2):
    """``levels`` cutoffs plus twice the drift, with a margin for float32 rounding."""
    return levels * cutoff * (1.0 + 1e-5) + 2.0 * drift * 1.01 + 1e-6


class _SlabEngines:
    """The engines of one case's slabs, one per local particle count (the
    count changes as particles cross slab boundaries)."""

    def __init__(self, setup, device):
        self.setup = setup
        self.solver = make_solver(setup)
        self.nl = make_neighbor_fns(setup, self.solver)
        flags = self.solver.solver_flags()
        # canonical pair order: the owned particles' sums match the undivided run
        self.cfg = self.nl.config(**flags, verlet_skin=0.0, canonical_order=1)
        self.device = torch.device(device)
        self.cutoff = float(self.solver._kernel_fn.cutoff)
        # cutoff levels a particle's step reaches: force <- neighbour density
        # <- its neighbours (delta-SPH evolution: density <- H of the
        # neighbours <- L of theirs <- their neighbours, three levels; a
        # renormalisation adds one); the wall BC of SPH and DELTA adds wall
        # pressure <- fluid pressure (solver.py:431-530)
        v = self.solver
        density = 3 if (v.solver == "DELTA" and v.is_rho_evol) else 1
        renorm = 1 if (v.is_rho_evol and v.is_rho_renorm) else 0
        gwbc = 1 if (v.solver != "RIE" and v.is_bc_trick) else 0
        self.levels = density + renorm + 1 + gwbc
        self.cv = float(setup.tvf) * 0.5 * float(setup.dt)
        self._engines = {}
        if self.solver.g_spec()["kind"] == _lib.GEXT_ARRAY:
            raise NotImplementedError("slabs need a g_ext_fn with a GPU spec")
        self.fields = state_fields(setup)
        self.out = out_fields(setup)

    def engine(self, n):
        e = self._engines.get(n)
        if e is None:
            s = self.setup
            case = self.solver.sph_case(self.nl, n, dt=s.dt, tvf=s.tvf, bc=s.bc_fn.spec)
            if len(self._engines) > 8:
                self._engines.clear()
            e = _lib.Engine(self.cfg, [case])
            if s.nw_fn is not None:  # moving walls: each slab recomputes its walls' normals
                spec = s.nw_fn.spec
                e.set_wall_layer(spec["layer"], spec["offset"], spec["cutoff"])
            self._engines[n] = e
        return e

    def advance(self, local):
        """One si_euler step of a local state (owned + halo particles in
        ascending global index); returns the new state's fields."""
        n = int(local["r"].shape[0])
        e = self.engine(n)
        e.set_state(local)
        e.step(1)
        out = {k: torch.empty_like(local[k]) for k in self.out}
        e.get_state(out)
        return out


class VirtualSlabs:
    """All slabs of a case in one process on one GPU.

    ``state`` holds the whole case in global order; ``step`` advances every
    slab on its owned + halo particles and keeps each slab's owned results.
    """

    def __init__(self, setup, n_parts, device="cuda", axis=None):
        _lib.require_cuda()
        self.n_parts = int(n_parts)
        self.axis = longest_axis(setup.box) if axis is None else int(axis)
        self.length = float(setup.box[self.axis])
        self.dim = setup.dim
        self.slabs = _SlabEngines(setup, device)
        st = prepare_state(setup.state, setup.dim, device,
                           heat=setup.solver.get("is_heat_conduction", False))
        if "nw" not in st:
            st["nw"] = torch.zeros_like(st["r"])
        self.state = st
        self.last_sizes = []

    def step(self, nsteps=1):
        s = self.slabs.setup
        for _ in range(int(nsteps)):
            st = self.state
            x = st["r"][:, self.axis]
            w = halo_width(self.slabs.cutoff, step_drift(st, s.dt, self.slabs.cv),
                           self.slabs.levels)
            owner = slab_of(x, self.length, self.n_parts)
            new = {k: st[k].clone() for k in self.slabs.out}
            self.last_sizes = []
            for k in range(self.n_parts):
                local = (owner == k) | near_slab(x, k, self.n_parts, self.length, w)
                idx = torch.nonzero(local).squeeze(1)  # ascending global index
                if idx.numel() == 0:
                    continue
                owned = owner[idx] == k
                out = self.slabs.advance({f: st[f][idx].contiguous() for f in self.slabs.fields})
                keep = idx[owned]
                for f in self.slabs.out:
                    new[f][keep] = out[f][owned]
                self.last_sizes.append((int(owned.sum()), int(idx.numel())))
            st.update(new)


# ------------------------------------------------------------------ distributed
def _pack(rows, fields=STATE_FIELDS):
    """Fields of a set of particles as one float64 matrix (global index,
    tag and every float field; float32 and int32 values are exact in it)."""
    cols = [rows["gid"].double()[:, None], rows["tag"].double()[:, None]]
    for f in fields:
        if f in ("tag",):
            continue
        t = rows[f].double()
        cols.append(t if t.ndim == 2 else t[:, None])
    return torch.cat(cols, dim=1).contiguous()


def _unpack(mat, dim, fields=STATE_FIELDS):
    out = {"gid": mat[:, 0].long(), "tag": mat[:, 1].to(torch.int32)}
    c = 2
    for f in fields:
        if f == "tag":
            continue
        width = dim if f in _VECTOR else 1
        t = mat[:, c:c + width].to(torch.float32)
        out[f] = t.contiguous() if width > 1 else t[:, 0].contiguous()
        c += width
    return out


def _columns(dim, fields=STATE_FIELDS):
    return 2 + sum(dim if f in _VECTOR else 1 for f in fields if f != "tag")


def exchange(rows, dest, dim, group=None, fields=STATE_FIELDS):
    """Point-to-point exchange: rank r receives the rows with ``dest[r]``
    true from every rank. ``rows``: fields of this rank's particles plus
    ``gid``; ``dest``: a bool mask per rank. Returns the received rows of all
    other ranks concatenated (not sorted)."""
    import torch.distributed as dist

    ws, me = dist.get_world_size(group), dist.get_rank(group)
    mat = _pack(rows, fields)
    # on the rows' device: NCCL exchanges device tensors, gloo host tensors
    counts = torch.tensor([int(dest[r].sum()) if r != me else 0 for r in range(ws)],
                          dtype=torch.int64, device=mat.device)
    table = [torch.zeros_like(counts) for _ in range(ws)]
    dist.all_gather(table, counts, group=group)  # who sends how much to whom
    reqs, recv = [], []
    for r in range(ws):
        if r == me:
            continue
        if int(counts[r]):
            reqs.append(dist.isend(mat[dest[r]].contiguous(), r, group=group))
        n = int(table[r][me])
        if n:
            buf = torch.empty((n, mat.shape[1]), dtype=mat.dtype, device=mat.device)
            reqs.append(dist.irecv(buf, r, group=group))
            recv.append(buf)
    for q in reqs:
        q.wait()
    if not recv:
        return _unpack(torch.empty((0, _columns(dim, fields)), dtype=torch.float64,
                                   device=mat.device), dim, fields)
    return _unpack(torch.cat(recv), dim, fields)


def merge(a, b):
    """Union of two row sets, sorted by global index."""
    gid = torch.cat([a["gid"], b["gid"]])
    order = torch.argsort(gid)
    return {f: torch.cat([a[f], b[f]])[order].contiguous() for f in a}


class DistributedSlabs:
    """One slab per rank of a ``torch.distributed`` group.

    Each rank holds the particles it owns (``owned``: fields plus ``gid``,
    ascending). A step: every rank sends each other rank its particles within
    the halo of that rank's slab; runs the step on owned + received; keeps
    the owned results; then sends the particles whose new position lies in
    another slab to their new owner (migration).
    """

    def __init__(self, setup, device="cuda", axis=None, group=None):
        import torch.distributed as dist

        self.group = group
        self.ws, self.rank = dist.get_world_size(group), dist.get_rank(group)
        self.axis = longest_axis(setup.box) if axis is None else int(axis)
        self.length = float(setup.box[self.axis])
        self.dim = setup.dim
        self.device = torch.device(device)
        self.slabs = _SlabEngines(setup, device)
        st = prepare_state(setup.state, setup.dim, self.device,
                           heat=setup.solver.get("is_heat_conduction", False))
        if "nw" not in st:
            st["nw"] = torch.zeros_like(st["r"])
        gid = torch.arange(setup.n, device=self.device)
        mine = slab_of(st["r"][:, self.axis], self.length, self.ws) == self.rank
        self.owned = {f: st[f][mine].contiguous() for f in self.slabs.fields}
        self.owned["gid"] = gid[mine]

    def local_state(self, width):
        """Owned particles plus the halo received from the other ranks."""
        x = self.owned["r"][:, self.axis]
        dest = [near_slab(x, r, self.ws, self.length, width) for r in range(self.ws)]
        halo = exchange(self.owned, dest, self.dim, self.group, self.slabs.fields)
        halo = {f: halo[f].to(self.device) for f in halo}
        return merge(self.owned, halo)

    def step(self, nsteps=1):
        import torch.distributed as dist

        s = self.slabs.setup
        for _ in range(int(nsteps)):
            drift = torch.tensor([step_drift(self.owned, s.dt, self.slabs.cv)],
                                 dtype=torch.float64, device=self.device)
            dist.all_reduce(drift, op=dist.ReduceOp.MAX, group=self.group)
            local = self.local_state(halo_width(self.slabs.cutoff, float(drift),
                                                self.slabs.levels))
            owned = torch.isin(local["gid"], self.owned["gid"])
            out = self.slabs.advance({f: local[f] for f in self.slabs.fields})
            for f in self.slabs.out:
                self.owned[f] = out[f][owned].contiguous()
            self.migrate()

    def migrate(self):
        """Hand the particles whose position left this rank's slab to their owner."""
        x = self.owned["r"][:, self.axis]
        owner = slab_of(x, self.length, self.ws)
        dest = [owner == r for r in range(self.ws)]
        arrived = exchange(self.owned, dest, self.dim, self.group, self.slabs.fields)
        arrived = {f: arrived[f].to(self.device) for f in arrived}
        stay = owner == self.rank
        kept = {f: self.owned[f][stay] for f in self.owned}
        self.owned = merge(kept, arrived)
