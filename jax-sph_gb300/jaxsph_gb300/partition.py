"""Cell-list neighbour search: drop-in for ``jax_sph.partition.neighbor_list``.

Mirrors the reference's two-phase protocol (``jax_sph/partition.py:492-571``,
``jax_sph/jax_md/partition.py:620-1026``): ``allocate`` measures capacities on
the host (not capturable, like the reference's non-jittable allocate),
``update`` rebuilds with fixed capacities and reports overflow through the
``PartitionErrorCode`` bits of ``NeighborList.error``.

The work runs in ``libsph_gb300``: counting sort of particles by cell hash
(stable by particle index, like the reference's ``argsort``), then a cell-tiled
pass that emits the sparse ``(2, max_occupancy)`` edge list -- row 0 the
neighbour (receiver), row 1 the particle (sender), padding ``N`` -- with the
reference's exact float32 membership test ``metric(r_sender, r_receiver) <
cutoff**2``. Edges are sender-major with receivers ascending per sender; the
reference's own order inside a sender is its cell-slot order, so compare edge
lists after the canonical sort of ``tests/test_neighbors.py:77-82``.
"""

import enum
from collections import OrderedDict

import numpy as np
import torch

from . import _lib
from .space import PeriodicDisplacement, square_distance


class PartitionErrorCode(enum.IntEnum):
    """jax_md/partition.py:434-457."""

    NONE = 0
    NEIGHBOR_LIST_OVERFLOW = 1 << 0
    CELL_LIST_OVERFLOW = 1 << 1
    CELL_SIZE_TOO_SMALL = 1 << 2
    MALFORMED_BOX = 1 << 3


PEC = PartitionErrorCode


class NeighborListFormat(enum.Enum):
    """jax_md/partition.py:580-598 (only Sparse is on the path)."""

    Dense = 0
    Sparse = 1
    OrderedSparse = 2


Dense = NeighborListFormat.Dense
Sparse = NeighborListFormat.Sparse
OrderedSparse = NeighborListFormat.OrderedSparse


class PartitionError:
    """``PartitionError`` (jax_md/partition.py:460-499): an error-code bitfield.

    The code is a Python int or, straight out of a GPU step, a 0-d integer
    device tensor that is read (one synchronisation) the first time ``code``
    is asked for -- as the reference's code stays a device array until the
    caller tests ``did_buffer_overflow``.
    """

    def __init__(self, code=0, base=0):
        if isinstance(code, torch.Tensor):
            self._dev, self._code, self._base = code, None, int(base)
        else:
            self._dev, self._code, self._base = None, (int(code) | int(base)) & 0xFF, 0

    @property
    def code(self):
        if self._code is None:
            self._code = (int(self._dev.item()) | self._base) & 0xFF
            self._dev = None
        return self._code

    def merged(self, status, moved=None):
        """This code OR the low bits of a device ``status`` (where the device
        bool ``moved`` holds, if given), without a host synchronisation."""
        if moved is None:
            if self._code is not None:
                return PartitionError(status, base=self._code)
            return PartitionError(self._dev | status, base=self._base)
        base = self._dev if self._code is None else torch.full_like(status, self._code)
        return PartitionError(torch.where(moved, base | status, base), base=self._base)

    def update(self, bit, pred):
        return PartitionError(self.code | (int(bit) if pred else 0))

    def __str__(self):
        if not self.code:
            return ""
        if self.code & PEC.NEIGHBOR_LIST_OVERFLOW:
            return "Partition Error: Neighbor list buffer overflow."
        if self.code & PEC.CELL_LIST_OVERFLOW:
            return "Partition Error: Cell list buffer overflow"
        if self.code & PEC.CELL_SIZE_TOO_SMALL:
            return "Partition Error: Cell size too small"
        return "Partition Error: Incorrect box format. Expecting upper triangular."

    __repr__ = __str__


class NeighborList:
    """``NeighborList`` (jax_md/partition.py:620-671), sparse format.

    ``idx`` is an int32 CUDA tensor of shape ``(2, max_occupancy)``. Lists
    produced inside a fused ``si_euler`` step emit their ``idx`` on first
    access.
    """

    def __init__(self, fns, reference_position, error, cell_list_capacity, max_occupancy,
                 idx=None, occupancy=None):
        self._fns = fns
        self.reference_position = reference_position
        self.error = error if isinstance(error, PartitionError) else PartitionError(error)
        self.cell_list_capacity = cell_list_capacity
        self.max_occupancy = int(max_occupancy)
        self.format = fns.format
        self.cell_size = fns.cutoff
        self._idx = idx
        self._occupancy = occupancy
        # matscipy backend: the particles that count (an int or a 0-d tensor,
        # read when idx is emitted) and the padding value of idx
        self._num_particles = None
        self._pad = None

    @property
    def idx(self):
        if self._idx is None:
            n = self._num_particles
            n = int(n.item()) if isinstance(n, torch.Tensor) else n
            self._idx, self._occupancy, code = self._fns._emit(
                self.reference_position, self.cell_list_capacity, self.max_occupancy, n,
                self._pad)
            self.error = self.error.update(code, code != 0)
        return self._idx

    @property
    def occupancy(self):
        if self._occupancy is None:
            _ = self.idx
        return self._occupancy

    def update(self, position, **kwargs):
        return self._fns.update(position, self, **kwargs)

    @property
    def did_buffer_overflow(self):
        return bool(self.error.code & (PEC.NEIGHBOR_LIST_OVERFLOW | PEC.CELL_LIST_OVERFLOW))

    @property
    def cell_size_too_small(self):
        return bool(self.error.code & PEC.CELL_SIZE_TOO_SMALL)

    @property
    def malformed_box(self):
        return bool(self.error.code & PEC.MALFORMED_BOX)


def _as_device_f32(x):
    t = torch.as_tensor(x)
    if not t.is_cuda:
        t = t.to("cuda")
    return t.to(torch.float32).contiguous()


class NeighborListFns:
    """``NeighborListFns(allocate, update)`` (jax_md/partition.py:674-717)."""

    def __init__(self, box_size, r_cutoff, dr_threshold=0.0, capacity_multiplier=1.25,
                 mask_self=True, format=Sparse, backend="jaxmd_vmap", num_particles_max=None):
        self.box = np.asarray(box_size, dtype=np.float64).reshape(-1)
        self.dim = int(self.box.size)
        if self.dim not in (2, 3):
            raise ValueError(f"Cell list spatial dimension must be 2 or 3. Found {self.dim}.")
        self.r_cutoff = float(r_cutoff)
        self.dr_threshold = float(dr_threshold)
        # cutoff = r_cutoff + dr_threshold, threshold_sq = (dr_threshold / 2)^2 (:814-823)
        self.cutoff = float(np.float32(self.r_cutoff) + np.float32(self.dr_threshold))
        self.threshold_sq = float(np.float32(np.float32(self.dr_threshold) / np.float32(2)) ** 2)
        self.capacity_multiplier = float(capacity_multiplier)
        self.mask_self = bool(mask_self)
        self.format = format
        # the matscipy backend (partition.py:356-482): a variable number of
        # particles padded to num_particles_max, float64 distances, edges
        # ordered by their first index with the self edges first
        self.matscipy = backend == "matscipy"
        self.num_particles_max = num_particles_max
        self._metric = PeriodicDisplacement(self.box)
        self._engines = OrderedDict()

    def __iter__(self):
        return iter((self.allocate, self.update))

    # -- engine plumbing
    def config(self, **solver):
        c = _lib.SphConfig()
        c.dim = self.dim
        c.kernel = solver.get("kernel", 0)
        c.solver = solver.get("solver", 0)
        c.is_rho_evol = int(solver.get("is_rho_evol", 0))
        c.is_bc_trick = int(solver.get("is_bc_trick", 0))
        c.is_free_slip = int(solver.get("is_free_slip", 0))
        c.mask_self = int(self.mask_self)
        c.kahan = int(solver.get("kahan", 0))
        c.fp64_positions = int(solver.get("fp64_positions", 0))
        c.capacity_multiplier = self.capacity_multiplier
        c.verlet_skin = float(solver.get("verlet_skin", 0.0))
        c.canonical_order = int(solver.get("canonical_order", 0))
        c.is_rho_renorm = int(solver.get("is_rho_renorm", 0))
        c.is_heat_conduction = int(solver.get("is_heat_conduction", 0))
        c.nl_backend = _lib.NL_MATSCIPY if self.matscipy else _lib.NL_JAXMD
        return c

    def case(self, n):
        """An SphCase with this list's geometry and neutral physics."""
        s = _lib.SphCase()
        s.n = int(n)
        for d in range(3):
            s.box[d] = float(self.box[d]) if d < self.dim else 1.0
        # matscipy compares float64 distances with the cutoff as given
        s.r_cutoff = self.r_cutoff if self.matscipy else self.cutoff
        s.dx = s.h = self.r_cutoff
        s.eos = _lib.EOS_TAIT
        s.p_ref = s.rho_ref = s.gamma = s.u_ref = 1.0
        s.eta_limiter = -1.0
        return s

    def _engine(self, n):
        e = self._engines.get(n)
        if e is None:
            e = _lib.Engine(self.config(), [self.case(n)])
            self._engines[n] = e
            while len(self._engines) > 2:
                self._engines.popitem(last=False)
        return e

    def _load(self, position, num_particles=None):
        r = _as_device_f32(position)
        n = r.shape[0]
        if r.ndim != 2 or r.shape[1] != self.dim:
            raise ValueError(f"positions must have shape (N, {self.dim})")
        e = self._engine(n)
        z1 = torch.zeros(n, dtype=torch.float32, device=r.device)
        zd = torch.zeros_like(r)
        tag = torch.zeros(n, dtype=torch.int32, device=r.device)
        if num_particles is not None:  # positions[num_particles:] pad the state
            tag[int(num_particles):] = _lib.TAG_PAD
        state = dict(r=r, tag=tag, u=zd, v=zd, dudt=zd, dvdt=zd, rho=z1 + 1.0, p=z1,
                     mass=z1 + 1.0, eta=z1)
        e.set_state(state)
        return e, r

    def _emit(self, position, cell_capacity, max_occupancy, num_particles=None, pad=None):
        e, r = self._load(position, num_particles)
        e.nl_set_capacity(cell_capacity if cell_capacity is not None else 2 ** 31 - 1,
                          max_occupancy)
        e.read_status(clear=True)
        e.nl_update()
        idx, count = e.nl_edges(max_occupancy, r.device)
        code = e.read_status(clear=True)
        n_edges = int(count.item())
        if self.matscipy:
            if n_edges > max_occupancy:  # all of them, to order before truncating
                idx, _ = e.nl_edges(n_edges, r.device)
            idx = self._matscipy_order(idx[:, :n_edges], max_occupancy,
                                       r.shape[0] if pad is None else pad)
        return idx, n_edges, code & 0xFF

    def _matscipy_order(self, edges, capacity, pad):
        """matscipy's "ij" list as the reference returns it: the self edges
        (when not masked) first, then every pair by first index (partition.py:
        387-404; within an index the second ascending here), truncated to
        ``capacity`` or padded with ``pad``."""
        i, j = edges[0].long(), edges[1].long()
        self_e = i == j
        n = int(max(int(torch.maximum(i, j).max()) + 1 if i.numel() else 0, 1))
        key = torch.where(self_e, i, n + i * n + j)  # self edges sort before all pairs
        order = torch.argsort(key)
        out = torch.full((2, int(capacity)), int(pad), dtype=torch.int32, device=edges.device)
        k = min(int(capacity), int(order.numel()))
        out[:, :k] = edges[:, order[:k]]
        return out

    # -- reference API
    def allocate(self, position, extra_capacity=0, **kwargs):
        """Build a list and size its capacities from the data (host-synchronous).

        The edge array ``idx`` is emitted when first read (the same array the
        reference's allocate returns); a fused si_euler step never reads it.
        With the matscipy backend ``num_particles`` (default all) particles
        count, the rest pad the state.
        """
        num = kwargs.get("num_particles") if self.matscipy else None
        e, r = self._load(position, num)  # loading clears the status word
        cap = e.nl_allocate(extra_capacity)
        code = e.read_status(clear=True) & 0xFF
        if self.matscipy:
            # (2, round(E * multiplier * num_particles_max / num_particles + extra)),
            # padded with num_particles (partition.py:458-466)
            n = int(r.shape[0] if num is None else num)
            n_max = int(self.num_particles_max or r.shape[0])
            edges = int(cap.occupancy)
            size = round(edges * (self.capacity_multiplier * n_max / n) + extra_capacity)
            nbrs = NeighborList(self, position, 0, None, size, occupancy=edges)
            nbrs._num_particles, nbrs._pad = n, n
            return nbrs
        cell_cap = int(cap.cell_capacity) if self._uses_cells() else None
        return NeighborList(self, position, code, cell_cap, cap.max_occupancy,
                            occupancy=int(cap.occupancy))

    def _uses_cells(self):
        box32 = self.box.astype(np.float32)
        return bool(np.all(np.float32(self.cutoff) < box32 / np.float32(3.0)))

    def moved(self, position, neighbors):
        """The reference's rebuild test ``any(metric(r, r_ref) > threshold_sq)`` (:1010-1018)."""
        r = _as_device_f32(position)
        ref = _as_device_f32(neighbors.reference_position)
        d2 = square_distance(self._metric(r, ref))
        return bool((d2 > self.threshold_sq).any().item())

    def moved_dev(self, position, neighbors):
        """``moved`` as a 0-d bool device tensor (no host synchronisation)."""
        r = _as_device_f32(position)
        ref = _as_device_f32(neighbors.reference_position)
        d2 = square_distance(self._metric(r, ref))
        return (d2 > self.threshold_sq).any()

    def update(self, position, neighbors, **kwargs):
        """Rebuild with fixed capacities if any particle moved beyond the threshold."""
        if self.matscipy:
            # always rebuilt; more edges than the capacity truncate and raise
            # NEIGHBOR_LIST_OVERFLOW; padded with num_particles_max (:414-443)
            n = kwargs.get("num_particles")
            r = _as_device_f32(position)
            n_max = int(self.num_particles_max or r.shape[0])
            idx, count, code = self._emit(position, None, neighbors.max_occupancy, n, n_max)
            over = PEC.NEIGHBOR_LIST_OVERFLOW if count > neighbors.max_occupancy else 0
            nbrs = NeighborList(self, position, neighbors.error.code | over, None,
                                neighbors.max_occupancy, idx=idx, occupancy=count)
            nbrs._num_particles, nbrs._pad = n, n_max
            return nbrs
        if not self.moved(position, neighbors):
            return neighbors
        idx, count, code = self._emit(position, neighbors.cell_list_capacity,
                                      neighbors.max_occupancy)
        return NeighborList(self, position, neighbors.error.code | code,
                            neighbors.cell_list_capacity, neighbors.max_occupancy, idx=idx,
                            occupancy=count)


BACKENDS = ("jaxmd_vmap", "jaxmd_scan", "matscipy")


def neighbor_list(displacement_or_metric, box_size, r_cutoff, backend="jaxmd_vmap",
                  dr_threshold=0.0, capacity_multiplier=1.25, disable_cell_list=False,
                  mask_self=True, custom_mask_function=None, fractional_coordinates=False,
                  format=Sparse, num_particles_max=None, num_partitions=1, pbc=None):
    """Drop-in for ``jax_sph.partition.neighbor_list`` (jax_sph/partition.py:492-571).

    ``jaxmd_vmap`` and ``jaxmd_scan`` produce the same neighbour sets and are
    served by the same GPU cell list; ``num_partitions`` is accepted for
    signature compatibility (the GPU search never materialises candidates, so
    it needs no memory chunking). ``disable_cell_list`` selects the same sets
    and is likewise served by the cell list. ``matscipy`` (periodic boxes) takes
    ``num_particles`` on allocate/update, the rest of the positions padding, and
    follows that backend's float64 membership, edge order, capacity rule and
    padding values; ``num_particles_max`` sizes its capacity.
    """
    if backend not in BACKENDS:
        raise NotImplementedError(f"backend {backend!r}: the GPU path serves {BACKENDS}")
    if backend == "matscipy" and pbc is not None and not np.all(np.asarray(pbc)):
        raise NotImplementedError("the matscipy backend is served for periodic boxes only")
    if format is not Sparse:
        raise NotImplementedError("only the Sparse format is on the hot path")
    if custom_mask_function is not None:
        raise NotImplementedError("custom_mask_function is not supported")
    if fractional_coordinates:
        raise NotImplementedError("fractional coordinates are not supported")
    return NeighborListFns(box_size, r_cutoff, dr_threshold, capacity_multiplier, mask_self,
                           format, backend, num_particles_max)
