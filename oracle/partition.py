"""Cell-list neighbour search restated from jax-sph's vendored JAX-MD (test oracle only).

Follows ``jax_sph/jax_md/partition.py`` (``cell_list`` :243-428,
``neighbor_list`` :723-1026) for the ``jaxmd_vmap`` backend and the sparse
format that ``jax_sph/simulate.py:75-86`` requests. The edge list is produced in
exactly the reference's order (sender-major, receivers in cell-slot order), so
the golden lists of ``tests/test_neighbors.py:89-121`` can be compared verbatim
after the same canonical sort.
"""

import itertools
from dataclasses import dataclass

import numpy as np
import torch

from . import space

# PartitionErrorCode bits (jax_md/partition.py:453-457)
NEIGHBOR_LIST_OVERFLOW = 1 << 0
CELL_LIST_OVERFLOW = 1 << 1
CELL_SIZE_TOO_SMALL = 1 << 2
MALFORMED_BOX = 1 << 3


def _np_dtype(dtype):
    return np.float64 if dtype == torch.float64 else np.float32


def cutoff_values(r_cutoff, dtype):
    """``cutoff`` and ``cutoff_sq`` as the jitted reference sees them.

    jax_md/partition.py:814-823: ``r_cutoff`` becomes a weakly typed array of
    the run dtype (float32 unless x64 is enabled) and is squared in that dtype.
    """
    f = _np_dtype(dtype)
    cut = f(r_cutoff) + f(0.0)
    return cut, f(cut * cut)


def cell_dimensions(box, cutoff, dtype):
    """``_cell_dimensions`` (jax_md/partition.py:114-156) on the f32-cast box.

    ``box = f32(box)`` (:819); ``minimum_cell_size`` keeps the run dtype, so the
    division promotes to float64 in x64 runs and stays float32 otherwise.
    Returns (cell_size per dim in the hash dtype, cells per side, use_cells).
    """
    box32 = np.asarray(box, dtype=np.float32).reshape(-1)
    cut, _ = cutoff_values(cutoff, dtype)
    f = np.result_type(np.float32, _np_dtype(dtype)).type
    # neighbor_list only builds cells when cell_size < box / 3 in every dim (:935)
    use_cells = bool(np.all(f(cut) < box32.astype(f) / f(3.0)))
    cps = np.floor(box32.astype(f) / f(cut))
    cell_size = (box32.astype(f) / cps).astype(f)
    return cell_size, cps.astype(np.int32), use_cells


def _hashes(position, cell_size, cps):
    """Cell hash ``sum(int32(r / cell_size) * mult)`` (jax_md/partition.py:367-368)."""
    cs = torch.as_tensor(cell_size, dtype=position.dtype)
    idx = (position / cs).to(torch.int32)
    dim = position.shape[1]
    mult = [1]
    for d in range(1, dim):
        mult.append(mult[-1] * int(cps[d - 1]))
    h = torch.zeros(position.shape[0], dtype=torch.int64)
    for d in range(dim):
        h = h + idx[:, d].to(torch.int64) * mult[d]
    return h


def estimate_cell_capacity(position, cell_size, cps, multiplier=1.25):
    """``_estimate_cell_capacity`` (jax_md/partition.py:195-199)."""
    h = _hashes(position, cell_size, cps)
    ncell = int(np.prod(cps))
    occ = torch.bincount(h.clamp(0, ncell - 1), minlength=ncell)
    return int(int(occ.max()) * multiplier)


def cell_list_ids(position, cell_size, cps, capacity):
    """``cell_list_fn`` id buffer (jax_md/partition.py:294-413).

    Stable argsort of the hashes, slot = hash * capacity + (sorted rank mod
    capacity), scatter of particle ids (out-of-range slots dropped, as JAX
    scatters drop them). Returns the buffer reshaped to
    ``cells_per_side[::-1] + (capacity,)`` and the overflow flag.
    """
    N, dim = position.shape
    h = _hashes(position, cell_size, cps)
    ncell = int(np.prod(cps))
    order = torch.argsort(h, stable=True)
    sorted_h = h[order]
    slot = sorted_h * capacity + torch.arange(N, dtype=torch.int64) % capacity
    buf = torch.full((ncell * capacity,), N, dtype=torch.int64)
    ok = (slot >= 0) & (slot < ncell * capacity)
    buf[slot[ok]] = order[ok]
    inb = (h >= 0) & (h < ncell)
    occ = torch.bincount(h[inb], minlength=ncell)
    overflow = bool(int(occ.max()) > capacity)
    shape = tuple(int(c) for c in cps[::-1]) + (capacity,)
    return buf.reshape(shape), overflow


def _shift_array(arr, dindex):
    """``shift_array`` (jax_md/partition.py:202-224): periodic roll of cells."""
    for axis, d in enumerate(dindex):
        if d < 0:
            arr = torch.roll(arr, -1, dims=axis)
        elif d > 0:
            arr = torch.roll(arr, 1, dims=axis)
    return arr


def cell_candidates(buf, N, dim):
    """``cell_list_candidate_fn`` (jax_md/partition.py:832-856).

    Each particle's candidates: its own cell's slots, then the slots of the
    3^d - 1 periodically shifted cells in ``onp.ndindex`` order (:190-192).
    """
    cells = [buf]
    for dindex in itertools.product((-1, 0, 1), repeat=dim):
        if all(d == 0 for d in dindex):
            continue
        cells.append(_shift_array(buf, dindex))
    cat = torch.cat(cells, dim=-1)                 # (*cells, 3^d * cap)
    cap = buf.shape[-1]
    ids = buf.reshape(-1)                           # particle id per slot
    rows = cat.reshape(-1, cat.shape[-1]).repeat_interleave(cap, dim=0)
    out = torch.zeros((N + 1, cat.shape[-1]), dtype=torch.int64)
    out[ids] = rows
    return out[:-1]


def prune_sparse(position, cand, metric, cutoff_sq, mask_self, chunk=4096):
    """``prune_neighbor_list_sparse`` (jax_md/partition.py:885-909).

    Senders are the candidate rows, receivers the candidates; an edge is kept
    when ``metric(r[sender], r[receiver]) < cutoff_sq`` (strict) and the
    receiver is a real particle. Returns the compacted (receiver, sender)
    arrays in sender-major order and the occupancy.
    """
    N = position.shape[0]
    cut = torch.as_tensor(cutoff_sq, dtype=position.dtype)
    recv_all, send_all = [], []
    for s0 in range(0, N, chunk):
        c = cand[s0:s0 + chunk]
        if mask_self:  # mask_self_fn (:858-863)
            rows = torch.arange(s0, s0 + c.shape[0])[:, None]
            c = torch.where(c == rows, torch.full_like(c, N), c)
        send = torch.arange(s0, s0 + c.shape[0])[:, None].expand_as(c).reshape(-1)
        recv = c.reshape(-1)
        valid = recv < N
        rr = torch.where(valid, recv, torch.zeros_like(recv))
        d2 = space.square_distance(metric(position[send], position[rr]))
        keep = (d2 < cut) & valid
        recv_all.append(recv[keep])
        send_all.append(send[keep])
    recv = torch.cat(recv_all) if recv_all else torch.zeros(0, dtype=torch.int64)
    send = torch.cat(send_all) if send_all else torch.zeros(0, dtype=torch.int64)
    return recv, send


@dataclass
class NeighborList:
    """``NeighborList`` (jax_md/partition.py:620-671), sparse format."""

    idx: torch.Tensor
    reference_position: torch.Tensor
    error: int
    cell_list_capacity: int
    max_occupancy: int
    occupancy: int

    @property
    def did_buffer_overflow(self):
        return bool(self.error & (NEIGHBOR_LIST_OVERFLOW | CELL_LIST_OVERFLOW))


class NeighborListFns:
    """``neighbor_list(...)`` for the ``jaxmd_vmap`` backend, sparse format.

    Restates jax_md/partition.py:723-1026 with ``dr_threshold`` support for the
    rebuild test (:1010-1018). ``dtype`` is the run dtype.
    """

    def __init__(self, box, r_cutoff, dtype, dr_threshold=0.0,
                 capacity_multiplier=1.25, mask_self=True):
        self.box = np.asarray(box, dtype=np.float64).reshape(-1)
        self.dim = self.box.size
        self.dtype = dtype
        self.mask_self = mask_self
        self.capacity_multiplier = capacity_multiplier
        f = _np_dtype(dtype)
        cut = f(r_cutoff) + f(dr_threshold)
        self.cutoff_sq = f(cut * cut)
        self.threshold_sq = f((f(dr_threshold) / f(2)) ** 2)
        self.cell_size, self.cps, self.use_cells = cell_dimensions(self.box, cut, dtype)
        side = torch.as_tensor(self.box, dtype=dtype)
        self.space = space.Periodic(side)

    def _build(self, position, cell_capacity, max_occupancy, err):
        N = position.shape[0]
        if self.use_cells:
            if cell_capacity is None:
                cell_capacity = estimate_cell_capacity(position, self.cell_size, self.cps,
                                                       self.capacity_multiplier)
            buf, cl_over = cell_list_ids(position, self.cell_size, self.cps, cell_capacity)
            if cl_over:
                err |= CELL_LIST_OVERFLOW
            cand = cell_candidates(buf, N, self.dim)
        else:
            cand = torch.arange(N)[None, :].expand(N, N)
        recv, send = prune_sparse(position, cand, self.space.displacement,
                                  self.cutoff_sq, self.mask_self)
        occupancy = int(recv.numel())
        if max_occupancy is None:
            f = _np_dtype(self.dtype)
            max_occupancy = int(f(occupancy) * f(self.capacity_multiplier))
            max_occupancy = min(max_occupancy, int(cand.numel()))
            limit = N * (N - 1) if self.mask_self else N * N
            max_occupancy = min(max_occupancy, limit)
        idx = torch.full((2, max_occupancy), N, dtype=torch.int64)
        k = min(occupancy, max_occupancy)
        idx[0, :k] = recv[:k]
        idx[1, :k] = send[:k]
        if occupancy > max_occupancy:
            err |= NEIGHBOR_LIST_OVERFLOW
        return NeighborList(idx, position.clone(), err, cell_capacity,
                            max_occupancy, occupancy)

    def allocate(self, position, **kwargs):
        return self._build(position, None, None, 0)

    def update(self, position, nbrs, **kwargs):
        d2 = space.square_distance(self.space.displacement(position, nbrs.reference_position))
        if bool((d2 > torch.as_tensor(self.threshold_sq, dtype=position.dtype)).any()):
            return self._build(position, nbrs.cell_list_capacity, nbrs.max_occupancy,
                               nbrs.error)
        return nbrs


def canonical_edges(idx, N):
    """Real edges sorted by receiver then stably by sender.

    The comparison used by the reference's golden test
    (tests/test_neighbors.py:77-82).
    """
    idx = torch.as_tensor(idx)
    real = idx[:, idx[0] < N]
    o = torch.argsort(real[0], stable=True)
    real = real[:, o]
    o = torch.argsort(real[1], stable=True)
    return real[:, o]


# ---------------------------------------------------------------- matscipy backend
def matscipy_edges(position, num_particles, box, r_cutoff, mask_self):
    """The edge list of the reference's matscipy backend (jax_sph/partition.py:
    356-482) for ``position[:num_particles]``: matscipy's ``neighbour_list("ij",
    cutoff, positions, cell=diag(box), pbc=True)`` -- every ordered pair i != j
    whose distance between nearest periodic images, in float64 from the float32
    positions, is below the cutoff -- with the self edges ``(arange(n),
    arange(n))`` in front when ``mask_self`` is off. matscipy (not installed
    here) orders the pairs by i; within an i they are taken in ascending j.
    Returns an int64 (2, E) tensor."""
    n = int(num_particles)
    r = torch.as_tensor(position)[:n].to(torch.float64)
    side = torch.as_tensor(np.asarray(box, dtype=np.float64))
    d = r[:, None, :] - r[None, :, :]
    d = d - side * torch.round(d / side)
    within = (d * d).sum(-1) < float(r_cutoff) ** 2
    within.fill_diagonal_(False)
    i, j = torch.nonzero(within, as_tuple=True)  # row-major: by i, then j
    pairs = torch.stack([i, j])
    if mask_self:
        return pairs
    ar = torch.arange(n)
    return torch.cat([torch.stack([ar, ar]), pairs], dim=1)


def matscipy_capacity(n_edges, num_particles, num_particles_max, capacity_multiplier=1.25,
                      extra_capacity=0):
    """``allocate``'s list size: round(E * multiplier * N_max / n + extra) (:458-463)."""
    factor = capacity_multiplier * num_particles_max / num_particles
    return round(n_edges * factor + extra_capacity)


def matscipy_idx(edges, capacity, pad):
    """The (2, capacity) list: truncated, or padded with ``pad`` (:399-404, :464-466)."""
    out = torch.full((2, int(capacity)), int(pad), dtype=torch.int64)
    k = min(int(capacity), edges.shape[1])
    out[:, :k] = edges[:, :k]
    return out, edges.shape[1] > capacity
