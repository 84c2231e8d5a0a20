"""The allocation-free neighbour-list entry point (sph_nl_edges_noalloc).

It serves callers that cannot call cudaMalloc -- a host framework that owns the
whole device memory pool, or code that must not allocate after start-up -- by
keeping its scratch in one fixed device array. Its edge lists must equal those
of the handle-based entry point (sph_nl_allocate + sph_nl_edges) exactly
(integer output: bit-exact), on consecutive calls that reuse the same array
with different sizes. This file is collected last on purpose.
"""

import ctypes

import numpy as np
import pytest
import torch

from jaxsph_gb300 import _lib, cases, partition, space
from jaxsph_gb300.kernel import make_kernel

pytestmark = pytest.mark.gpu


def call_noalloc(lib, r, box, cutoff, mask_self, capacity):
    dim = r.shape[1]
    boxd = (ctypes.c_double * 3)(*([float(x) for x in box] + [1.0] * (3 - len(box))))
    idx = torch.full((2, capacity), -7, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.sph_nl_edges_noalloc(dim, boxd, float(cutoff), int(mask_self), r.data_ptr(),
                                  r.shape[0], idx.data_ptr(), capacity, cnt.data_ptr(),
                                  st.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.sph_last_error()
    torch.cuda.synchronize()
    return idx, int(cnt.item()), int(st.item())


def _inputs():
    s2 = cases.tgv(dim=2)  # lattice with exact cutoff ties
    s3 = cases.tgv(dim=3, dx=2 * np.pi / 20)
    g = torch.Generator().manual_seed(3)
    side = torch.as_tensor(s3.box, dtype=torch.float32)
    r3 = torch.remainder(s3.state["r"] + 0.3 * s3.dx * torch.randn(s3.state["r"].shape,
                                                                  generator=g), side)
    return [(r3, s3.box, make_kernel("WC2K", s3.dx, 3).cutoff, True),
            (s2.state["r"], s2.box, make_kernel("QSK", s2.dx, 2).cutoff, False),
            (r3, s3.box, make_kernel("WC2K", s3.dx, 3).cutoff, False)]


def test_noalloc_equals_handle_path_on_consecutive_calls():
    lib = _lib.load()
    for r, box, cutoff, mask_self in _inputs():
        r = r.to(torch.float32).cuda().contiguous()
        disp, _ = space.periodic(box)
        fns = partition.neighbor_list(disp, box, cutoff, mask_self=mask_self)
        nb = fns.allocate(r)
        idx, count, status = call_noalloc(lib, r, box, cutoff, mask_self, nb.max_occupancy)
        assert status & 0xFF == 0
        assert count == nb.occupancy
        assert torch.equal(idx, nb.idx)


def test_noalloc_equals_handle_path_at_its_limits():
    """65,536 particles in 65,536 cells (2D, cutoff = spacing, jittered
    lattice): every region of the fixed array is used to its end."""
    lib = _lib.load()
    n_side = 256
    dx = 1.0 / n_side
    box = np.array([1.0, 1.0])
    g = torch.Generator().manual_seed(5)
    ax = (torch.arange(n_side, dtype=torch.float64) + 0.5) * dx
    yy, xx = torch.meshgrid(ax, ax, indexing="ij")
    r = torch.stack([xx.reshape(-1), yy.reshape(-1)], 1)
    r = torch.remainder(r + 0.2 * dx * torch.randn(r.shape, generator=g, dtype=torch.float64),
                        1.0).to(torch.float32)
    r = torch.where(r >= 1.0, torch.zeros_like(r), r).cuda().contiguous()
    assert r.shape[0] == 65536
    cutoff = dx
    disp, _ = space.periodic(box)
    fns = partition.neighbor_list(disp, box, cutoff, mask_self=False)
    nb = fns.allocate(r)
    for _ in range(2):
        idx, count, status = call_noalloc(lib, r, box, cutoff, False, nb.max_occupancy)
        assert status & 0xFF == 0
        assert count == nb.occupancy
        assert torch.equal(idx, nb.idx)


def test_noalloc_rejects_sizes_beyond_its_array():
    lib = _lib.load()
    n = 65537
    r = torch.rand((n, 2), device="cuda")
    boxd = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    idx = torch.empty((2, 8), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = lib.sph_nl_edges_noalloc(2, boxd, 0.01, 0, r.data_ptr(), n, idx.data_ptr(), 8,
                                  cnt.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.ERR_INVALID_ARG
    assert b"65536" in lib.sph_last_error()
