"""GPU neighbour search vs the reference's golden lists and the float32 oracle.

Bar: bit-exact neighbour sets (canonical sort of tests/test_neighbors.py:77-82
of the reference), on the golden cases, on lattices with exact cutoff ties,
on jittered lattices and on walled boxes.
"""

import json
import os

import numpy as np
import pytest
import torch

import oracle
from jaxsph_gb300 import cases, partition, space

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "neighbors_golden.json")


def gpu_edges(box, cutoff, r, mask_self):
    disp, _ = space.periodic(box)
    fns = partition.neighbor_list(disp, box, cutoff, mask_self=mask_self,
                                  format=partition.Sparse)
    rr = torch.as_tensor(r, dtype=torch.float32).cuda()
    nb = fns.allocate(rr)
    return fns, nb, rr


def oracle_edges(box, cutoff, r, mask_self, dtype=torch.float32):
    fns = oracle.partition.NeighborListFns(box, cutoff, dtype, mask_self=mask_self)
    nb = fns.allocate(torch.as_tensor(r, dtype=dtype))
    return nb


def canon(idx, n):
    return oracle.partition.canonical_edges(torch.as_tensor(idx).long().cpu(), n)


@pytest.mark.parametrize("case", range(4))
def test_golden_lists(case):
    c = json.load(open(GOLDEN))["cases"][case]
    r = np.array(c["r"])
    fns, nb, rr = gpu_edges(np.array(c["box_size"]), c["cutoff"], r, c["mask_self"])
    n = r.shape[0]
    nb2 = fns.update(rr + 0.0, nb)
    assert not nb.did_buffer_overflow and not nb2.did_buffer_overflow
    assert torch.equal(nb.idx, nb2.idx), "allocate differs from update"
    idx = nb.idx.cpu()
    assert torch.equal(idx[0] == n, idx[1] == n), "one-sided edges"
    real = idx[:, idx[0] < n]
    self_edges = real[0] == real[1]
    if c["mask_self"]:
        assert int(self_edges.sum()) == 0
    else:
        assert len(np.unique(real[0][self_edges].numpy())) == n
    assert canon(idx, n).tolist() == c["target"]


def _lattice_cases():
    yield "tgv2d_qsk_ties", cases.tgv(dim=2)
    yield "tgv3d_wc2k_ties", cases.tgv(dim=3, dx=2 * np.pi / 20)
    yield "ldc_walls", cases.lid_driven_cavity(dx=0.04)
    yield "db_walls", cases.dam_break(dx=0.04)
    yield "pf_walls", cases.poiseuille(dx=0.05)


@pytest.mark.parametrize("name,setup", list(_lattice_cases()))
@pytest.mark.parametrize("mask_self", [False, True])
def test_lattice_sets_bit_exact(name, setup, mask_self):
    from jaxsph_gb300.kernel import make_kernel

    cutoff = make_kernel(setup.solver["kernel"], setup.dx, setup.dim).cutoff
    r = setup.state["r"]
    fns, nb, rr = gpu_edges(setup.box, cutoff, r, mask_self)
    ref = oracle_edges(setup.box, cutoff, r, mask_self)
    n = r.shape[0]
    assert nb.occupancy == ref.occupancy
    assert nb.max_occupancy == ref.max_occupancy
    assert nb.cell_list_capacity == ref.cell_list_capacity
    assert torch.equal(canon(nb.idx, n), canon(ref.idx, n))


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("dim", [2, 3])
def test_jittered_sets_bit_exact(seed, dim):
    setup = cases.tgv(dim=dim, dx=(0.02 if dim == 2 else 2 * np.pi / 24))
    g = torch.Generator().manual_seed(seed)
    r = setup.state["r"] + 0.3 * setup.dx * torch.randn(setup.state["r"].shape, generator=g)
    side = torch.as_tensor(setup.box, dtype=torch.float32)
    r = oracle.space.periodic_shift(side, setup.state["r"], r - setup.state["r"])
    from jaxsph_gb300.kernel import make_kernel

    cutoff = make_kernel(setup.solver["kernel"], setup.dx, dim).cutoff
    fns, nb, rr = gpu_edges(setup.box, cutoff, r, False)
    ref = oracle_edges(setup.box, cutoff, r, False)
    n = r.shape[0]
    assert torch.equal(canon(nb.idx, n), canon(ref.idx, n))


def test_overflow_flags_and_truncation():
    setup = cases.tgv(dim=2, dx=0.05)
    cutoff = 3 * setup.dx
    r = setup.state["r"]
    fns, nb, rr = gpu_edges(setup.box, cutoff, r, False)
    assert not nb.did_buffer_overflow
    # squeeze the particles towards the origin: cells and the edge list overflow
    rr2 = (rr * 0.5).contiguous()
    nb2 = fns.update(rr2, nb)
    assert nb2.did_buffer_overflow
    assert nb2.error.code & partition.PEC.NEIGHBOR_LIST_OVERFLOW
    assert nb2.error.code & partition.PEC.CELL_LIST_OVERFLOW
    assert nb2.idx.shape == nb.idx.shape  # fixed capacity, truncated
    # re-allocation (simulate.py:120-128) fits again and matches the oracle
    nb3 = fns.allocate(rr2)
    assert not nb3.did_buffer_overflow
    ref = oracle_edges(setup.box, cutoff, rr2.cpu(), False)
    assert torch.equal(canon(nb3.idx, r.shape[0]), canon(ref.idx, r.shape[0]))


def test_update_skips_rebuild_when_nothing_moved():
    setup = cases.tgv(dim=2, dx=0.05)
    fns, nb, rr = gpu_edges(setup.box, 3 * setup.dx, setup.state["r"], False)
    assert fns.update(rr.clone(), nb) is nb
