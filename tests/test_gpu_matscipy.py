"""The matscipy backend and padded states (jax_sph/partition.py:356-482,
Tag.PAD_VALUE): a state padded to num_particles_max with tag -1 particles.

The edge list equals the oracle's restatement of matscipy (float64 distances
below the cutoff, self edges first, pairs by first index), with its capacity
rule, truncation and padding values; padding particles take part in no
neighbour set, so a padded drop-in step leaves the real particles exactly as
the unpadded step does.
"""

import numpy as np
import pytest
import torch

import oracle
from jaxsph_gb300 import _lib, cases, integrator, partition, simulate, space

pytestmark = pytest.mark.gpu


def padded_positions(n, n_max, box, seed):
    g = torch.Generator().manual_seed(seed)
    r = torch.rand((n_max, len(box)), generator=g, dtype=torch.float64) * torch.tensor(box)
    return r.float()


@pytest.mark.parametrize("mask_self", [True, False])
def test_edges_match_the_oracle(mask_self):
    box = (1.0, 0.8)
    n, n_max = 500, 640
    r = padded_positions(n, n_max, box, seed=1)
    disp, _ = space.periodic(np.array(box))
    fns = partition.neighbor_list(disp, np.array(box), 0.09, backend="matscipy",
                                  mask_self=mask_self, num_particles_max=n_max)
    nb = fns.allocate(r, num_particles=n)
    want = oracle.partition.matscipy_edges(r, n, box, 0.09, mask_self)
    cap = oracle.partition.matscipy_capacity(want.shape[1], n, n_max)
    assert nb.max_occupancy == cap
    idx_want, _ = oracle.partition.matscipy_idx(want, cap, n)
    assert torch.equal(nb.idx.cpu().long(), idx_want)
    # update: new positions, the same capacity, padded with num_particles_max
    r2 = padded_positions(n, n_max, box, seed=2)
    nb2 = nb.update(r2, num_particles=n)
    want2 = oracle.partition.matscipy_edges(r2, n, box, 0.09, mask_self)
    idx2, over = oracle.partition.matscipy_idx(want2, cap, n_max)
    assert torch.equal(nb2.idx.cpu().long(), idx2)
    assert nb2.did_buffer_overflow == over
    # fewer particles count: the list shrinks, padding grows
    nb3 = nb.update(r2, num_particles=300)
    want3 = oracle.partition.matscipy_edges(r2, 300, box, 0.09, mask_self)
    idx3, _ = oracle.partition.matscipy_idx(want3, cap, n_max)
    assert torch.equal(nb3.idx.cpu().long(), idx3)


def test_float64_membership_at_exact_lattice_distances():
    # lattice spacing 0.1, cutoff 0.3: pairs three spacings apart sit on the
    # cutoff, decided by the float64 distance of the float32 positions
    setup = cases.tgv(dim=2, dx=0.1)
    r = setup.state["r"]
    disp, _ = space.periodic(setup.box)
    for cut in (0.3, 0.2, np.sqrt(0.08)):
        fns = partition.neighbor_list(disp, setup.box, cut, backend="matscipy",
                                      mask_self=False, num_particles_max=setup.n)
        nb = fns.allocate(r, num_particles=setup.n)
        want = oracle.partition.matscipy_edges(r, setup.n, setup.box, cut, False)
        assert nb.occupancy == want.shape[1]
        assert torch.equal(nb.idx.cpu().long()[:, :want.shape[1]], want)


def test_padding_does_not_touch_the_real_particles():
    setup = cases.tgv(dim=2, dx=0.05)
    n = setup.n
    n_pad = 37
    pad = {k: v.clone() for k, v in setup.state.items()}
    g = torch.Generator().manual_seed(4)
    for k, v in setup.state.items():
        extra = v[:n_pad].clone()
        if k == "r":  # padding on top of real particles, to be ignored
            extra = v[torch.randint(0, n, (n_pad,), generator=g)] + 1e-3
        if k == "tag":
            extra = torch.full((n_pad,), _lib.TAG_PAD, dtype=v.dtype)
        pad[k] = torch.cat([v, extra])
    results = []
    for st, n_max in ((setup.state, n), (pad, n + n_pad)):
        wc = simulate.make_solver(setup)
        disp, shift = setup.space()
        fns = partition.neighbor_list(disp, setup.box, wc._kernel_fn.cutoff, backend="matscipy",
                                      mask_self=False, num_particles_max=n_max)
        adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
        s = {k: v.cuda() for k, v in st.items()}
        nb = fns.allocate(s["r"], num_particles=n)
        for _ in range(4):
            s, nb = adv(setup.dt, s, nb)
        assert not nb.did_buffer_overflow
        results.append(s)
    for k in ("r", "u", "v", "rho", "p", "dudt", "dvdt"):
        assert torch.equal(results[0][k], results[1][k][:n]), k
    # the step's list of the padded state counts only real particles
    assert int(nb.occupancy) == int(fns.allocate(results[0]["r"], num_particles=n).occupancy)
