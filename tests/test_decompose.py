"""Slab decomposition, host logic on CPU: selection, halo exchange and
migration between gloo ranks (world size 2 and 3).

Every rank must receive exactly the particles the decomposition assigns to
its halo, computed here from the whole state, and after a move every
particle must be owned by exactly one rank, the one whose slab holds it.
"""

import os
import socket
import sys

import numpy as np
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _setup(case="tgv"):
    sys.path.insert(0, os.path.join(ROOT, "jax-sph_gb300"))
    from jaxsph_gb300 import cases

    if case == "ht":
        # heat transfer: walls, and the temperature fields ride along
        s = cases.heat_transfer(dx=0.05)
        g = torch.Generator().manual_seed(4)
        s.state["T"] = 1.0 + torch.rand(s.n, generator=g)
        s.state["dTdt"] = torch.randn(s.n, generator=g)
        return s
    s = cases.tgv(dim=3, dx=2 * np.pi / 12)
    g = torch.Generator().manual_seed(3)
    L = 2 * np.pi
    r = s.state["r"].double() + (torch.rand(s.state["r"].shape, generator=g) - 0.5) * 0.3
    s.state["r"] = torch.remainder(r, L).float()
    return s


def _worker(rank, ws, port, out, case="tgv"):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    from jaxsph_gb300 import decompose as dc
    from jaxsph_gb300.solver import prepare_state

    s = _setup(case)
    slabs = dc.DistributedSlabs(s, device="cpu")
    whole = prepare_state(s.state, s.dim, "cpu", heat=case == "ht")
    whole.setdefault("nw", torch.zeros_like(whole["r"]))
    L = slabs.length
    x = s.state["r"][:, slabs.axis]
    owner = dc.slab_of(x, L, ws)
    ok = torch.equal(slabs.owned["gid"], torch.nonzero(owner == rank).squeeze(1))
    # halo: everything within w of this slab, from the other ranks, every
    # field the slabs exchange
    w = 0.27 * L
    local = slabs.local_state(w)
    want = torch.nonzero((owner == rank) | dc.near_slab(x, rank, ws, L, w)).squeeze(1)
    ok = ok and torch.equal(local["gid"], want)
    for f in slabs.slabs.fields:
        ok = ok and torch.equal(local[f], whole[f][want])
    # migration after a move along the slab axis
    shift = torch.zeros(s.dim)
    shift[slabs.axis] = 0.4 * L / ws
    slabs.owned["r"] = torch.remainder(slabs.owned["r"] + shift, L).float()
    slabs.migrate()
    moved = torch.remainder(s.state["r"] + shift, L).float()
    new_owner = dc.slab_of(moved[:, slabs.axis], L, ws)
    ok = ok and torch.equal(slabs.owned["gid"], torch.nonzero(new_owner == rank).squeeze(1))
    ok = ok and torch.equal(slabs.owned["r"], moved[new_owner == rank])
    for f in slabs.slabs.fields:
        if f != "r":
            ok = ok and torch.equal(slabs.owned[f], whole[f][new_owner == rank])
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(ws)]
    dist.all_gather(counts, torch.tensor([slabs.owned["gid"].numel()]))
    ok = ok and int(sum(c.item() for c in counts)) == s.n
    out[rank] = bool(ok)
    dist.destroy_process_group()


def _run(ws, case="tgv"):
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, out, case)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {r: True for r in range(ws)}


def test_exchange_and_migration_two_ranks():
    _run(2)


def test_exchange_and_migration_three_ranks():
    _run(3)


def test_exchange_and_migration_of_heat_fields_two_ranks():
    _run(2, "ht")


def test_halo_width_covers_two_cutoffs_and_the_drift():
    sys.path.insert(0, os.path.join(ROOT, "jax-sph_gb300"))
    from jaxsph_gb300 import decompose as dc

    st = {"u": torch.tensor([[1.0, 0.0, 0.0]]), "dudt": torch.tensor([[0.0, 2.0, 0.0]]),
          "dvdt": torch.tensor([[0.0, 0.0, 4.0]])}
    d = dc.step_drift(st, 0.1, 0.05)
    assert abs(d - 0.1 * float(np.linalg.norm([1.0, 0.2, 0.2]))) < 1e-12
    assert dc.halo_width(0.5, d) > 1.0 + 2 * d
    assert dc.halo_width(0.5, d, levels=3) > 1.5 + 2 * d


def test_slab_fields_follow_the_case():
    """Heat conduction adds the temperature fields to what slabs exchange and
    keep; moving walls add the recomputed normals to what a step changes; the
    exchange matrix round-trips every field exactly."""
    sys.path.insert(0, os.path.join(ROOT, "jax-sph_gb300"))
    from jaxsph_gb300 import cases
    from jaxsph_gb300 import decompose as dc

    ht = cases.heat_transfer(dx=0.05)
    assert dc.state_fields(ht)[-4:] == ("T", "dTdt", "kappa", "Cp")
    assert dc.out_fields(ht)[-2:] == ("T", "dTdt")
    ldc = cases.lid_driven_cavity(dx=0.05, solver_name="RIE")
    assert dc.out_fields(ldc)[-1] == "nw" and "T" not in dc.state_fields(ldc)
    assert dc.state_fields(cases.tgv(dim=2, dx=0.1)) == dc.STATE_FIELDS
    fields = dc.state_fields(ht)
    g = torch.Generator().manual_seed(0)
    rows = {k: (torch.randn(v.shape, generator=g) if v.is_floating_point() else v)
            for k, v in ht.state.items() if k in fields}
    rows["gid"] = torch.arange(ht.n)
    back = dc._unpack(dc._pack(rows, fields), ht.dim, fields)
    for k in fields + ("gid",):
        assert torch.equal(back[k], rows[k]), k
