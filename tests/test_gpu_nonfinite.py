"""Non-finite positions fed from the host: the step returns and reports it.

A NaN or infinite position is parked in cell 0 by the binning, and every
comparison with it is false, so it enters no other particle's neighbour set
and no loop bound is derived from it (the cell walks are clamped to the
receiver's cell neighbourhood). The kick's reference-cell test and the
binning set SPH_ERR_NONFINITE in the status word; the call returns normally
and the finite particles' results stay finite. (The reference itself has no
such signal -- its error word holds the partition overflow bits,
jax_md/partition.py:453-457 -- so this is an addition, not parity.)
"""

import math

import pytest
import torch

from jaxsph_gb300 import _lib, cases, simulate, solver

pytestmark = pytest.mark.gpu

CASES = {
    # 8 x 8 particles, fewer than 3 reference cells per side: the generic passes
    "tgv2d_64": lambda: cases.tgv(dim=2, dx=0.125),
    # 16 x 16 particles, the fast test and the lean passes
    "tgv2d_256": lambda: cases.tgv(dim=2, dx=1.0 / 16),
}
BAD = (3, 7)


def bad_state(setup):
    st = {k: v.clone() for k, v in setup.state.items()}
    st["r"][BAD[0]] = float("nan")
    st["r"][BAD[1], 0] = math.inf
    return st


def good_mask(n):
    m = torch.ones(n, dtype=torch.bool)
    m[list(BAD)] = False
    return m


@pytest.mark.parametrize("name", list(CASES))
def test_resident_step_reports_nonfinite(name):
    setup = CASES[name]()
    sim = simulate.Simulation(setup)
    sim.load([bad_state(setup)])
    code = sim.run(3)
    assert code & _lib.ERR_NONFINITE
    st = sim.state()[0]
    good = good_mask(setup.n).cuda()
    for k in ("r", "u", "rho", "dudt"):
        assert torch.isfinite(st[k][good]).all(), k


@pytest.mark.parametrize("name", list(CASES))
def test_drop_in_step_from_pinned_host_reports_nonfinite(name):
    setup = CASES[name]()
    wc = simulate.make_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    case = wc.sph_case(fns, setup.n, dt=setup.dt, tvf=setup.tvf, bc=setup.bc_fn.spec)
    e = wc.engine(fns, case)
    e.nl_set_capacity(2 ** 31 - 1, 2 ** 40)
    host = {k: v.to(torch.int32 if k == "tag" else torch.float32).contiguous().pin_memory()
            for k, v in bad_state(setup).items() if k in solver.STATE_KEYS}
    keys = solver.OUT_KEYS_SUMMATION
    out, status, vout = _lib.host_outputs(setup.n, setup.dim, keys)
    e.advance(host, out, None, 0.0, vout=vout, status=status)  # returns with host results
    assert int(status.item()) & _lib.ERR_NONFINITE
    good = good_mask(setup.n)
    for k in ("r", "u", "rho", "dudt"):
        assert torch.isfinite(out[k][good]).all(), k
