"""Host logic of ``Simulation.run``: the reference driver's overflow protocol
(jax_sph/simulate.py:120-128) and status polling, with a fake engine (no GPU).

The fake engine records the calls the rollout makes and reports a scripted
status word after each batch of steps, so the tests check when the status is
polled, that an overflow re-allocates the capacities (and clears the word),
that a CUDA or argument error raises, and that other bits reach the caller.
"""

import pytest

from jaxsph_gb300 import _lib, simulate


class FakeEngine:
    def __init__(self, statuses):
        self.statuses = list(statuses)
        self.calls = []
        self.word = 0

    def step(self, k):
        self.calls.append(("step", k))
        if self.statuses:
            self.word |= self.statuses.pop(0)

    def read_status(self, clear=False):
        self.calls.append(("read", clear))
        w = self.word
        if clear:
            self.word = 0
        return w

    def nl_allocate(self):
        self.calls.append(("allocate",))
        return "capacity"


def _sim(statuses):
    sim = object.__new__(simulate.Simulation)
    sim.engine = FakeEngine(statuses)
    sim.steps_done = 0
    sim.capacity = None
    return sim


def test_run_polls_every_check_every_steps():
    sim = _sim([0, 0, 0])
    assert sim.run(25, check_every=10) == 0
    steps = [c[1] for c in sim.engine.calls if c[0] == "step"]
    assert steps == [10, 10, 5] and sim.steps_done == 25
    # one poll after each batch
    assert sum(1 for c in sim.engine.calls if c[0] == "read") == 3


def test_overflow_reallocates_and_is_reported():
    sim = _sim([0, _lib.NEIGHBOR_LIST_OVERFLOW, 0])
    seen = sim.run(30, check_every=10)
    assert seen & _lib.NEIGHBOR_LIST_OVERFLOW
    assert sim.capacity == "capacity"
    alloc = sim.engine.calls.index(("allocate",))
    # the re-allocation follows the second batch and the word is cleared after it
    assert sim.engine.calls[alloc - 2:alloc] == [("step", 10), ("read", True)]
    assert sim.engine.calls[alloc + 1] == ("read", True)
    assert sim.engine.word == 0


def test_cell_list_overflow_also_reallocates():
    sim = _sim([_lib.CELL_LIST_OVERFLOW])
    assert sim.run(5) & _lib.CELL_LIST_OVERFLOW
    assert ("allocate",) in sim.engine.calls


@pytest.mark.parametrize("bit", [_lib.ERR_CUDA, _lib.ERR_INVALID_ARG])
def test_device_errors_raise(bit):
    sim = _sim([0, bit])
    with pytest.raises(_lib.SphError):
        sim.run(20, check_every=10)


def test_other_bits_reach_the_caller_without_reallocation():
    sim = _sim([_lib.ERR_NONFINITE | _lib.WARN_BOX_EDGE])
    seen = sim.run(3)
    assert seen & _lib.ERR_NONFINITE and seen & _lib.WARN_BOX_EDGE
    assert ("allocate",) not in sim.engine.calls


def test_zero_steps_still_report_the_status_word():
    sim = _sim([])
    sim.engine.word = _lib.WARN_BOX_EDGE
    assert sim.run(0) == _lib.WARN_BOX_EDGE
    assert not any(c[0] == "step" for c in sim.engine.calls)
