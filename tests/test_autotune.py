"""Host logic of the launch-shape autotuner, without a GPU.

A fake engine stands in for ``_lib.Engine``: it reports a fixed step time per
block size, so the tests check which block the tuner keeps, what it writes to
its JSON cache, and that a cache hit sets the block without timing anything.
"""

import json
import os

from jaxsph_gb300 import _lib, autotune


class FakeEngine:
    def __init__(self, ms_per_step, n=40_000, cases=2):
        self.config = _lib.SphConfig()
        self.config.dim = 2
        self.cases = [object()] * cases
        self.n = n
        self.ms = ms_per_step
        self.block = None
        self.history = []

    def set_block_size(self, b):
        self.block = b
        self.history.append(b)

    def profile(self, steps):
        return [self.ms.get(self.block, 1.0)] * steps


def test_tune_picks_the_fastest_block_and_caches_it(tmp_path, monkeypatch):
    monkeypatch.setenv("JAXSPH_GB300_CACHE", str(tmp_path))
    eng = FakeEngine({64: 0.30, 128: 0.20, 256: 0.25})
    best, times = autotune.tune(eng, steps=3)
    assert best == 128 and eng.block == 128
    assert set(times) == set(autotune.CANDIDATES)
    assert abs(times[128] - 0.60) < 1e-12
    with open(os.path.join(str(tmp_path), "autotune.json")) as f:
        db = json.load(f)
    assert db[autotune.key(eng)]["block"] == 128

    # a second engine with the same key takes the cached block without timing
    eng2 = FakeEngine({64: 0.01})
    eng2.profile = None  # any timing call would fail
    best2, times2 = autotune.tune(eng2)
    assert best2 == 128 and eng2.history == [128]
    assert times2 == times


def test_cache_key_separates_configurations():
    a = FakeEngine({}, n=1000)
    b = FakeEngine({}, n=40_000)
    c = FakeEngine({}, n=1000, cases=1)
    assert len({autotune.key(a), autotune.key(b), autotune.key(c)}) == 3
    # particle counts in the same power-of-two bucket share an entry
    assert autotune.key(FakeEngine({}, n=1000)) == autotune.key(FakeEngine({}, n=1100))


def test_unwritable_cache_only_loses_the_cache(tmp_path, monkeypatch):
    blocker = tmp_path / "file"
    blocker.write_text("")
    monkeypatch.setenv("JAXSPH_GB300_CACHE", str(blocker / "sub"))
    eng = FakeEngine({64: 0.1, 128: 0.2, 256: 0.3})
    best, _ = autotune.tune(eng, steps=1)
    assert best == 64 and eng.block == 64


def test_tune_without_cache_always_times(tmp_path, monkeypatch):
    monkeypatch.setenv("JAXSPH_GB300_CACHE", str(tmp_path))
    eng = FakeEngine({64: 0.3, 128: 0.2, 256: 0.1})
    best, _ = autotune.tune(eng, steps=1, use_cache=False)
    assert best == 256
    assert not os.path.exists(os.path.join(str(tmp_path), "autotune.json"))
