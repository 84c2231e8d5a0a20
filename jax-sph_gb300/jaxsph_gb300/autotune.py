"""Launch-shape autotuner for the forward passes, with a JSON cache.

The density, wall and force passes run one thread per particle; their block
size trades occupancy against tail effects and depends on the particle count,
dimension and solver. ``tune`` times whole steps of an ``Engine`` for every
candidate block size with CUDA events (``sph_profile_step``), keeps the
fastest, and caches the choice per (GPU, dimension, kernel, solver, particle
count bucket) in ``$JAXSPH_GB300_CACHE`` (default
``~/.cache/jaxsph_gb300/autotune.json``). Results do not depend on the block
size, so a tuned engine computes exactly what an untuned one does.
"""

import json
import math
import os

import torch

CANDIDATES = (64, 128, 256)


def cache_path():
    base = os.environ.get("JAXSPH_GB300_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "jaxsph_gb300"))
    return os.path.join(base, "autotune.json")


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(db, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home only loses the cache, not the tuning


def key(engine):
    cfg = engine.config
    bucket = int(round(math.log2(max(engine.n, 1))))
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{name}|d{cfg.dim}|k{cfg.kernel}|s{cfg.solver}|e{cfg.is_rho_evol}|" \
           f"w{cfg.is_bc_trick}|c{len(engine.cases)>1}|n2^{bucket}"


def tune(engine, steps=6, candidates=CANDIDATES, use_cache=True):
    """Pick and set the fastest block size; returns (block, {block: ms per step}).

    The timing runs real steps (the engine's state advances by
    ``steps * (len(candidates) + 1)`` steps); tune before loading the state
    to be simulated, or on a copy.
    """
    db = _load() if use_cache else {}
    k = key(engine)
    if use_cache and k in db:
        engine.set_block_size(db[k]["block"])
        return db[k]["block"], {int(b): t for b, t in db[k]["ms"].items()}
    times = {}
    engine.profile(1)  # warm-up: first step of a freshly loaded state
    for b in candidates:
        engine.set_block_size(b)
        times[b] = float(sum(engine.profile(steps)))
    best = min(times, key=times.get)
    engine.set_block_size(best)
    if use_cache:
        db[k] = {"block": best, "ms": {str(b): t for b, t in times.items()}}
        _store(db)
    return best, times
