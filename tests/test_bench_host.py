"""Host logic of bench.py on CPU: the two arms print the same ``config``, and
the status word of the timed steps is decoded by the header's bit values."""

import json
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    sys.path.insert(0, ROOT)
    import bench

    return bench


class _Args:
    steps, warmup, gpus, n_side, skin = 2, 3, 1, 64, 0.1


def test_reference_arm_config_is_the_gpu_arms(capsys, monkeypatch):
    bench = _bench()
    monkeypatch.setattr(bench, "cpu_oracle_rate",
                        lambda *a, **k: (5.0e5, 2, 1.0, 262144, 3))
    bench.reference_arm(_Args(), 1, 0)
    line = json.loads(capsys.readouterr().out)
    assert line["impl"] == "reference"
    # the GPU arm prints workload_config(args, n, world size) unchanged
    assert line["config"] == bench.workload_config(_Args(), 262144, 1)
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_status_bits_match_the_header():
    bench = _bench()
    with open(os.path.join(ROOT, "include", "sph_gb300.h")) as f:
        text = f.read()
    defs = {name: int(val, 16) for name, val in
            re.findall(r"#define SPH_([A-Z_]+) (0x[0-9a-fA-F]+)u", text)}
    for bit, name in bench.STATUS_BITS.items():
        assert defs[name] == bit, name
    rep = bench.status_report(0x2 | 0x800)
    assert rep["bits"] == ["CELL_LIST_OVERFLOW", "ERR_NONFINITE"] and "note" in rep
    assert bench.status_report(0) == {"word": 0, "bits": []}
