"""The product path has no CPU fallback and never reaches the oracle.

* Without a CUDA device the drop-in neighbour search raises instead of
  computing anything on the host.
* No module of the package, nor ``bench.py``'s GPU arm helpers, imports the
  oracle: the oracle is test infrastructure only (the tests, ``smoke()`` and
  the bench's CPU-baseline leg use it as the checker).
"""

import ast
import os

import pytest
import torch

from jaxsph_gb300 import cases, partition, solver

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "jax-sph_gb300", "jaxsph_gb300")


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_neighbor_search_raises_without_a_gpu():
    setup = cases.tgv(dim=2, dx=0.05)
    disp, _ = setup.space()
    wc = solver.WCSPH(disp, setup.eos, setup.g_ext_fn, setup.dx, 2, setup.dt, setup.c_ref,
                      kernel="QSK")
    fns = partition.neighbor_list(disp, setup.box, wc._kernel_fn.cutoff, mask_self=False)
    with pytest.raises(RuntimeError):
        fns.allocate(setup.state["r"])


def _imports(path):
    tree = ast.parse(open(path).read(), filename=path)
    names = set()
    for node in ast.walk(tree):
        if isinstance(node, ast.Import):
            names.update(a.name.split(".")[0] for a in node.names)
        elif isinstance(node, ast.ImportFrom) and node.module and node.level == 0:
            names.add(node.module.split(".")[0])
    return names


def test_package_never_imports_the_oracle():
    files = [os.path.join(PKG, f) for f in sorted(os.listdir(PKG)) if f.endswith(".py")]
    assert len(files) > 10
    for f in files:
        assert "oracle" not in _imports(f), f"{os.path.basename(f)} imports the oracle"
        assert "oracle_setup" not in _imports(f)
