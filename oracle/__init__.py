"""CPU oracle for the jax-sph per-step hot path -- TEST INFRASTRUCTURE ONLY.

This package is a PyTorch-CPU restatement, op for op, of the JAX program that
jax-sph runs per step (cell-list neighbour search, WCSPH forward pass,
semi-implicit-Euler kick-drift). It exists to check the CUDA product path; it is
never part of it. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` may import it, and only as the checker.

Every function cites the reference file and line range it restates (paths are
relative to the tumaer/jax-sph project root).

Pinning: the neighbour search is pinned against the four golden edge lists of
the reference's own ``tests/test_neighbors.py:89-121`` (fixture
``tests/golden/neighbors_golden.json``), and the kernels against the
normalisation test of ``tests/test_kernel.py:17-44``. JAX itself is not
installable in this environment, so per-element density/force values are
pinned only by this restatement plus the analytical Poiseuille-flow solution
of ``tests/test_pf2d.py:14-41``.

The restatement runs in float64 (the reference default dtype,
``jax_sph/defaults.py:20``) and in float32, the dtype of the GPU product path.
"""

from . import space, partition, sph  # noqa: F401
