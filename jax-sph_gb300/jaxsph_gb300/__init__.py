"""jaxsph_gb300: the jax-sph per-step hot path on GB300 (sm_103a).

Drop-in modules with the reference's call signatures:

* ``space.periodic``                 (jax_sph/jax_md/space.py)
* ``partition.neighbor_list``        (jax_sph/partition.py)
* ``solver.WCSPH``                   (jax_sph/solver.py)
* ``integrator.si_euler``            (jax_sph/integrator.py)
* ``eos.TaitEoS`` / ``eos.RIEMANNEoS`` and the QSK / WC2K ``kernel`` classes

plus ``cases`` (initial states of TGV, dam break, lid-driven cavity,
Poiseuille and Couette flow), ``simulate`` (resident and batched GPU
rollouts), ``decompose`` (slab domain decomposition over GPUs) and
``io_state`` (the reference's .h5 state files and restarts).
All arithmetic runs in ``libsph_gb300.so`` (hand-written CUDA, C ABI in
``include/sph_gb300.h``); there is no CPU path.
"""

from . import eos, kernel, space  # noqa: F401
from ._build import build  # noqa: F401
from ._lib import SphError, load  # noqa: F401


def __getattr__(name):
    # modules that need torch.cuda are imported lazily
    import importlib

    if name in ("partition", "solver", "integrator", "cases", "simulate", "decompose",
                "io_state", "adjoint"):
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
