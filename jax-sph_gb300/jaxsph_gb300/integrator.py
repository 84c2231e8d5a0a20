"""Semi-implicit Euler with transport velocity: drop-in for ``jax_sph.integrator.si_euler``.

``advance(dt, state, neighbors) -> (state, neighbors)`` performs, in one GPU
pass chain (integrator.py:22-56): ``u += dt*dudt``, ``v = u + tvf*dt/2*dvdt``,
``r = shift(r, dt*v)``, neighbour-list rebuild (fused with the kick-drift into
the cell binning), the WCSPH forward pass and ``bc_fn``.

The fused chain needs the case's callables in a form the kernels evaluate:
``g_ext_fn`` and ``nw_fn`` as the package's descriptors (``cases.GExt``,
``cases.WallNormals``; ``bc_fn`` may be any callable). With any other
``g_ext_fn`` or ``nw_fn`` -- a user's own function of the positions -- the step
is composed the way the reference composes it: the kick-drift as float32
tensor arithmetic on the GPU, ``nw_fn(r)``, the neighbour-list update, the
forward pass (which evaluates ``g_ext_fn`` on the drifted positions and hands
the result to the kernels) and ``bc_fn``, each a call of its own.
"""

import torch

from . import _lib


def si_euler(tvf, model, shift_fn, bc_fn, nw_fn):
    """Return ``advance(dt, state, neighbors)`` for a ``WCSPH`` forward ``model``."""
    solver = getattr(model, "__wcsph__", None)
    if solver is None:
        raise NotImplementedError("model must be WCSPH(...).forward_wrapper() of jaxsph_gb300")
    tvf = float(tvf)
    composed = (solver.g_spec()["kind"] == _lib.GEXT_ARRAY
                or (nw_fn is not None and getattr(nw_fn, "spec", None) is None))

    def advance_composed(dt, state, neighbors):
        # integrator.py:26-53, step by step
        dev = torch.device("cuda")
        st = {k: (torch.as_tensor(v).to(dev) if v is not None else v)
              for k, v in state.items()}
        st["u"] = st["u"] + 1.0 * dt * st["dudt"]
        st["v"] = st["u"] + tvf * 0.5 * dt * st["dvdt"]
        st["r"] = shift_fn(st["r"], 1.0 * dt * st["v"])
        if nw_fn is not None:
            st["nw"] = torch.as_tensor(nw_fn(st["r"])).to(dev, torch.float32)
        neighbors = neighbors.update(st["r"], num_particles=(st["tag"] != _lib.TAG_PAD).sum())
        st = model(st, neighbors)
        if bc_fn is not None:
            st = bc_fn(st)
        return st, neighbors

    def advance(dt, state, neighbors):
        if composed:
            return advance_composed(float(dt), state, neighbors)
        return solver.advance(float(dt), tvf, state, neighbors, bc_fn, nw_fn)

    advance.__si_euler__ = (solver, tvf, bc_fn)
    return advance
