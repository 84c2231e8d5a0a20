"""Semi-implicit Euler with transport velocity: drop-in for ``jax_sph.integrator.si_euler``.

``advance(dt, state, neighbors) -> (state, neighbors)`` performs, in one GPU
pass chain (integrator.py:22-56): ``u += dt*dudt``, ``v = u + tvf*dt/2*dvdt``,
``r = shift(r, dt*v)``, neighbour-list rebuild (fused with the kick-drift into
the cell binning), the WCSPH forward pass and ``bc_fn``.
"""


def si_euler(tvf, model, shift_fn, bc_fn, nw_fn):
    """Return ``advance(dt, state, neighbors)`` for a ``WCSPH`` forward ``model``."""
    solver = getattr(model, "__wcsph__", None)
    if solver is None:
        raise NotImplementedError("model must be WCSPH(...).forward_wrapper() of jaxsph_gb300")
    if nw_fn is not None and getattr(nw_fn, "spec", None) is None:
        raise NotImplementedError(
            "nw_fn must be the GPU descriptor jaxsph_gb300.cases.WallNormals")
    tvf = float(tvf)

    def advance(dt, state, neighbors):
        return solver.advance(float(dt), tvf, state, neighbors, bc_fn, nw_fn)

    advance.__si_euler__ = (solver, tvf, bc_fn)
    return advance
