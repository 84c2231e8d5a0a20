"""Poiseuille flow against the Morris et al. (1997) series solution.

Port of the reference's own physics test (tests/test_pf2d.py:14-115): the
channel of cases/pf.yaml at dx = 0.0333333, dt = 2e-6, run on the GPU; the
x-velocity is SPH-interpolated at x = 0.2 across the channel (with the wall
velocities inverted like utils.sph_interpolator, utils.py:299-399) at
t = 5e-4, 1e-3 and 5e-3 and compared with the series at atol 1e-2.
Variants (tvf, solver): (0, SPH), (1, SPH), (0, RIE); the DELTA solver of the
reference test is outside the GPU path.
"""

import numpy as np
import pytest
import torch

from jaxsph_gb300 import cases, simulate
from jaxsph_gb300.kernel import QuinticKernel

pytestmark = pytest.mark.gpu


def u_series_exp(y, t, n_max=10):
    """Morris et al. 1997 unsteady Poiseuille series (as in tests/test_pf2d.py:14-41)."""
    eta, rho, u_max, d = 100.0, 1.0, 1.25, 1.0
    nu = eta / rho
    fx = -8 * nu * u_max / d ** 2
    res = fx / (2 * nu) * y * (y - d)
    for n in range(n_max):
        base = np.pi * (2 * n + 1) / d
        res = res + 4 * fx / (nu * base ** 3 * d) * np.sin(base * y) * np.exp(-(base ** 2) * nu * t)
    return res


def interpolate_u(st, dx, box, targets):
    """SPH interpolation of u_x at target points (utils.sph_interpolator)."""
    r = st["r"].double().cpu()
    u = st["u"].double().cpu()
    tag = st["tag"].cpu()
    k = QuinticKernel(h=dx, dim=2)
    side = torch.as_tensor(box, dtype=torch.float64)
    # invert wall velocities: 2 u_wall - Shepard average of fluid velocities
    d = r[:, None, :] - r[None, :, :]
    d = d - side * torch.round(d / side)
    w = k.w(d.norm(dim=-1)) * (tag == 0).double()[None, :]
    w = torch.where(d.norm(dim=-1) < 3 * dx, w, torch.zeros_like(w))
    u_wall = (w @ u) / (w.sum(1, keepdim=True) + 2.220446049250313e-16)
    u = torch.where((tag != 0)[:, None], 2 * u - u_wall, u)
    dist = (targets[:, None, :] - r[None, :, :]).norm(dim=-1)
    wt = k.w(dist)
    return ((wt * u[:, 0][None, :]).sum(1) / wt.sum(1)).numpy()


@pytest.mark.parametrize("tvf,solver", [(0.0, "SPH"), (1.0, "SPH"), (0.0, "RIE"),
                                        (0.0, "DELTA")])
def test_poiseuille_matches_series(tvf, solver):
    dx, dt = 0.0333333, 0.000002
    setup = cases.poiseuille(dx=dx, dt=dt, t_end=0.005, tvf=tvf, solver_name=solver)
    sim = simulate.Simulation(setup)
    y = np.linspace(0, 1, 21)
    targets = torch.tensor(np.stack([np.full_like(y, 0.2), y + 3 * dx], 1))
    done = 0
    for t in (0.0005, 0.001, 0.005):
        # the reference writes the state after step k as file k - 1
        # (simulate.py:112-113), so file t/dt holds t/dt + 1 steps
        steps = int(round(t / dt)) + 1
        sim.run(steps - done)
        done = steps
        got = interpolate_u(sim.state()[0], dx, setup.box, targets)
        ref = u_series_exp(y, t)
        assert np.allclose(got, ref, atol=1e-2), (t, np.abs(got - ref).max())
