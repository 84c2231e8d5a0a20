"""Couette flow against the Morris et al. (1997) series solution.

Port of the reference's own physics test (tests/test_cf2d.py:14-123): the
channel of cases/cf.yaml at dx = 0.0333333, dt = 2e-6, its top wall moving at
1.25, run on the GPU; the x-velocity is SPH-interpolated at x = 0.2 across the
channel (walls inverted like utils.sph_interpolator, utils.py:299-399) at
t = 5e-4, 1e-3 and 5e-3 and compared with the series at atol 1e-2.
Variants (tvf, solver): (0, SPH), (1, SPH), (0, RIE); the DELTA solver of the
reference test is outside the GPU path.
"""

import numpy as np
import pytest

from jaxsph_gb300 import cases, simulate
from test_gpu_poiseuille import interpolate_u

pytestmark = pytest.mark.gpu


def u_series_couette(y, t, n_max=10):
    """Morris et al. 1997 start-up Couette series: u = U y / d plus decaying sine modes."""
    nu, u_wall, d = 100.0, 1.25, 1.0
    res = u_wall * y / d
    for n in range(1, n_max):
        res = res + 2 * u_wall / (n * np.pi) * (-1) ** n * np.sin(n * np.pi * y / d) * np.exp(
            -((n * np.pi / d) ** 2) * nu * t)
    return res


@pytest.mark.parametrize("tvf,solver", [(0.0, "SPH"), (1.0, "SPH"), (0.0, "RIE"),
                                        (0.0, "DELTA")])
def test_couette_matches_series(tvf, solver):
    import torch

    dx, dt = 0.0333333, 0.000002
    setup = cases.couette(dx=dx, dt=dt, t_end=0.005, tvf=tvf, solver_name=solver)
    sim = simulate.Simulation(setup)
    y = np.linspace(0, 1, 21)
    targets = torch.tensor(np.stack([np.full_like(y, 0.2), y + 3 * dx], 1))
    done = 0
    for t in (0.0005, 0.001, 0.005):
        # the reference writes the state after step k as file k - 1
        steps = int(round(t / dt)) + 1
        sim.run(steps - done)
        done = steps
        got = interpolate_u(sim.state()[0], dx, setup.box, targets)
        ref = u_series_couette(y, t)
        assert np.allclose(got, ref, atol=1e-2), (t, np.abs(got - ref).max())
