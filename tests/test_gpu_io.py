"""Trajectory files of a GPU rollout and a restart from one of them
(simulate.py:110-134 and case_setup.py:184-194 of the reference)."""

import os

import pytest
import torch

from jaxsph_gb300 import cases, io_state, simulate

pytestmark = pytest.mark.gpu

KEYS = ("r", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p")


def test_simulate_writes_the_reference_trajectory_files(tmp_path):
    setup = cases.tgv(dim=2, dx=0.05)
    setup.sequence_length = 10
    final = simulate.simulate(setup, data_path=str(tmp_path), write_every=4)
    # sequence_length + 2 steps; file k holds the state after k + 1 of them
    assert sorted(os.listdir(tmp_path)) == ["traj_00.h5", "traj_04.h5", "traj_08.h5"]
    sim = simulate.Simulation(setup)
    sim.run(5)
    want = sim.state()[0]
    got = io_state.read_h5(str(tmp_path / "traj_04.h5"))
    for k in KEYS + ("tag", "mass"):
        assert torch.equal(got[k], want[k].cpu()), k

    # restart from the state after 9 steps with every key: 3 more steps give
    # the 12-step state (pair sums may run in another order after the rebinning)
    again = cases.tgv(dim=2, dx=0.05).load_state0(str(tmp_path / "traj_08.h5"), keys=KEYS)
    sim2 = simulate.Simulation(again)
    sim2.run(3)
    res = sim2.state()[0]
    # float32 rounding scales: accelerations and pressures carry p_ref
    F = setup.p_ref / setup.dx
    tol = {"r": 1e-6, "u": 1e-5, "v": 1e-5, "rho": 2e-6, "p": 2e-6 * setup.c_ref ** 2,
           "dudt": 1e-5 * F, "dvdt": 1e-5 * F, "drhodt": 1e-5 * F}
    for k in KEYS:
        err = float((res[k].double() - final[k].double()).abs().max())
        assert err <= tol[k], (k, err)
