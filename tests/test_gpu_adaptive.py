"""Adaptive solvers on the GPU (md_step_adaptive): Heun-Euler 1(2),
Bogacki-Shampine 2(3) and Dormand-Prince 4(5) with the reference's step
control (src/simulation.cpp:707-951), against the reference's own adaptive
runs (fixtures made by tests/golden/make_golden.py with the reference's
noise, rejections included) and against the oracle with Philox noise."""
import numpy as np
import pytest

import oracle as O
from helpers import gpu_system, load_golden, oracle_system, random_system
from test_oracle_golden import ADAPTIVE_CASES, xi_adaptive

pytestmark = pytest.mark.gpu


def _ref_noise(ini, g):
    return np.stack([xi_adaptive(ini, g, s) for s in range(g["nsteps"])])


# FP64: the reference's trajectory.  Mixed: the embedded error estimates are
# small differences of the stage slopes, and the FP32 stage fields carry
# ~1e-6 relative noise from stage to stage, so the estimates (and with them
# the chosen steps) differ at the 1e-3 level; the states then differ by the
# slope times that step difference.
@pytest.mark.parametrize("prec,tol_dt,tol_m,tol_pos", [(0, 1e-9, 1e-10, 1e-12), (1, 2e-2, 5e-3, 2e-6)])
@pytest.mark.parametrize("name", ADAPTIVE_CASES)
def test_adaptive_vs_reference(name, prec, tol_dt, tol_m, tol_pos):
    ini, g = load_golden(name)
    sim = gpu_system(ini, g, prec, noise=1)
    dt_next, done = sim.step_adaptive(g["nsteps"], float(g["ref_dt0"][0]), xi=_ref_noise(ini, g))
    assert done == g["nsteps"]
    rec = sim.records()
    t_ref = np.concatenate([[0.0], np.cumsum(g["ref_dtUsed"])])
    np.testing.assert_allclose(rec[:, 0], t_ref[:-1], rtol=tol_dt, atol=0)
    np.testing.assert_allclose(np.diff(np.append(rec[:, 0], t_ref[-1])), g["ref_dtUsed"], rtol=tol_dt)
    p, m, e = sim.get_state()
    assert np.abs(m - g["ref_mmF"]).max() < tol_m
    assert np.abs(e - g["ref_eaF"]).max() < tol_m
    d = np.abs(p - g["ref_posF"])
    d = np.minimum(d, g["lBox"] - d)
    assert d.max() < tol_pos * g["lBox"]
    np.testing.assert_allclose(rec[:, 1], g["ref_obs"][:, 1], rtol=0, atol=tol_m)


@pytest.mark.parametrize("solver", [0, 1, 2])
def test_adaptive_philox_vs_oracle_and_stop_time(solver):
    ini, g = random_system(125, seed=60 + solver, rc_frac=0.4, noise=True, B0=0.02)
    ini["adaptive_timestepping_solver"]["SOLVER"] = solver
    ini["solver_settings"]["absTol"] = 1e-4
    d = O.derive(ini)
    sim = gpu_system(ini, g, 0, noise=2, seed=33)
    orc = oracle_system(ini, g)
    dt, t = 1e-12, 0.0
    for _ in range(8):
        dt, used, att, obs = orc.step_adaptive(solver, dt, d["absTol"], d["deltaTmin"], d["deltaTmax"], 2, None, 33)
        t += used
    dt_gpu, done = sim.step_adaptive(8, 1e-12)
    assert done == 8
    assert abs(dt_gpu - dt) <= 1e-9 * dt
    p, m, e = sim.get_state()
    po, mo, eo, to = orc.get_state()
    assert abs(sim.get_time()[0] - to) <= 1e-9 * to
    assert np.abs(m - mo).max() < 1e-10 and np.abs(e - eo).max() < 1e-10
    # the loop runs while t <= t_end: one more step, then it stops
    dt2, done2 = sim.step_adaptive(100, dt_gpu, t_end=sim.get_time()[0])
    assert done2 == 1
