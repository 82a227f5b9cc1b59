"""The real-space Verlet list: rebuilt on the device when a particle has moved
more than half the skin; a list that does not fit falls back to the direct
cell scan.  Results must equal the oracle's all-pairs evaluation either way."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_FP64, TOL_MIXED, gpu_system, oracle_system, random_system, scales

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("skin", [1e-9, 0.02, 0.3])
def test_trajectory_with_frequent_or_rare_rebuilds(prec, skin):
    """skin 1e-9: a rebuild almost every step; 0.02: none in 30 steps; 0.3:
    many extra list entries, all filtered by the exact rc test."""
    ini, g = random_system(512, seed=51, rc_frac=0.3, noise=True, B0=0.02)
    sim = gpu_system(ini, g, prec, noise=2, seed=9)
    sim.set_neighbor_skin(skin)
    orc = oracle_system(ini, g)
    for _ in range(30):
        orc.step(g["dt"], 2, None, 9)
    sim.step(30, g["dt"])
    p, m, e = sim.get_state()
    po, mo, eo, _ = orc.get_state()
    d = np.abs(p - po)
    d = np.minimum(d, g["lBox"] - d)
    assert d.max() < (1e-13 if prec == 0 else 1e-10) * g["lBox"]
    assert np.abs(m - mo).max() < (1e-11 if prec == 0 else 1e-5)
    assert np.abs(e - eo).max() < (1e-11 if prec == 0 else 1e-5)


@pytest.mark.parametrize("prec,tol", [(0, TOL_FP64), (1, TOL_MIXED)])
def test_list_overflow_falls_back_to_cell_scan(prec, tol):
    ini, g = random_system(2000, seed=52, rc_frac=0.22)
    fAl, bAl, _ = scales(ini, g)
    sim = gpu_system(ini, g, prec)
    orc = oracle_system(ini, g)
    Bo, Fo, _ = orc.compute_interactions()
    B0, F0, _ = sim.CompInteractions()
    used = sim.neighbor_capacity()
    assert used > 0
    sim.neighbor_capacity(cap=used // 10)       # the next build cannot fit
    sim.set_state(g["pos"], g["mm"], g["ea"])
    B1, F1, _ = sim.CompInteractions()            # direct scan this time
    assert O.rms_rel(B1, Bo, bAl) < tol and O.rms_rel(F1, Fo, fAl) < tol
    sim.set_state(g["pos"], g["mm"], g["ea"])
    B2, F2, _ = sim.CompInteractions()            # grown list again
    assert sim.neighbor_capacity() == used
    assert O.rms_rel(B2, Bo, bAl) < tol and O.rms_rel(F2, Fo, fAl) < tol
    assert O.rms_rel(B0, Bo, bAl) < tol
