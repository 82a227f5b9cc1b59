"""Edge cases of the interaction kernels against the oracle: the smallest
systems (2, 3 and 8 particles: one cell holds everything, every pair is a
minimum-image pair), the largest cutoff rc = L/2, the smallest k-space cutoff
kc = 1, a large kc, and particle counts that fill no block evenly."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_FP64, TOL_MIXED, gpu_system, oracle_system, random_system, scales

pytestmark = pytest.mark.gpu
PRECS = [(0, TOL_FP64), (1, TOL_MIXED)]


def _compare(ini, g, prec, tol):
    fAl, bAl, _ = scales(ini, g)
    sim = gpu_system(ini, g, prec)
    orc = oracle_system(ini, g)
    B, F, _ = sim.CompInteractions()
    Bo, Fo, _ = orc.compute_interactions()
    assert O.rms_rel(B, Bo, bAl) < tol
    assert O.rms_rel(F, Fo, fAl) < tol
    sim.close()


@pytest.mark.parametrize("prec,tol", PRECS)
@pytest.mark.parametrize("n", [2, 3, 8, 33, 1001])
def test_small_and_ragged_systems(n, prec, tol):
    ini, g = random_system(n, seed=300 + n, rc_frac=0.45 if n < 100 else 0.3, phi=0.02 if n < 10 else 0.05)
    _compare(ini, g, prec, tol)


@pytest.mark.parametrize("prec,tol", PRECS)
def test_cutoff_at_half_box(prec, tol):
    ini, g = random_system(300, seed=41, rc_frac=0.5)
    _compare(ini, g, prec, tol)


@pytest.mark.parametrize("prec,tol", PRECS)
@pytest.mark.parametrize("kc", [1, 40])
def test_extreme_k_cutoffs(kc, prec, tol):
    ini, g = random_system(256, seed=42 + kc, rc_frac=0.3)
    g = dict(g)
    g["kc"] = kc
    _compare(ini, g, prec, tol)


def test_one_particle_is_rejected():
    import md_sim_wolfschwenger_gb300 as m
    cfg = m.Configuration.default()
    with pytest.raises(m.MdError) as e:
        m.Simulation(cfg, 1)
    assert e.value.status == 1
