"""Device post-processing: g(r) of a frame (md_rdf) against the numpy
restatement of the reference's script (mFiles/radial_dist_fun.m) on the
same positions, with and without the script's last-particle loop bound."""
import numpy as np
import pytest

from helpers import gpu_system, random_system
from md_sim_wolfschwenger_gb300 import analysis

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("include_last", [False, True])
@pytest.mark.parametrize("n,lognormal", [(1500, False), (700, True)])
def test_rdf_matches_script(n, lognormal, include_last):
    ini, g = random_system(n, seed=n + 7, rc_frac=0.3, phi=0.1, lognormal=lognormal)
    sim = gpu_system(ini, g, 1)
    sim.CompInteractions()  # moves nothing without overlaps; positions as uploaded
    pos, _, _ = sim.get_state()
    r0 = float(g["rMag"][0])
    x, gd, cnt = sim.rdf(bins=500, range_mag=8.0, r_mag0=r0, include_last=include_last)
    xr, gr = analysis.radial_distribution(pos, g["lBox"], r0, include_last=include_last)
    np.testing.assert_allclose(x, xr, rtol=1e-14)
    # integer pair counts: identical except where a pair sits within rounding
    # of a bin edge (then it moves to the neighbouring bin)
    mismatch = np.abs(gd - gr) > 1e-12 * gr.max()
    assert mismatch.sum() <= 2
    assert cnt.sum() > 0
