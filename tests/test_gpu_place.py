"""GPU initial placement (md_place_rsa, random sequential addition with a
Philox stream per particle) against its sequential restatement in the C
oracle (orc_rsa_philox): the same positions bit for bit, in the reference's
index order (InitCoordsFromSketch, src/simulation.cpp:241-264) and largest
first; dense systems where candidates of one batch overlap each other; a
large system checked for overlaps and box bounds."""
import os
import sys
import time

import numpy as np
import pytest

import md_sim_wolfschwenger_gb300 as m

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _radii(n, seed, sigma=0.0, r0=15e-9):
    rng = np.random.default_rng(seed)
    r = r0 * np.exp(sigma * rng.standard_normal(n)) if sigma > 0 else np.full(n, r0)
    return r


def _box(rH, phi):
    return float((np.sum(4.0 / 3.0 * np.pi * rH ** 3) / phi) ** (1.0 / 3.0))


@pytest.mark.parametrize("n,sigma,phi,largest,seed", [
    (2000, 0.25, 0.15, False, 11),   # log-normal, index order (the reference's)
    (700, 0.0, 0.30, False, 12),     # dense monodisperse: batch-mates overlap each other
    (3000, 0.25, 0.20, True, 13),    # largest first, several batches
    (1, 0.0, 0.01, False, 14),       # a single particle
])
def test_place_matches_sequential_restatement(n, sigma, phi, largest, seed):
    rH = _radii(n, seed, sigma)
    L = _box(rH, phi)
    got = m.place_rsa(rH, L, 1000 + seed, largest_first=largest)
    order = np.argsort(-rH, kind="stable") if largest else None
    want, tries = O.rsa_philox(n, L, rH, 1000 + seed, order=order)
    assert np.array_equal(got, want)
    if n > 1:
        assert tries.max() >= 1  # some candidates were rejected, so the rule was exercised


def test_place_large_system_no_overlaps():
    n = 131072
    rH = _radii(n, 5, 0.25, 17.5e-9)
    L = _box(rH, 0.20)
    m.place_rsa(rH[:1000], _box(rH[:1000], 0.2), 1)  # module load and first launch
    t0 = time.perf_counter()
    pos = m.place_rsa(rH, L, 7, largest_first=True)
    dt = time.perf_counter() - t0
    assert np.all(np.abs(pos) <= L / 2 - rH[None, :] + 1e-12 * L)
    from scipy.spatial import cKDTree
    tree = cKDTree(pos.T)
    pairs = tree.query_pairs(2.0 * rH.max(), output_type="ndarray")
    d = np.linalg.norm(pos[:, pairs[:, 0]] - pos[:, pairs[:, 1]], axis=0)
    assert np.all(d >= rH[pairs[:, 0]] + rH[pairs[:, 1]])
    print(f"md_place_rsa N={n}: {dt * 1e3:.1f} ms")
    assert dt < 10.0


def test_place_rejects_impossible_density():
    rH = _radii(400, 3)
    L = _box(rH, 0.9)  # beyond random close packing
    with pytest.raises(m.MdError):
        m.place_rsa(rH, L, 1)
