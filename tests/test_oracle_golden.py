"""The C oracle against the reference's own outputs (tests/golden/, made by
oracle/_ref/ref_harness from the reference sources).  CPU only."""
import numpy as np
import pytest

import oracle as O
from helpers import GOLDEN_CASES, load_golden, oracle_system, scales, xi_from_ref

TOL = 1e-12  # FP64 vs FP64, same loop order


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_reference_steps(name):
    ini, g = load_golden(name)
    fAl, bAl, _ = scales(ini, g)
    # the reference's own semantics: sequential in-place overlap push
    orc = oracle_system(ini, g, overlap_mode=0)
    for s in range(g["nsteps"]):
        xi = xi_from_ref(ini, g, s)
        o = orc.step(g["dt"], 1, xi, dump=True)
        assert O.rms_rel(o["B1"], g["ref_B1"][s], bAl) < TOL
        assert O.rms_rel(o["F1"], g["ref_F1"][s], fAl) < TOL
        assert O.rms_rel(o["B2"], g["ref_B2"][s], bAl) < TOL
        pos, mm, ea, t = orc.get_state()
        assert np.max(np.abs(pos - g["ref_pos"][s])) <= 1e-12 * g["lBox"]
        assert np.max(np.abs(mm - g["ref_mm"][s])) < 1e-12
        assert np.max(np.abs(ea - g["ref_ea"][s])) < 1e-12
        ref_obs = g["ref_obs"][s]
        np.testing.assert_allclose(o["obs"][:2], ref_obs[:2], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(o["obs"][2:5], ref_obs[2:5], rtol=1e-9, atol=1e-30)
        np.testing.assert_allclose(o["obs"][5:], ref_obs[5:], rtol=1e-9, atol=1e-9 * np.max(np.abs(ref_obs[5:])))


def test_overlap_case_really_overlaps():
    ini, g = load_golden("n64_overlap")
    moved = np.abs(g["ref_posCorr"][0] - g["pos"]).max()
    assert moved > 1e-10, "fixture must exercise the overlap push"


def test_jacobi_overlap_differs_only_on_overlapping_particles():
    """The GPU resolves all overlaps from the starting positions (Jacobi).
    Where no particle takes part in two overlaps it equals the reference's
    sequential push; the bracketed difference is bounded by the push size."""
    ini, g = load_golden("n64_overlap")
    fAl, bAl, _ = scales(ini, g)
    seq = oracle_system(ini, g, overlap_mode=0)
    jac = oracle_system(ini, g, overlap_mode=1)
    Bs, Fs, _ = seq.compute_interactions()
    Bj, Fj, _ = jac.compute_interactions()
    ps, _, _, _ = seq.get_state()
    pj, _, _, _ = jac.get_state()
    push = np.abs(ps - g["pos"]).max()
    assert np.abs(pj - ps).max() <= push
    # fixture overlaps are deep (cores 28-40 % inside each other); the
    # field difference stays a few per cent of the contact field
    assert O.rms_rel(Bj, g["ref_B1"][0], bAl) < 5e-2
    assert O.rms_rel(Bs, g["ref_B1"][0], bAl) < 1e-12


def test_philox_known_answer():
    """Philox4x32-10 against the known-answer vectors published with the
    Random123 library (Salmon et al., SC'11): counter 0 / key 0, all ones,
    and the digits of pi as counter and key.  The GPU's noise is checked
    bit for bit against this generator elsewhere, so these pin both."""
    kat = [([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
           ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
           ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
            [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])]
    for ctr, key, want in kat:
        assert O.philox_block(ctr, key) == want, (ctr, key)
    # the uniform-to-normal map (Box-Muller) through its first two moments
    xs = O.philox_normals(1234, 7, 20000).reshape(9, -1)
    assert np.all(np.isfinite(xs))
    assert abs(xs.mean()) < 0.01
    assert abs(xs.std() - 1) < 0.01


ADAPTIVE_CASES = ["n64_adapt_he", "n64_adapt_bs", "n64_adapt_dp"]


def xi_adaptive(ini, g, step):
    """Unit normals of step `step` from the reference's thermal arrays, which
    DefThermFluct scaled with that step's trial dt (simulation.cpp:563-603)."""
    d = O.derive(ini)
    sT, sB, sF = O.noise_scales(d, g["rMag"], g["rHydr"], float(g["ref_dt0"][step]), g["vis"])
    return np.stack([g["ref_thermTorque"][step] / sT, g["ref_thermField"][step] / sB,
                     g["ref_thermForce"][step] / sF])


@pytest.mark.parametrize("name", ADAPTIVE_CASES)
def test_oracle_matches_reference_adaptive(name):
    """Heun-Euler, Bogacki-Shampine and Dormand-Prince with the reference's
    step control (rejections included): the same trial and used steps, the
    same states."""
    ini, g = load_golden(name)
    d = O.derive(ini)
    orc = oracle_system(ini, g, overlap_mode=0)
    dt = float(g["ref_dt0"][0])
    for s in range(g["nsteps"]):
        assert abs(dt - g["ref_dt0"][s]) <= 1e-9 * dt  # error estimates are differences of slopes
        dt, used, att, obs = orc.step_adaptive(int(g["solver"]), dt, d["absTol"], d["deltaTmin"], d["deltaTmax"], 1,
                                               xi_adaptive(ini, g, s))
        assert abs(used - g["ref_dtUsed"][s]) <= 1e-9 * used
        pos, mm, ea, t = orc.get_state()
        assert np.max(np.abs(pos - g["ref_pos"][s])) <= 1e-12 * g["lBox"]
        assert np.max(np.abs(mm - g["ref_mm"][s])) < 1e-11
        assert np.max(np.abs(ea - g["ref_ea"][s])) < 1e-11
        np.testing.assert_allclose(obs[:2], g["ref_obs"][s][:2], rtol=1e-11, atol=1e-15)
    # the cases exercise rejections
    assert np.any(g["ref_dtUsed"] != g["ref_dt0"])


def test_rsa_philox_restatement_properties():
    """The placement restatement (orc_rsa_philox): inside the box, no
    overlaps, deterministic, and the largest-first order places the same
    particles differently but validly."""
    rng = np.random.default_rng(3)
    n = 400
    rH = 15e-9 * np.exp(0.25 * rng.standard_normal(n))
    L = float((np.sum(4.0 / 3.0 * np.pi * rH ** 3) / 0.2) ** (1.0 / 3.0))
    for order in (None, np.argsort(-rH, kind="stable")):
        pos, tries = O.rsa_philox(n, L, rH, 9, order=order)
        pos2, _ = O.rsa_philox(n, L, rH, 9, order=order)
        assert np.array_equal(pos, pos2)
        assert np.all(np.abs(pos) <= L / 2 - rH[None, :])
        d = np.linalg.norm(pos[:, :, None] - pos[:, None, :], axis=0)
        s = rH[:, None] + rH[None, :]
        np.fill_diagonal(d, np.inf)
        assert np.all(d >= s)
        assert tries.min() >= 0
