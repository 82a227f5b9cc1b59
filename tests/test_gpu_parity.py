"""Parity of the CUDA path (through the C ABI) with the reference's outputs
(tests/golden/) and with the C oracle, in FP64 and mixed precision."""
import numpy as np
import pytest

import oracle as O
from helpers import (GOLDEN_CASES, TOL_FP64, TOL_MIXED, gpu_system, load_golden, oracle_system, random_system,
                     scales, torque, xi_from_ref)

pytestmark = pytest.mark.gpu

PRECS = [(0, TOL_FP64), (1, TOL_MIXED)]
NO_OVERLAP = [c for c in GOLDEN_CASES if c != "n64_overlap"]


def magmom(ini, g):
    d = O.derive(ini)
    return d["satMag"] * 4.0 / 3.0 * d["my_pi"] * g["rMag"] ** 3.0


@pytest.mark.parametrize("prec,tol", PRECS)
@pytest.mark.parametrize("name", NO_OVERLAP)
def test_interactions_vs_reference(name, prec, tol):
    """CompInteractions: B, F, torque and pressure at the first step."""
    ini, g = load_golden(name)
    fAl, bAl, tAl = scales(ini, g)
    sim = gpu_system(ini, g, prec)
    assert sim.lBox == pytest.approx(g["lBox"], rel=1e-14)
    B, F, P3 = sim.CompInteractions()
    Fref = g["ref_F1"][0] - g["ref_thermForce"][0]
    assert O.rms_rel(B, g["ref_B1"][0], bAl) < tol
    assert O.rms_rel(F, Fref, fAl) < tol
    mu = magmom(ini, g)
    assert O.rms_rel(torque(g["mm"], B, mu), torque(g["mm"], g["ref_B1"][0], mu), tAl) < tol
    vol = g["lBox"] ** 3
    pref = g["ref_obs"][0][5:8]
    np.testing.assert_allclose(P3 / vol, pref, rtol=1e-8 if prec == 0 else 1e-4,
                               atol=(1e-8 if prec == 0 else 1e-4) * np.abs(pref).max())


@pytest.mark.parametrize("prec,tol", PRECS)
@pytest.mark.parametrize("name", ["n64_refnoise", "n512_cfg1_refnoise", "n64_lognormal", "n512_cfg1_noiseoff"])
def test_steps_vs_reference_uploaded_noise(name, prec, tol):
    """Full Heun steps with the reference's own noise stream uploaded."""
    ini, g = load_golden(name)
    sim = gpu_system(ini, g, prec, noise=1)
    for s in range(g["nsteps"]):
        sim.step(1, g["dt"], xi=xi_from_ref(ini, g, s))
        pos, mm, ea = sim.get_state()
        ptol = 1e-13 * g["lBox"] if prec == 0 else 1e-9 * g["lBox"]
        assert np.abs(pos - g["ref_pos"][s]).max() < ptol
        atol = 1e-12 if prec == 0 else 2e-6
        assert np.abs(mm - g["ref_mm"][s]).max() < atol
        assert np.abs(ea - g["ref_ea"][s]).max() < atol
    rec = sim.records()
    assert rec.shape == (g["nsteps"], 8)
    np.testing.assert_allclose(rec[:, 0], g["ref_obs"][:, 0], rtol=1e-14, atol=0)
    np.testing.assert_allclose(rec[:, 1], g["ref_obs"][:, 1], atol=1e-12 if prec == 0 else 2e-6)
    np.testing.assert_allclose(rec[:, 2:5], g["ref_obs"][:, 2:5], rtol=1e-6 if prec == 0 else 1e-2)


@pytest.mark.parametrize("prec,tol", PRECS)
def test_overlap_push_matches_oracle_jacobi(prec, tol):
    """Overlapping cores: all overlaps resolved from the same positions; the
    oracle's Jacobi mode is the bit-for-bit restatement of that choice."""
    ini, g = load_golden("n64_overlap")
    fAl, bAl, _ = scales(ini, g)
    sim = gpu_system(ini, g, prec)
    orc = oracle_system(ini, g, overlap_mode=1)
    B, F, _ = sim.CompInteractions()
    Bo, Fo, _ = orc.compute_interactions()
    assert O.rms_rel(B, Bo, bAl) < tol
    assert O.rms_rel(F, Fo, fAl) < tol
    p, _, _ = sim.get_state()
    po, _, _, _ = orc.get_state()
    push = np.abs(po - g["pos"]).max()
    assert push > 0
    # FP64: rounding of the positions; mixed: the push itself is FP32
    assert np.abs(p - po).max() < (1e-12 if prec == 0 else 1e-6) * push


@pytest.mark.parametrize("prec,tol", PRECS)
def test_demag_field_for_arbitrary_moments(prec, tol):
    """CompDemagField with non-unit predictor-like moments."""
    ini, g = load_golden("n512_cfg1_noiseoff")
    fAl, bAl, _ = scales(ini, g)
    sim = gpu_system(ini, g, prec)
    orc = oracle_system(ini, g)
    sim.CompInteractions()
    orc.compute_interactions()
    rng = np.random.default_rng(5)
    mm2 = g["mm"] + 0.01 * rng.standard_normal(g["mm"].shape)
    assert O.rms_rel(sim.CompDemagField(mm2), orc.compute_field(mm2), bAl) < tol


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("n,rc_frac", [(512, 0.3), (4096, 0.25), (3000, 0.2)])
def test_cell_list_is_a_stable_counting_sort(n, rc_frac, prec):
    ini, g = random_system(n, seed=n, rc_frac=rc_frac)
    sim = gpu_system(ini, g, prec)
    sim.CompInteractions()
    ncx, cs, perm = sim.debug_cells()
    assert ncx >= 5, "stencil mode expected"
    xb = g["pos"] / g["lBox"]
    xb = xb - np.floor(xb + 0.5)
    c = np.clip(((xb + 0.5) * ncx).astype(np.int64), 0, ncx - 1)
    cell = (c[2] * ncx + c[1]) * ncx + c[0]
    order = np.argsort(cell, kind="stable")
    counts = np.bincount(cell, minlength=ncx ** 3)
    np.testing.assert_array_equal(perm, order)
    np.testing.assert_array_equal(cs, np.concatenate([[0], np.cumsum(counts)]))


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-6)])
def test_structure_factor(prec, tol):
    ini, g = random_system(512, seed=9, rc_frac=0.3)
    sim = gpu_system(ini, g, prec)
    sim.CompInteractions()
    S = sim.debug_structure_factor()
    d = O.derive(ini)
    mu = g["mm"] * magmom(ini, g)[None, :]
    nvec = S[:, :3]
    ph = 2 * d["my_pi"] * (nvec @ g["pos"]) / g["lBox"]
    w = nvec @ mu
    Sc = (w * np.cos(ph)).sum(1)
    Ss = (w * np.sin(ph)).sum(1)
    scale = np.abs(mu).max() * np.sqrt(g["n"]) * np.abs(nvec).max()
    assert np.abs(S[:, 3] - Sc).max() < tol * scale
    assert np.abs(S[:, 4] - Ss).max() < tol * scale
    nk = len(S)
    kc = g["kc"]
    full = sum(1 for nz in range(kc + 1) for ny in range(-kc, kc + 1) for nx in range(-kc, kc + 1)
               if 0 < nx * nx + ny * ny + nz * nz <= kc * kc)
    plane = sum(1 for ny in range(-kc, kc + 1) for nx in range(-kc, kc + 1) if 0 < nx * nx + ny * ny <= kc * kc)
    assert nk == full - plane // 2


@pytest.mark.parametrize("prec,tol", PRECS)
@pytest.mark.parametrize("n,rc_frac,lognormal", [(512, 0.3, False), (2000, 0.22, True), (4096, 0.4, False)])
def test_interactions_vs_oracle_random(n, rc_frac, lognormal, prec, tol):
    ini, g = random_system(n, seed=n + 1, rc_frac=rc_frac, lognormal=lognormal)
    fAl, bAl, tAl = scales(ini, g)
    sim = gpu_system(ini, g, prec)
    orc = oracle_system(ini, g)
    B, F, P = sim.CompInteractions()
    Bo, Fo, Po = orc.compute_interactions()
    assert O.rms_rel(B, Bo, bAl) < tol
    assert O.rms_rel(F, Fo, fAl) < tol
    mu = magmom(ini, g)
    assert O.rms_rel(torque(g["mm"], B, mu), torque(g["mm"], Bo, mu), tAl) < tol


@pytest.mark.parametrize("prec", [0, 1])
def test_philox_noise_trajectory_vs_oracle(prec):
    """Device Philox noise equals the oracle's Philox restatement."""
    ini, g = random_system(256, seed=21, rc_frac=0.45, noise=True)
    sim = gpu_system(ini, g, prec, noise=2, seed=77)
    orc = oracle_system(ini, g)
    for _ in range(5):
        orc.step(g["dt"], 2, None, 77)
    sim.step(5, g["dt"])
    p, m, e = sim.get_state()
    po, mo, eo, _ = orc.get_state()
    d = np.abs(p - po)
    d = np.minimum(d, g["lBox"] - d)
    assert d.max() < (1e-13 if prec == 0 else 1e-10) * g["lBox"]
    assert np.abs(m - mo).max() < (1e-11 if prec == 0 else 1e-5)
    assert np.abs(e - eo).max() < (1e-11 if prec == 0 else 1e-5)


@pytest.mark.parametrize("prec", [0, 1])
def test_noise_off_trajectory_vs_oracle(prec):
    ini, g = random_system(512, seed=31, rc_frac=0.3, noise=False, B0=0.02)
    sim = gpu_system(ini, g, prec, noise=0)
    orc = oracle_system(ini, g)
    for _ in range(20):
        orc.step(g["dt"], 0)
    sim.step(20, g["dt"])
    p, m, e = sim.get_state()
    po, mo, eo, _ = orc.get_state()
    assert np.abs(p - po).max() < (1e-14 if prec == 0 else 1e-12) * g["lBox"]
    assert np.abs(m - mo).max() < (1e-11 if prec == 0 else 1e-5)
    assert np.abs(e - eo).max() < (1e-11 if prec == 0 else 1e-5)
    rec = sim.records()
    assert rec.shape[0] == 20 and np.all(np.diff(rec[:, 0]) > 0)


def test_momentum_and_translation_invariance_full_size():
    """Size-independent properties at the largest single-system size
    (N = 32768, phi = 0.10): the interaction forces sum to zero, a rigid
    shift of all particles leaves B and F unchanged, and the mixed path
    agrees with the FP64 path within the 1e-5 contact-normalised budget."""
    n = 32768
    ini, g = random_system_fast(n, seed=2, phi=0.10, B0=0.02)
    fAl, bAl, _ = scales(ini, g)
    mix = gpu_system(ini, g, 1)
    B1, F1, _ = mix.CompInteractions()
    ref = gpu_system(ini, g, 0)
    B0, F0, _ = ref.CompInteractions()
    assert O.rms_rel(B1, B0, bAl) < TOL_MIXED
    assert O.rms_rel(F1, F0, fAl) < TOL_MIXED
    assert np.abs(F0.sum(axis=1)).max() < 1e-9 * fAl * np.sqrt(n)
    g2 = dict(g)
    g2["pos"] = g["pos"] + np.array([0.123, -0.077, 0.31])[:, None] * g["lBox"]
    g2["pos"] = g2["pos"] - g["lBox"] * np.round(g2["pos"] / g["lBox"])
    sh = gpu_system(ini, g2, 0)
    B2, F2, _ = sh.CompInteractions()
    assert O.rms_rel(B2, B0, bAl) < 1e-9
    assert O.rms_rel(F2, F0, fAl) < 1e-9


def random_system_fast(n, seed, phi, B0):
    """Jittered lattice (no overlaps) for large N; polydisperse physics
    (log-normal cores, median 20 nm diameter, sigma 0.2, 5 nm shell)."""
    import ref_io
    ini = ref_io.ini_dict(volFrac=phi, magFluxDens=B0, ENABLE_THERM_FIELD="false", ENABLE_THERM_TORQUE="false",
                          ENABLE_THERM_FORCE="false")
    d = O.derive(ini)
    rng = np.random.default_rng(seed)
    rMag = 1e-8 * np.exp(0.2 * rng.standard_normal(n))
    rHydr = rMag + 5e-9
    L = O.box_length(rHydr, phi, d["my_pi"])
    m = int(np.ceil(n ** (1 / 3)))
    a = L / m
    idx = rng.permutation(m ** 3)[:n]
    grid = np.stack([idx % m, (idx // m) % m, idx // (m * m)]).astype(float)
    jit = max(0.0, (a - 2 * rMag.max() - 2e-10) / 2) * 0.95  # cores never overlap
    pos = (grid + 0.5) * a - L / 2 + rng.uniform(-jit, jit, (3, n))
    v = rng.standard_normal((3, n))
    mm = v / np.linalg.norm(v, axis=0)
    v = rng.standard_normal((3, n))
    ea = v / np.linalg.norm(v, axis=0)
    alpha, kc, _ = O.ewald_for_rc(d, rMag, rHydr, L, 0.22 * L)
    g = dict(n=n, dt=1e-12, alpha=alpha, rc=0.22 * L, kc=kc, vis=1e-3, lBox=L, rMag=rMag, rHydr=rHydr, pos=pos,
             mm=mm, ea=ea, rCutSR=2 * rMag.max())
    return ini, g


def test_invalid_calls_return_errors():
    from md_sim_wolfschwenger_gb300 import MdError
    ini, g = load_golden("n64_noiseoff")
    sim = gpu_system(ini, g, 1)
    with pytest.raises(MdError) as e:
        sim.set_ewald(g["alpha"], 0.6 * g["lBox"], g["kc"])
    assert e.value.status == 1
    sim.set_ewald(g["alpha"], g["rc"], g["kc"])
    with pytest.raises(MdError):
        sim.step(1, -1.0)
    bad = g["pos"].copy()
    bad[0, 3] = np.nan
    sim.set_state(bad, g["mm"], g["ea"])
    with pytest.raises(MdError) as e:
        sim.step(1, g["dt"])
    assert e.value.status == 4
