"""Tensor-core reciprocal space (md_ktc.cu: 3-pass TF32 matrix products over k
rows) against the FP32 CUDA-core kernels and the FP64 path: the same
CompDipInteractEwaldF / CompDipFieldEwaldF sums (src/interaction.cpp:429-514,
588-672)."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_MIXED, gpu_system, random_system, scales

pytestmark = pytest.mark.gpu

CASES = [(77, 4, False), (1000, 9, True), (1500, 15, False), (700, 20, True), (300, 25, False)]


def engines(ini, g):
    ref = gpu_system(ini, g, 0)
    out = {}
    for e in ("tc", "simt"):
        s = gpu_system(ini, g, 1)
        s.set_kspace_engine(e)
        out[e] = s
    return ref, out


def sf(sim):
    k = sim.debug_structure_factor()
    return k[:, 3] + 1j * k[:, 4]


@pytest.mark.parametrize("n,kc,lognormal", CASES)
def test_interactions_tc_vs_fp64_and_simt(n, kc, lognormal):
    ini, g = random_system(n, seed=n + kc, rc_frac=0.3, lognormal=lognormal)
    g["kc"] = kc
    fAl, bAl, _ = scales(ini, g)
    ref, s = engines(ini, g)
    assert s["tc"].kspace_tensor_cores() and not s["simt"].kspace_tensor_cores()
    B0, F0, P0 = ref.CompInteractions()
    Bt, Ft, Pt = s["tc"].CompInteractions()
    Bs, Fs, Ps = s["simt"].CompInteractions()
    assert O.rms_rel(Bt, B0, bAl) < TOL_MIXED
    assert O.rms_rel(Ft, F0, fAl) < TOL_MIXED
    # the two mixed engines differ only in the FP32 rounding of the k-space sums
    assert O.rms_rel(Bt, Bs, bAl) < 2e-6
    assert O.rms_rel(Ft, Fs, fAl) < 2e-6
    np.testing.assert_allclose(Pt, Ps, rtol=1e-5, atol=1e-5 * np.abs(Ps).max())
    # structure factor: FP64 sums of 3-pass TF32 chunk products
    S0, St = sf(ref), sf(s["tc"])
    assert len(St) == len(S0) > 0
    assert np.sqrt(np.mean(np.abs(St - S0) ** 2) / np.mean(np.abs(S0) ** 2)) < 1e-6


@pytest.mark.parametrize("n,kc,lognormal", CASES[:3])
def test_field_tc_vs_fp64(n, kc, lognormal):
    """CompDemagField for moments other than the state's (the Heun predictor)."""
    ini, g = random_system(n, seed=3 * n + kc, rc_frac=0.3, lognormal=lognormal)
    g["kc"] = kc
    _, bAl, _ = scales(ini, g)
    ref, s = engines(ini, g)
    rng = np.random.default_rng(n)
    mm = g["mm"] + 0.2 * rng.standard_normal(g["mm"].shape)
    mm /= np.linalg.norm(mm, axis=0)
    for sim in (ref, s["tc"], s["simt"]):
        sim.CompInteractions()  # geometry of the state first, like CompInteractions before CompDemagField
    B0 = ref.CompDemagField(mm)
    Bt = s["tc"].CompDemagField(mm)
    Bs = s["simt"].CompDemagField(mm)
    assert O.rms_rel(Bt, B0, bAl) < TOL_MIXED
    assert O.rms_rel(Bt, Bs, bAl) < 2e-6


def test_tc_deterministic_and_steps():
    """Bit-identical repeats; Heun steps follow the FP64 path."""
    ini, g = random_system(1200, seed=5, rc_frac=0.28)
    ref, s = engines(ini, g)
    tc = s["tc"]
    B1, F1, _ = tc.CompInteractions()
    B2, F2, _ = tc.CompInteractions()
    assert np.array_equal(B1, B2) and np.array_equal(F1, F2)
    for sim in (ref, tc):
        sim.step(5, g["dt"])
    p0, m0, e0 = ref.get_state()
    p1, m1, e1 = tc.get_state()
    assert np.abs(p1 - p0).max() < 1e-9 * g["lBox"]
    assert np.abs(m1 - m0).max() < 2e-6
    assert np.abs(e1 - e0).max() < 2e-6


def test_engine_switch_rules():
    ini, g = random_system(200, seed=9, rc_frac=0.3)
    mixed = gpu_system(ini, g, 1)
    assert mixed.kspace_tensor_cores()              # the default engine takes the tensor cores
    mixed.set_kspace_engine("simt")
    assert not mixed.kspace_tensor_cores()
    mixed.set_kspace_engine("auto")
    assert mixed.kspace_tensor_cores()
    mixed.set_ewald(g["alpha"], g["rc"], 30)        # beyond the tensor-core shared memory
    assert not mixed.kspace_tensor_cores()
    with pytest.raises(Exception):
        mixed.set_kspace_engine("tc")
    fp64 = gpu_system(ini, g, 0)
    assert not fp64.kspace_tensor_cores()
    with pytest.raises(Exception):
        fp64.set_kspace_engine("tc")


def test_tc_accuracy_large():
    """N = 32768 polydisperse system: the accuracy of the tensor-core k space
    depends on how many MMAs one FP32 tensor-memory accumulator takes (its
    rounding error grows with that count), which small systems do not show.
    The structure factor, the k-space field and the k-space force stay within
    a few times the FP32 CUDA-core engine's error against FP64."""
    from test_gpu_parity import random_system_fast
    n = 32768
    ini, g = random_system_fast(n, seed=4, phi=0.10, B0=0.02)
    fAl, bAl, _ = scales(ini, g)
    ref, s = engines(ini, g)
    out = {}
    for name, sim in (("fp64", ref), ("tc", s["tc"]), ("simt", s["simt"])):
        B, F, _ = sim.CompInteractions()
        Br, Fr = sim.debug_real_part()
        out[name] = (B - Br, F - Fr, sf(sim))
    S0 = out["fp64"][2]
    srel = {k: np.sqrt(np.mean(np.abs(out[k][2] - S0) ** 2) / np.mean(np.abs(S0) ** 2)) for k in ("tc", "simt")}
    assert srel["tc"] < 3e-6 and srel["simt"] < 1e-6
    for k in ("tc", "simt"):
        assert O.rms_rel(out[k][0], out["fp64"][0], bAl) < 1e-6
        assert O.rms_rel(out[k][1], out["fp64"][1], fAl) < 1e-6


@pytest.mark.parametrize("n,kc", [(2, 3), (5, 6), (17, 8), (129, 12)])
def test_tc_small_and_ragged(n, kc):
    """Partial 16-particle stages, one mostly empty 128-particle scatter
    block, chunk ends inside a stage block."""
    ini, g = random_system(n, seed=100 + n, rc_frac=0.4)
    g["kc"] = kc
    fAl, bAl, _ = scales(ini, g)
    ref, s = engines(ini, g)
    assert s["tc"].kspace_tensor_cores()
    B0, F0, _ = ref.CompInteractions()
    Bt, Ft, _ = s["tc"].CompInteractions()
    Bs, Fs, _ = s["simt"].CompInteractions()
    assert np.all(np.isfinite(Bt)) and np.all(np.isfinite(Ft))
    assert O.rms_rel(Bt, B0, bAl) < TOL_MIXED and O.rms_rel(Ft, F0, fAl) < TOL_MIXED
    # with a handful of particles the k-space (periodic image) field is most
    # of the field, so the engines' FP32-level differences weigh more
    assert O.rms_rel(Bt, Bs, bAl) < 5e-6 and O.rms_rel(Ft, Fs, fAl) < 5e-6


def test_tiling_options_give_the_same_sums():
    """Every tensor-core tiling the autotuner may pick (structure-factor ring
    option, chunk-count multiple) computes the same k-space sums: field and
    force against the FP64 path within the mixed budget, and against each
    other to the tensor cores' accumulation error."""
    ini, g = random_system(3000, seed=17, rc_frac=0.25)
    fAl, bAl, _ = scales(ini, g)
    ref = gpu_system(ini, g, 0)
    B0, F0, _ = ref.CompInteractions()
    base = None
    for ring in (-1, 0, 3, 4, 5):
        for waves in (1, 2):
            sim = gpu_system(ini, g, 1)
            sim.set_kspace_tiling(ring, waves)
            assert sim.kspace_tensor_cores()
            B, F, _ = sim.CompInteractions()
            assert O.rms_rel(B, B0, bAl) < TOL_MIXED and O.rms_rel(F, F0, fAl) < TOL_MIXED, (ring, waves)
            if base is None:
                base = (B, F)
            else:
                assert O.rms_rel(B, base[0], bAl) < 1e-6 and O.rms_rel(F, base[1], fAl) < 1e-6, (ring, waves)
            sim.close()


def test_autotune_keeps_tiling_in_cache():
    """The autotuner's k-space choices (engine, ring, waves) are cached with
    the cut-off and applied again on a hit."""
    import md_sim_wolfschwenger_gb300 as m
    m.tune_cache_clear()
    ini, g = random_system(2048, seed=19, rc_frac=0.3)
    a = gpu_system(ini, g, 1)
    r1 = m.autotune_ewald_cached(a, 0.05)
    assert not r1[3]
    t1, e1 = a.kspace_tiling()[:2], a.kspace_tensor_cores()
    ini2, g2 = random_system(2048, seed=20, rc_frac=0.3)
    b = gpu_system(ini2, g2, 1)
    r2 = m.autotune_ewald_cached(b, 0.05)
    assert r2[3]
    assert b.kspace_tiling()[:2] == t1 and b.kspace_tensor_cores() == e1
    B, F, _ = b.CompInteractions()
    assert np.all(np.isfinite(B)) and np.all(np.isfinite(F))
    m.tune_cache_clear()
