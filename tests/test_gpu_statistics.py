"""Noise on: the GPU's Philox thermal noise against the reference's own
Mersenne-Twister noise, statistically.  16 seeds, each starting from the same
state in both arms (tests/golden/stats_n216.npz, written by
tests/golden/make_stats.py with the reference simulator's code), N = 216,
20 mT, 1000 steps of 1 ps.  Compared per seed pair (same initial state,
independent noise): the magnetisation m_z(t), the mean-squared displacement,
the orientation autocorrelations of moments and easy axes, the Einstein
diffusion coefficient (mFiles/eval_diffusion.m) and g(r) of the final frame
(mFiles/radial_dist_fun.m).  Criterion: |mean paired difference| <= 4.5
standard errors (+ a small floor for FP32 rounding on the mixed path)."""
import json
import os

import numpy as np
import pytest

from helpers import GOLDEN, md_config
import md_sim_wolfschwenger_gb300 as m
from md_sim_wolfschwenger_gb300 import analysis

pytestmark = pytest.mark.gpu

Z = 4.5


def _load():
    d = np.load(os.path.join(GOLDEN, "stats_n216.npz"), allow_pickle=False)
    ini = json.loads(str(d["ini"]))
    return ini, {k: d[k] for k in d.files if k != "ini"}


def _gpu_ensemble(ini, f, prec):
    n, nsteps, every, dt = int(f["n"]), int(f["nsteps"]), int(f["every"]), float(f["dt"])
    out = {k: [] for k in ("mz", "msd", "cm", "cn", "D", "g")}
    rMag = np.full(n, 1e-8)
    rHydr = rMag + 5e-9
    for s in range(f["init_pos"].shape[0]):
        ini_s = json.loads(json.dumps(ini))
        ini_s["thermal_fluctuations"]["seed"] = s + 1
        cfg = md_config(ini_s, vis=float(f["vis"]), n=n)
        sim = m.Simulation(cfg, n, prec, rMag=rMag, rHydr=rHydr)
        sim.set_ewald(float(f["init_alpha"][s]), float(f["init_rc"][s]), int(f["init_kc"][s]))
        mm0, ea0 = f["init_mm"][s], f["init_ea"][s]
        sim.set_state(f["init_pos"][s], mm0, ea0)
        sim.set_noise(m.MD_NOISE_PHILOX, 9000 + s)
        cm, cn = [], []
        for _ in range(nsteps // every):
            sim.step(every, dt)
            _, mm_t, ea_t = sim.get_state()
            cm.append(analysis.orientation_autocorrelation(mm_t, mm0))
            cn.append(analysis.orientation_autocorrelation(ea_t, ea0))
        rec = sim.records()
        pos, _, _ = sim.get_state()
        sim.close()
        idx = np.arange(every - 1, nsteps, every)
        msd = rec[:, 2] + rec[:, 3] + rec[:, 4]
        out["mz"].append(rec[idx, 1])
        out["msd"].append(msd[idx])
        out["cm"].append(np.array(cm))
        out["cn"].append(np.array(cn))
        out["D"].append(analysis.einstein_diffusion(msd / 3.0, dt)[0])
        out["g"].append(analysis.radial_distribution(pos, float(f["init_L"][s]), 1e-8)[1])
    return {k: np.array(v) for k, v in out.items()}


def _paired(a, b, floor):
    d = np.asarray(a) - np.asarray(b)
    mean, se = analysis.ensemble_mean(d)
    ok = np.abs(mean) <= Z * se + floor
    return bool(np.all(ok)), mean, se


@pytest.mark.parametrize("prec", [m.MD_PREC_MIXED, m.MD_PREC_FP64])
def test_noisy_ensemble_matches_reference_statistics(prec):
    ini, f = _load()
    g = _gpu_ensemble(ini, f, prec)
    pts = slice(9, None, 10)  # every 100 steps
    for key, floor in (("mz", 1e-4), ("cm", 1e-4), ("cn", 1e-6)):
        ok, mean, se = _paired(g[key][:, pts], f["ref_" + key][:, pts], floor)
        assert ok, (key, mean, se)
    # MSD: relative to its size
    scale = f["ref_msd"][:, pts].mean(axis=0)
    ok, mean, se = _paired(g["msd"][:, pts] / scale, f["ref_msd"][:, pts] / scale, 1e-4)
    assert ok, ("msd", mean, se)
    ok, mean, se = _paired(g["D"] / 1e-11, f["ref_D"] / 1e-11, 1e-4)
    assert ok, ("D", mean, se)
    # g(r) in 25 coarse bins
    gc = g["g"].reshape(g["g"].shape[0], 25, 20).mean(axis=2)
    rc = f["ref_g"].reshape(f["ref_g"].shape[0], 25, 20).mean(axis=2)
    ok, mean, se = _paired(gc, rc, 1e-3 * max(1.0, float(rc.max())))
    assert ok, ("g", mean, se)
    # physics: the Einstein coefficient is the free-particle kT / (6 pi eta r_h) within the scatter
    d_theory = 1.380648e-23 * 300.0 / (6 * np.pi * float(f["vis"]) * 15e-9)
    mean, se = analysis.ensemble_mean(g["D"])
    assert abs(mean - d_theory) <= Z * se + 0.02 * d_theory, (mean, se, d_theory)
