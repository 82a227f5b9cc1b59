"""Shared test helpers: one system description handed to the reference
fixtures, the C oracle and the CUDA library alike."""
import json
import os
import tempfile

import numpy as np

import oracle as O
import ref_io

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["n64_noiseoff", "n64_refnoise", "n512_cfg1_noiseoff", "n512_cfg1_refnoise", "n64_coating",
                "n64_lognormal", "n64_overlap", "n64_outputs"]

# Tolerances (contact-normalised RMS, the metric of CheckEwaldSum,
# src/interaction.cpp:741-754).
TOL_FP64 = 1e-10   # FP64 GPU vs FP64 CPU: summation order only
TOL_MIXED = 1e-5   # mixed precision vs FP64: the 1e-5 Ewald error budget


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    ini = json.loads(str(d["ini"]))
    g = {k: d[k] for k in d.files if k != "ini"}
    for k in ("n", "nsteps", "kc"):
        g[k] = int(g[k])
    for k in ("dt", "alpha", "rc", "vis", "lBox", "rCutSR"):
        g[k] = float(g[k])
    return ini, g


def md_config(ini, vis=None, n=None):
    """md_config loaded through md_config_load_ini from the INI text."""
    from md_sim_wolfschwenger_gb300 import Configuration
    with tempfile.NamedTemporaryFile("w", suffix=".ini", delete=False) as f:
        f.write(ref_io.ini_text(ini))
        path = f.name
    try:
        cfg = Configuration.from_ini(path)
    finally:
        os.unlink(path)
    kw = {}
    if vis is not None:
        kw["visOverride"] = vis
    if n is not None and n != cfg.numb_part():
        kw["numbPartOverride"] = n
    if kw:
        cfg.set(**kw)
    return cfg


def gpu_system(ini, g, precision, noise=0, seed=1):
    from md_sim_wolfschwenger_gb300 import Simulation
    cfg = md_config(ini, vis=g["vis"], n=g["n"])
    sim = Simulation(cfg, g["n"], precision, rMag=g["rMag"], rHydr=g["rHydr"])
    sim.set_ewald(g["alpha"], g["rc"], g["kc"])
    sim.set_state(g["pos"], g["mm"], g["ea"], reset=True)
    sim.set_noise(noise, seed)
    return sim


def oracle_system(ini, g, overlap_mode=1):
    d = O.derive(ini)
    orc = O.Oracle(d, g["rMag"], g["rHydr"], g["lBox"], g["alpha"], g["rc"], g["kc"], vis=g["vis"],
                   overlap_mode=overlap_mode, rCutSR=g["rCutSR"])
    orc.set_state(g["pos"], g["mm"], g["ea"])
    return orc


def scales(ini, g):
    d = O.derive(ini)
    return O.contact_scales(d, g["rMag"], g["rHydr"])


def xi_from_ref(ini, g, step):
    d = O.derive(ini)
    sT, sB, sF = O.noise_scales(d, g["rMag"], g["rHydr"], g["dt"], g["vis"])
    xi = np.zeros((3, 3, g["n"]))
    if d["ENABLE_THERM_TORQUE"]:
        xi[0] = g["ref_thermTorque"][step] / sT
    if d["ENABLE_THERM_FIELD"]:
        xi[1] = g["ref_thermField"][step] / sB
    if d["ENABLE_THERM_FORCE"]:
        xi[2] = g["ref_thermForce"][step] / sF
    return xi


def torque(mm, B, magMom):
    """tau = mu x B (CheckEwaldSum's torque, src/interaction.cpp:702)."""
    mu = mm * magMom[None, :]
    return np.cross(mu.T, B.T).T


def random_system(n, seed, rc_frac=0.3, phi=0.05, lognormal=False, noise=False, B0=0.01, min_gap=0.0):
    """Seeded system: monodisperse 20 nm magnetite cores with a 5 nm shell in a
    10 mT field unless overridden."""
    ini = ref_io.ini_dict(volFrac=phi, magFluxDens=B0, ENABLE_THERM_FIELD="true" if noise else "false",
                          ENABLE_THERM_TORQUE="true" if noise else "false",
                          ENABLE_THERM_FORCE="true" if noise else "false", seed=seed)
    d = O.derive(ini)
    rng = np.random.default_rng(seed)
    rMag = 1e-8 * np.exp(0.2 * rng.standard_normal(n)) if lognormal else np.full(n, 1e-8)
    rHydr = rMag + 5e-9
    L = O.box_length(rHydr, phi, d["my_pi"])
    pos, mm, ea = O.random_state(n, L, rHydr, rng, rot=3, min_gap=min_gap)
    alpha, kc, _ = O.ewald_for_rc(d, rMag, rHydr, L, rc_frac * L)
    g = dict(n=n, dt=1e-12, alpha=alpha, rc=rc_frac * L, kc=kc, vis=1e-3, lBox=L, rMag=rMag, rHydr=rHydr,
             pos=pos, mm=mm, ea=ea, rCutSR=O.cutoff_sr(d, rMag, rHydr))
    return ini, g
