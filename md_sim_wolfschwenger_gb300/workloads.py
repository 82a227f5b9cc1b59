"""The benchmark systems, named by what they are.

Each workload is a magnetite suspension (Ms 4.8e5 A/m, K 1.1e4 J/m^3,
damping 0.1, 5 nm shell, T = 300 K, viscosity 1e-3 Pa s, dt = 1e-12 s,
Philox thermal noise, Ewald parameters for 1e-5 relative force error) with
the particle count, size distribution, volume fraction and static field
below.  `WORKLOADS` is plain data (importable without the CUDA library);
`config` and `state` build the system through the library's host code
(md_config_derive, md_init_system: log-normal radii, random sequential
addition placed largest first, moments and easy axes independent and
uniform on the sphere).
"""
from __future__ import annotations

COMMON = ("magnetite (Ms 4.8e5 A/m, K 1.1e4 J/m^3, damping 0.1), 5 nm shell, T=300 K, viscosity 1e-3 Pa s, "
          "dt=1e-12 s, Philox thermal noise, Ewald at 1e-5 relative force error")

WORKLOADS = {
    # single large instance: chain-forming polydisperse suspension
    "large": dict(n=32768, median=1e-8, sigma=0.2, phi=0.10, B0=0.02,
                  desc="single large instance: N=32768, log-normal core diameters (median 20 nm, sigma 0.2), "
                       "volume fraction 0.10, static 20 mT, " + COMMON),
    # the reference's own CPU-runnable case (monodisperse, N=512)
    "small": dict(n=512, median=1e-8, sigma=0.0, phi=0.05, B0=0.01,
                  desc="plain case: N=512 monodisperse 20/30 nm, volume fraction 0.05, static 10 mT, " + COMMON),
    # stress instance: dense, strongly polydisperse, k space dominant
    "stress": dict(n=131072, median=1.25e-8, sigma=0.25, phi=0.20, B0=0.03,
                   desc="stress instance: N=131072, log-normal core diameters (median 25 nm, sigma 0.25), "
                        "volume fraction 0.20, static 30 mT, " + COMMON),
}


def spec(name: str, n: int | None = None) -> dict:
    """The workload's parameters; n overrides the particle count."""
    w = dict(WORKLOADS[name])
    if n and n != w["n"]:
        w["desc"] = w["desc"].replace(f"N={w['n']}", f"N={n}")
        w["n"] = int(n)
    return w


def config(w: dict, seed: int):
    """Configuration (INI keys) of workload spec w."""
    from . import MD_NOISE_PHILOX, MD_PREC_MIXED, Configuration
    cfg = Configuration.default()
    cfg.set(SIZE_DIST=1 if w["sigma"] > 0 else 0, rMagMean=w["median"], sigmaLog=w["sigma"], dShell=5e-9,
            volFrac=w["phi"], magFluxDens=w["B0"], tMag=1.0, tRelax=0.0, deltaTinit=1e-12, satMag=4.8e5,
            anisEn=1.1e4, magDamp=0.1, temp=300.0, visOverride=1e-3, numbPartOverride=w["n"], errTolEwald=1e-5,
            seed=seed, SOLVER=0, ENABLE_MOBILIZATION=1, ENABLE_THERM_FIELD=1, ENABLE_THERM_TORQUE=1,
            ENABLE_THERM_FORCE=1, ENABLE_COATING_POT=0, INIT_CONFIG_ROT=4, INIT_CONFIG_TRANS=1,
            precision=MD_PREC_MIXED, noise=MD_NOISE_PHILOX)
    return cfg


def state(w: dict, seed: int):
    """(rMag, rHydr, L, pos, mm, ea) of workload spec w for this seed."""
    from .batch import init_system
    rMag, rHydr, pos, mm, ea, L = init_system(config(w, seed), w["n"], 1000 + seed)
    return rMag, rHydr, L, pos, mm, ea


def contact_scales(cfg, rMag, rHydr):
    """Contact force, field and torque of the smallest particles
    (CompEwaldParams / CheckEwaldSum, src/interaction.cpp:180-181, 743-753):
    the scales of the reference's relative error."""
    import numpy as np
    mu0, pi, ms = cfg.c.mu0, cfg.c.my_pi, cfg.c.satMag
    mmin = float(np.min(ms * 4.0 / 3.0 * pi * np.asarray(rMag) ** 3))
    rh = float(np.min(rHydr))
    return (3 * mu0 * mmin ** 2 / (2 * pi * (2 * rh) ** 4), mu0 * mmin / (2 * pi * (2 * rh) ** 3),
            mmin ** 2 * mu0 / (16 * pi * rh ** 3))


def mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, ewald, theta=None):
    """CompInteractions on the same state through the mixed and the plain
    FP64 path: contact-normalised RMS differences of B, F and the torque
    mu x B (the metric of CheckEwaldSum, src/interaction.cpp:741-754), and
    the FP64 B, F.  theta: strong-pair threshold of the mixed path (None:
    the library default)."""
    import math

    import numpy as np

    from . import MD_PREC_FP64, MD_PREC_MIXED, Simulation
    n = len(rMag)
    out = {}
    strong = 0
    for prec in (MD_PREC_MIXED, MD_PREC_FP64):
        sim = Simulation(cfg, n, prec, rMag=rMag, rHydr=rHydr)
        sim.set_state(pos, mm, ea)
        sim.set_ewald(*ewald)
        if prec == MD_PREC_MIXED and theta is not None:
            sim.set_strong_pairs(theta)
        out[prec] = sim.CompInteractions()[:2]
        if prec == MD_PREC_MIXED:
            strong = sim.strong_pairs()
        sim.close()
    fAl, bAl, tAl = contact_scales(cfg, rMag, rHydr)
    mom = cfg.c.satMag * 4.0 / 3.0 * cfg.c.my_pi * np.asarray(rMag) ** 3

    def rms(a, b, s):
        d = np.asarray(a) - np.asarray(b)
        return math.sqrt(float((d * d).sum()) / d.shape[-1]) / s

    tq = {p: np.cross((np.asarray(mm) * mom).T, out[p][0].T).T for p in out}
    err = {"B": rms(out[MD_PREC_MIXED][0], out[MD_PREC_FP64][0], bAl),
           "F": rms(out[MD_PREC_MIXED][1], out[MD_PREC_FP64][1], fAl),
           "torque": rms(tq[MD_PREC_MIXED], tq[MD_PREC_FP64], tAl), "strong_entries": strong}
    return err, out[MD_PREC_FP64]
