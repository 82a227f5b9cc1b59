"""Writes the golden fixtures of tests/golden/ by running the reference
simulator's own code (oracle/_ref/ref_harness, built from the reference
sources by oracle/build_ref.sh) on seeded initial states.

Run from the repository root:  python tests/golden/make_golden.py [case ...]
Each case stores its inputs (configuration, radii, state, Ewald parameters,
dt) and the reference's FP64 outputs per step: B after CompInteractions, F
(including the thermal force), the thermal arrays, the positions after the
overlap push, B at the Heun predictor, the state after the step and the
per-step records {t, mz, MSDx, MSDy, MSDz, Pxy, Pxz, Pyz}.  Cases with
txt=True also keep the text files the reference's own writers produce after
the last step (data.txt, coords.txt, dtMean/P/MSD/mz/t .txt) in
tests/golden/<case>_txt/.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402
import ref_io  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
VIS = 1e-3  # water at room temperature, 1 mPa s (the reference's Vogel formula gives 8.5e-4 at 300 K)


def case(name, n, nsteps, rc_frac, seed, noise=True, coating=False, lognormal=False, overlap=False, dt=1e-12,
         B0=0.01, rot=3, txt=False, solver=None, absTol=1e-4):
    """solver None: fixed step (Heun, every step accepted); 0, 1, 2: the
    reference's adaptive step control with that SOLVER, starting from dt."""
    extra = {} if solver is None else dict(SOLVER=solver, absTol=absTol, deltaTinit=dt)
    ini = ref_io.ini_dict(npDim=round(n ** (1 / 3)) if round(n ** (1 / 3)) ** 3 == n else 4,
                          ENABLE_THERM_FIELD="true" if noise else "false",
                          ENABLE_THERM_TORQUE="true" if noise else "false",
                          ENABLE_THERM_FORCE="true" if noise else "false",
                          ENABLE_COATING_POT="true" if coating else "false", magFluxDens=B0, seed=seed, **extra)
    d = O.derive(ini)
    rng = np.random.default_rng(seed)
    if lognormal:
        rMag = 1e-8 * np.exp(0.2 * rng.standard_normal(n))
    else:
        rMag = np.full(n, 1e-8)
    if coating:
        rHydr = np.array([max(O_eff(d, 2 * r) / 2, r) for r in rMag])
    else:
        rHydr = rMag + 5e-9
    L = O.box_length(rHydr, d["volFrac"], d["my_pi"])
    pos, mm, ea = O.random_state(n, L, rHydr, rng, rot=rot)
    if overlap:
        # push a few pairs into core overlap
        for a in range(0, 8, 2):
            pos[:, a + 1] = pos[:, a] + np.array([1.2e-8, 0.8e-8, 0.0])[:, None][:, 0] * (1 + 0.1 * a)
    alpha, kc, _ = O.ewald_for_rc(d, rMag, rHydr, L, rc_frac * L)
    txt_dir = None
    if txt:
        txt_dir = os.path.join(OUT, name + "_txt")
        os.makedirs(txt_dir, exist_ok=True)
    ref = ref_io.run_ref(ini, n, nsteps, dt, alpha=alpha, rc=rc_frac * L, kc=kc, vis=VIS,
                         rmag=rMag if (lognormal or coating) else None, pos=pos.ravel(), mm=mm.ravel(),
                         ea=ea.ravel(), txt_dir=txt_dir, adaptive=solver is not None)
    assert abs(ref["lBox"] - L) <= 1e-15 * L, (ref["lBox"], L)
    out = dict(n=n, nsteps=nsteps, dt=dt, alpha=alpha, rc=rc_frac * L, kc=kc, vis=VIS, lBox=L, rMag=rMag,
               rHydr=ref["rHydr"], pos=pos, mm=mm, ea=ea, rCutSR=ref["rCutSR"])
    for k in ("B1", "F1", "thermTorque", "thermField", "thermForce", "posCorr", "B2", "pos", "mm", "ea", "obs",
              "pairs"):
        out["ref_" + k] = ref[k]
    out["ref_posF"], out["ref_mmF"], out["ref_eaF"] = ref["posF"], ref["mmF"], ref["eaF"]
    if solver is not None:
        out["solver"], out["absTol"] = solver, absTol
        out["ref_dt0"], out["ref_dtUsed"] = ref["dt0"], ref["dtUsed"]
    np.savez_compressed(os.path.join(OUT, name + ".npz"), ini=json.dumps(ini), **out)
    print(name, "n", n, "L", L, "alpha*L", alpha * L, "kc", kc, "pairs", ref["pairs"])


def O_eff(d, dmag):
    # IntegralEffDiameter (src/mathFun.cpp:27-43), restated for the fixture inputs
    import math
    eff = d["effLenSurfMol"]
    hi = dmag + 2 * eff
    h = hi / 1000

    def f(r):
        dd = dmag + 2 * eff
        return 1 - math.exp(-d["my_pi"] * dmag * dmag * d["densSurfMol"] / (2 * eff) *
                            (dd - r * (math.log(dd / (r + 1e-20)) + 1)))

    return sum(h / 6 * (f(i * h) + 4 * f((i + 0.5) * h) + f((i + 1) * h)) for i in range(1000))


if __name__ == "__main__":
    if not ref_io.available():
        sys.exit("build the reference harness first: oracle/build_ref.sh")
    CASES = {
        "n64_noiseoff": lambda: case("n64_noiseoff", 64, 3, 0.45, seed=11, noise=False),
        "n64_refnoise": lambda: case("n64_refnoise", 64, 3, 0.45, seed=12, noise=True),
        "n512_cfg1_noiseoff": lambda: case("n512_cfg1_noiseoff", 512, 2, 0.45, seed=1, noise=False),
        "n512_cfg1_refnoise": lambda: case("n512_cfg1_refnoise", 512, 2, 0.3, seed=1, noise=True),
        "n64_coating": lambda: case("n64_coating", 64, 1, 0.45, seed=13, noise=False, coating=True),
        "n64_lognormal": lambda: case("n64_lognormal", 64, 2, 0.4, seed=14, noise=True, lognormal=True),
        "n64_overlap": lambda: case("n64_overlap", 64, 1, 0.45, seed=15, noise=False, overlap=True),
        "n64_outputs": lambda: case("n64_outputs", 64, 6, 0.4, seed=16, noise=True, lognormal=True, txt=True),
        # adaptive step control (SOLVER 0, 1, 2), with rejections
        "n64_adapt_he": lambda: case("n64_adapt_he", 64, 12, 0.45, seed=21, rot=4, B0=0.02, solver=0),
        "n64_adapt_bs": lambda: case("n64_adapt_bs", 64, 12, 0.45, seed=22, rot=4, B0=0.02, solver=1),
        "n64_adapt_dp": lambda: case("n64_adapt_dp", 64, 12, 0.45, seed=23, rot=4, B0=0.02, solver=2, dt=2e-12,
                                     absTol=3e-5),
    }
    for name in (sys.argv[1:] or CASES):
        CASES[name]()
