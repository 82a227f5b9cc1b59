"""Writes tests/golden/stats_n216.npz: the reference simulator's own noisy
trajectories (its Mersenne-Twister thermal noise, oracle/_ref/ref_harness
built from the reference sources) for an ensemble of 16 seeds, reduced to the
statistics the noisy GPU runs are compared with.

Run from the repository root:  python tests/golden/make_stats.py
System: N = 216 monodisperse magnetite (20/30 nm), volume fraction 0.05,
20 mT along z, T = 300 K, viscosity 1e-3 Pa s, dt = 1e-12 s, 1000 steps,
all thermal noise on.  Each seed has its own initial state (random
sequential addition, m = n uniform on the sphere), stored so that the GPU
runs start from the same states; only the noise streams differ.
Stored per seed, every 10 steps: mz, MSD = MSDx + MSDy + MSDz, and the
orientation autocorrelations mean_i m_i(t).m_i(0), mean_i n_i(t).n_i(0);
per seed: D from the Einstein fit of MSD/3, and g(r) of the final frame.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402
import ref_io  # noqa: E402
from md_sim_wolfschwenger_gb300 import analysis  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
N, NSTEPS, SEEDS, EVERY, DT, VIS, B0, PHI = 216, 1000, 16, 10, 1e-12, 1e-3, 0.02, 0.05


def system(seed):
    ini = ref_io.ini_dict(npDim=6, magFluxDens=B0, volFrac=PHI, seed=seed, INIT_CONFIG_ROT=2)
    d = O.derive(ini)
    rng = np.random.default_rng(500 + seed)
    rMag = np.full(N, 1e-8)
    rHydr = rMag + 5e-9
    L = O.box_length(rHydr, PHI, d["my_pi"])
    pos, mm, ea = O.random_state(N, L, rHydr, rng, rot=2)
    alpha, kc, _ = O.ewald_for_rc(d, rMag, rHydr, L, 0.45 * L)
    return ini, dict(rMag=rMag, rHydr=rHydr, L=L, pos=pos, mm=mm, ea=ea, alpha=alpha, rc=0.45 * L, kc=kc)


def reduce(mm0, ea0, mms, eas, obs, pos_final, L):
    """Statistics of one trajectory: mms/eas (nsteps, 3, N) after each step."""
    idx = np.arange(EVERY - 1, NSTEPS, EVERY)
    cm = np.array([analysis.orientation_autocorrelation(mms[s], mm0) for s in idx])
    cn = np.array([analysis.orientation_autocorrelation(eas[s], ea0) for s in idx])
    msd = obs[:, 2] + obs[:, 3] + obs[:, 4]
    D, _, _ = analysis.einstein_diffusion(msd / 3.0, DT)
    _, g = analysis.radial_distribution(pos_final, L, 1e-8)
    return dict(mz=obs[idx, 1], msd=msd[idx], cm=cm, cn=cn, D=D, g=g)


def main():
    if not ref_io.available():
        sys.exit("build the reference harness first: oracle/build_ref.sh")
    keys = ("mz", "msd", "cm", "cn", "D", "g")
    acc = {k: [] for k in keys}
    init = {k: [] for k in ("pos", "mm", "ea", "alpha", "rc", "kc", "L")}
    ini0 = None
    for seed in range(1, SEEDS + 1):
        ini, s = system(seed)
        ini0 = ini0 or ini
        ref = ref_io.run_ref(ini, N, NSTEPS, DT, alpha=s["alpha"], rc=s["rc"], kc=s["kc"], vis=VIS,
                             pos=s["pos"].ravel(), mm=s["mm"].ravel(), ea=s["ea"].ravel())
        r = reduce(s["mm"], s["ea"], ref["mm"], ref["ea"], ref["obs"], ref["posF"], s["L"])
        for k in keys:
            acc[k].append(r[k])
        for k in init:
            init[k].append(s[k])
        print("seed", seed, "mz end", r["mz"][-1], "D", r["D"])
    out = {"ref_" + k: np.array(v) for k, v in acc.items()}
    out.update({"init_" + k: np.array(v) for k, v in init.items()})
    np.savez_compressed(os.path.join(OUT, "stats_n216.npz"), ini=json.dumps(ini0), n=N, nsteps=NSTEPS, every=EVERY,
                        dt=DT, vis=VIS, B0=B0, phi=PHI, **out)


if __name__ == "__main__":
    main()
