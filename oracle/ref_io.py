"""TEST INFRASTRUCTURE: configuration.ini writer and reference-harness driver.

Only tests/ (and tests/golden/make_golden.py) use this module.  It writes a
configuration.ini with the reference's section and key names
(src/configuration.ini:1-79 of MD_Sim_Wolfschwenger), feeds injected particle
states to oracle/_ref/ref_harness (built by oracle/build_ref.sh from the
reference's own sources), and parses the harness's binary dump.

Arrays are N x 3 column-major FP64, the layout of the reference's Eigen
ArrayXXd (src/typedefs.h:37-47): x[0..N), y[0..N), z[0..N).
"""
from __future__ import annotations

import copy
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")

# Section -> key -> value, in the order of src/configuration.ini.  Values are
# the monodisperse physics (20 nm magnetite cores, 5 nm shell, 10 mT);
# the physical constants are the reference's own (src/configuration.ini:69-79).
DEFAULT_INI = {
    "initial_configuration": {"INIT_CONFIG_ROT": 2, "INIT_CONFIG_TRANS": 1, "READ_FROM_FILE": "false"},
    "size_distribution": {"SIZE_DIST": 0},
    "mobilization": {"ENABLE_MOBILIZATION": "true"},
    "thermal_fluctuations": {"ENABLE_THERM_FIELD": "true", "ENABLE_THERM_TORQUE": "true",
                             "ENABLE_THERM_FORCE": "true", "seed": 1},
    "interactions": {"ENABLE_COATING_POT": "false"},
    "adaptive_timestepping_solver": {"SOLVER": 0},
    "particle_properties": {"npDim": 8, "magDamp": 0.1, "temp": 300.0, "satMag": 4.8e5, "anisEn": 1.1e4},
    "assemble_properties": {"rMagMean": 1e-8, "dShell": 5e-9, "volFrac": 0.05},
    "steric_repulsion": {"densSurfMol": 5e17},
    "vdw_attraction": {"hamaker": 33e-21},
    "electrostat_repulsion": {"z_valency": 1, "epsilon_r": 78.5, "gamma_0": 0.04, "conc": 50},
    "time_settings": {"tMag": 1e-8, "tRelax": 0, "deltaTinit": 1e-12},
    "external_magnetic_field_t": {"magFluxDens": 0.01},
    "solver_settings": {"absTol": 1e-4, "deltaTmin": 1e-14, "deltaTmax": 1e-9},
    "long_range_interactions": {"errTolEwald": 1e-5},
    "short_range_interactions": {"errTolSR": 0.01},
    "output_settings": {"npCoords": 100},
    "physical_constants": {"my_pi": 3.14159265359, "kB": 1.380648e-23, "gyroMr": 1.7595e11,
                           "avogadro": 6.02214076e23, "epsilon_0": 8.8541e-12, "el": 1.6e-19},
    "faster_calculation": {"facEwald": 1e-7},
}


def ini_dict(**overrides):
    """Copy of DEFAULT_INI with overrides given as KEY=value (key names are unique)."""
    d = copy.deepcopy(DEFAULT_INI)
    for k, v in overrides.items():
        for sec in d.values():
            if k in sec:
                sec[k] = v
                break
        else:
            raise KeyError(k)
    return d


def ini_text(d) -> str:
    out = []
    for sec, kv in d.items():
        out.append(f"[{sec}]")
        for k, v in kv.items():
            out.append(f"{k} = {v!r}" if isinstance(v, float) else f"{k} = {v}")
    return "\n".join(out) + "\n"


def write_ini(path, d):
    with open(path, "w") as f:
        f.write(ini_text(d))


def available() -> bool:
    return os.path.exists(REF_HARNESS)


def run_ref(ini, n, nsteps, dt, alpha=0.0, rc=0.0, kc=0.0, vis=0.0, rmag=None, pos=None,
            mm=None, ea=None, dump_level=1, ewald_search=False, timeout=3600, txt_dir=None, adaptive=False):
    """Runs the reference harness and returns a dict of arrays.

    Per-step arrays (dump_level >= 1) are stacked along axis 0 and reshaped to
    (nsteps, 3, N) so that [s, c, i] is component c of particle i.  With
    txt_dir, the reference's own writers also put its text output files
    there after the last step.
    """
    if not available():
        raise RuntimeError("reference harness not built (oracle/build_ref.sh)")
    with tempfile.TemporaryDirectory() as td:
        run = os.path.join(td, "run")
        os.mkdir(run)
        write_ini(os.path.join(td, "configuration.ini"), ini)
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            magic = 0x4D44524547 if adaptive else 0x4D44524546
            f.write(struct.pack("<8q", magic, n, nsteps, dump_level, int(ewald_search),
                                rmag is not None, pos is not None, mm is not None))
            f.write(struct.pack("<5d", dt, alpha, rc, kc, vis))
            if adaptive:
                f.write(struct.pack("<q", 1))
            for a in (rmag, pos, mm, ea):
                if a is not None:
                    f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        argv = [REF_HARNESS, fin, fout] + ([os.path.abspath(txt_dir)] if txt_dir else [])
        r = subprocess.run(argv, cwd=run, capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"ref_harness failed ({r.returncode}): {r.stderr[-2000:]}")
        raw = np.fromfile(fout, dtype=np.float64)
    return parse_out(raw, n, nsteps, dump_level, adaptive)


def parse_out(raw, n, nsteps, dump_level, adaptive=False):
    o = {}
    p = 0

    def take(k):
        nonlocal p
        v = raw[p:p + k]
        p += k
        return v

    o["lBox"], o["alpha"], o["rc"], o["kc"], o["rCutSR"], o["vis"] = take(6)
    o["rMag"], o["rHydr"] = take(n).copy(), take(n).copy()
    o["pos0"], o["mm0"], o["ea0"] = (take(3 * n).reshape(3, n).copy() for _ in range(3))
    names = ["B1", "F1", "thermTorque", "thermField", "thermForce", "posCorr"]
    steps = {k: [] for k in names + ["pairs", "B2", "pos", "mm", "ea", "obs", "dt0", "dtUsed"]}
    for _ in range(nsteps):
        if adaptive:
            steps["dt0"].append(take(1)[0])
        if dump_level >= 1:
            for k in names:
                steps[k].append(take(3 * n).reshape(3, n).copy())
            steps["pairs"].append(take(1)[0])
            steps["B2"].append(take(3 * n).reshape(3, n).copy())
            for k in ("pos", "mm", "ea"):
                steps[k].append(take(3 * n).reshape(3, n).copy())
        if dump_level >= 0:
            steps["obs"].append(take(8).copy())
        if adaptive:
            steps["dtUsed"].append(take(1)[0])
    for k, v in steps.items():
        if v:
            o[k] = np.array(v)
    o["posF"], o["mmF"], o["eaF"] = (take(3 * n).reshape(3, n).copy() for _ in range(3))
    o["elapsed"] = take(1)[0]
    assert p == raw.size, (p, raw.size)
    return o


def reference_root():
    """Root of the reference sources the harness was built from (recorded by
    oracle/build_ref.sh in oracle/_ref/reference_root), or None."""
    f = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "reference_root")
    try:
        root = open(f).read().strip()
    except OSError:
        return None
    return root if os.path.isdir(root) else None
