"""TEST INFRASTRUCTURE: ctypes wrapper of the C oracle (oracle/md_oracle.c).

This module is the checker.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py import it; the product never does.  It also holds
a Python restatement of the reference's configuration derivations
(src/configuration.cpp:38-84 of MD_Sim_Wolfschwenger) and initial-state
helpers, so that a test can describe a system once and hand it to the
reference harness, to this oracle and to the CUDA library alike.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmd_oracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False) -> str:
    """Compiles md_oracle.c with gcc (portable flags only: x86 here, Arm on the GPU machine)."""
    src = os.path.join(HERE, "md_oracle.c")
    with _lock:
        if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
                os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "md_oracle.h"))):
            os.makedirs(BUILD, exist_ok=True)
            tmp = LIB + f".{os.getpid()}.tmp"
            subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-std=c11", "-fPIC", "-shared", "-pthread", "-o", tmp, src,
                                   "-lm"])
            os.replace(tmp, LIB)
    return LIB


class Adapt(C.Structure):
    _fields_ = [("solver", C.c_int64), ("absTol", C.c_double), ("dtMin", C.c_double), ("dtMax", C.c_double)]


class Cfg(C.Structure):
    _fields_ = [("n", C.c_int64), ("lBox", C.c_double), ("alpha", C.c_double), ("rCutLR", C.c_double),
                ("nc", C.c_int64), ("rCutSR", C.c_double)] + [
        (k, C.c_double) for k in ("my_pi", "facEwald", "irPi", "kB", "temp", "magDamp", "gyroMr", "satMag",
                                  "anisEn", "anisConst", "velMmConst", "effLenSurfMol", "sterRepFac",
                                  "electrostatRepFac", "kappa", "hamaker", "magFluxDens", "tMag")] + [
        (k, C.c_int64) for k in ("enable_mobilization", "enable_therm_torque", "enable_therm_field",
                                 "enable_therm_force", "enable_coating", "field_kind")] + [
        ("field_amp", C.c_double), ("field_freq", C.c_double), ("overlap_mode", C.c_int64)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER(C.c_double)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Cfg)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_props.argtypes = [C.c_void_p, P, P, C.c_double]
        L.orc_set_state.argtypes = [C.c_void_p, P, P, P, C.c_double]
        L.orc_get_state.argtypes = [C.c_void_p, P, P, P, P]
        L.orc_reset_observables.argtypes = [C.c_void_p]
        L.orc_compute_interactions.argtypes = [C.c_void_p, P, P, P]
        L.orc_compute_field.argtypes = [C.c_void_p, P, P]
        L.orc_step.argtypes = [C.c_void_p, C.c_double, C.c_int, P, C.c_uint64, P, P, P, P]
        L.orc_thermal.argtypes = [C.c_void_p, C.c_double, C.c_int, P, C.c_uint64, P, P, P]
        L.orc_step_adaptive.argtypes = [C.c_void_p, C.POINTER(Adapt), P, C.c_int, P, C.c_uint64, P, P,
                                        C.POINTER(C.c_int)]
        L.orc_philox_normals.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, P]
        L.orc_fun_real_error.restype = C.c_double
        L.orc_fun_real_error.argtypes = [C.c_double] * 8
        L.orc_fun_rez_error.restype = C.c_double
        L.orc_fun_rez_error.argtypes = [C.c_double] * 9
        L.orc_ewald_for_rc.restype = C.c_int
        L.orc_ewald_for_rc.argtypes = [C.c_double] * 8 + [P, P]
        L.orc_pairs.restype = C.c_int64
        L.orc_pairs.argtypes = [C.c_void_p]
        L.orc_last_seconds.restype = C.c_double
        L.orc_last_seconds.argtypes = [C.c_void_p]
        L.orc_set_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_rsa.restype = C.c_int
        L.orc_rsa.argtypes = [C.c_int64, C.c_double, P, C.c_uint64, C.c_int64, P]
        L.orc_rsa_philox.restype = C.c_int
        L.orc_rsa_philox.argtypes = [C.c_int64, C.c_double, P, C.c_uint64, C.c_void_p, C.c_int64, P, C.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


# ----------------------------------------------------------- configuration


def derive(ini) -> dict:
    """Flat dict of Configuration values (src/configuration.cpp:11-84)."""
    g = {}
    for sec in ini.values():
        g.update(sec)
    b = lambda v: str(v).strip().lower() in ("true", "yes", "on", "1")
    pi = float(g["my_pi"])
    d = dict(
        INIT_CONFIG_ROT=int(g["INIT_CONFIG_ROT"]), INIT_CONFIG_TRANS=int(g["INIT_CONFIG_TRANS"]),
        SIZE_DIST=int(g["SIZE_DIST"]), ENABLE_MOBILIZATION=b(g["ENABLE_MOBILIZATION"]),
        ENABLE_THERM_FIELD=b(g["ENABLE_THERM_FIELD"]), ENABLE_THERM_TORQUE=b(g["ENABLE_THERM_TORQUE"]),
        ENABLE_THERM_FORCE=b(g["ENABLE_THERM_FORCE"]), seed=int(g["seed"]),
        ENABLE_COATING_POT=b(g["ENABLE_COATING_POT"]), SOLVER=int(g["SOLVER"]),
        npDim=int(g["npDim"]))
    for k in ("magDamp", "temp", "satMag", "anisEn", "rMagMean", "dShell", "volFrac", "densSurfMol", "hamaker",
              "z_valency", "epsilon_r", "gamma_0", "conc", "tMag", "tRelax", "deltaTinit", "magFluxDens",
              "absTol", "deltaTmin", "deltaTmax", "errTolEwald", "errTolSR", "npCoords", "my_pi", "kB",
              "gyroMr", "avogadro", "epsilon_0", "el", "facEwald"):
        d[k] = float(g[k])
    T, kB, el, z = d["temp"], d["kB"], d["el"], d["z_valency"]
    d["effLenSurfMol"] = 0.2 * d["rMagMean"]
    d["mu0"] = 4.0 * pi * math.pow(10, -7)
    d["numbPart"] = d["npDim"] ** 3
    d["velMmConst"] = d["gyroMr"] / (1.0 + math.pow(d["magDamp"], 2.0))
    d["anisConst"] = 2.0 * d["anisEn"] / d["satMag"]
    d["sterRepFac"] = 4 * kB * T * pi * d["densSurfMol"] / (2 * d["effLenSurfMol"])
    d["gamma"] = math.tanh(z * el * d["gamma_0"] / (4 * kB * T))
    d["epsilon"] = d["epsilon_0"] * d["epsilon_r"]
    d["kappa"] = math.sqrt(el * el * d["avogadro"] * d["conc"] * z * z / (d["epsilon"] * kB * T))
    d["electrostatRepFac"] = (d["kappa"] * 64 * pi * d["epsilon"] * math.pow(kB * T / (z * el), 2.0) *
                              d["gamma"] * d["gamma"])
    d["irPi"] = 1 / math.sqrt(pi)
    d["vis"] = (2.414e-5) * math.pow(10, 247.8 / (T - 140))
    d["sigma"] = math.sqrt(0.1) * 2.0 * d["rMagMean"]
    d["tEnd"] = d["tMag"] + d["tRelax"]
    return d


def box_length(rHydr, volFrac, my_pi):
    """InitSimulation: L = (sum V_h / phi)^(1/3) (simulation.cpp:56)."""
    volHydr = 4.0 / 3.0 * my_pi * np.asarray(rHydr) ** 3.0
    return math.pow(float(volHydr.sum()) / volFrac, 1.0 / 3.0)


def cutoff_sr(d, rMag, rHydr):
    """InitCutOffSR (interaction.cpp:20-57)."""
    rMax = float(np.max(rMag))
    if not d["ENABLE_COATING_POT"]:
        return 2 * rMax
    mMax = float(np.max(d["satMag"] * 4.0 / 3.0 * d["my_pi"] * np.asarray(rMag) ** 3.0))
    c1 = 128 * d["hamaker"] * math.pow(rMax, 6.0) * d["my_pi"] / (18 * d["mu0"] * mMax * mMax)

    def f(x, der):
        if der:
            return c1 * (4 * rMax * rMax + 3 * x * x) / math.pow(4 * rMax * rMax - x * x, 3.0)
        return c1 * x / math.pow(x * x - 4 * rMax * rMax, 2.0) - d["errTolSR"]

    x = 1.1 * 2 * rMax
    while True:
        x -= f(x, False) / f(x, True)
        if abs(f(x, False)) <= 1e-7:
            break
    if x < 2 * float(np.max(rHydr)):
        raise ValueError("particles can only interact if they overlap")
    return x


def contact_scales(d, rMag, rHydr):
    """F, B and torque contact values (interaction.cpp:180-181, 743-753)."""
    mu0, pi = d["mu0"], d["my_pi"]
    mmin = float(np.min(d["satMag"] * 4.0 / 3.0 * pi * np.asarray(rMag) ** 3.0))
    rh = float(np.min(rHydr))
    fAl = 3 * mu0 * math.pow(mmin, 2.0) / (2.0 * pi * math.pow(2.0 * rh, 4.0))
    bAl = mu0 * mmin / (2 * pi * math.pow(2 * rh, 3.0))
    tAl = math.pow(mmin, 2.0) * mu0 / (16.0 * pi * math.pow(rh, 3.0))
    return fAl, bAl, tAl


def rms_rel(a, b, scale):
    """RMS over particles of |a_i - b_i| / scale; a, b shaped (3, N) (interaction.cpp:741-754)."""
    diff = np.asarray(a) - np.asarray(b)
    return math.sqrt(float((diff * diff).sum(axis=0).sum()) / diff.shape[-1]) / scale


def ewald_for_rc(d, rMag, rHydr, lBox, rc):
    """Reference grid scan for alpha and kc at a given rc; kc is rounded like
    interaction.cpp:304.  Returns (alpha, kc_int, kc_raw)."""
    n = len(rMag)
    m = d["satMag"] * 4.0 / 3.0 * d["my_pi"] * np.asarray(rMag) ** 3.0
    M = float((m ** 2.0).sum())
    fAl, _, _ = contact_scales(d, rMag, rHydr)
    a, k = C.c_double(), C.c_double()
    rcode = lib().orc_ewald_for_rc(rc, M, fAl, lBox, float(n), d["facEwald"], d["my_pi"], d["errTolEwald"],
                                   C.byref(a), C.byref(k))
    if rcode not in (0, 1):
        raise ValueError(f"no kc for rc={rc} (code {rcode})")
    return a.value, int(math.floor(k.value + 0.5)), k.value


# ------------------------------------------------------------------ oracle


class Oracle:
    """One simulation instance on the CPU (FP64, one thread)."""

    def __init__(self, d, rMag, rHydr, lBox, alpha, rc, kc, vis=None, overlap_mode=0,
                 field_kind=0, field_amp=0.0, field_freq=0.0, rCutSR=None):
        self.n = n = len(rMag)
        self.d = d
        cfg = Cfg(n=n, lBox=lBox, alpha=alpha, rCutLR=rc, nc=int(kc),
                  rCutSR=cutoff_sr(d, rMag, rHydr) if rCutSR is None else rCutSR,
                  my_pi=d["my_pi"], facEwald=d["facEwald"], irPi=d["irPi"], kB=d["kB"], temp=d["temp"],
                  magDamp=d["magDamp"], gyroMr=d["gyroMr"], satMag=d["satMag"], anisEn=d["anisEn"],
                  anisConst=d["anisConst"], velMmConst=d["velMmConst"], effLenSurfMol=d["effLenSurfMol"],
                  sterRepFac=d["sterRepFac"], electrostatRepFac=d["electrostatRepFac"], kappa=d["kappa"],
                  hamaker=d["hamaker"], magFluxDens=d["magFluxDens"], tMag=d["tMag"],
                  enable_mobilization=int(d["ENABLE_MOBILIZATION"]),
                  enable_therm_torque=int(d["ENABLE_THERM_TORQUE"]),
                  enable_therm_field=int(d["ENABLE_THERM_FIELD"]),
                  enable_therm_force=int(d["ENABLE_THERM_FORCE"]), enable_coating=int(d["ENABLE_COATING_POT"]),
                  field_kind=field_kind, field_amp=field_amp, field_freq=field_freq, overlap_mode=overlap_mode)
        self.cfg = cfg
        self.L = lib()
        self.h = self.L.orc_create(C.byref(cfg))
        self.rMag = np.ascontiguousarray(rMag, dtype=np.float64)
        self.rHydr = np.ascontiguousarray(rHydr, dtype=np.float64)
        self.L.orc_set_props(self.h, _p(self.rMag), _p(self.rHydr), d["vis"] if vis is None else vis)

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    __del__ = close

    def set_state(self, pos, mm, ea, t=0.0, reset_observables=True):
        a = [np.ascontiguousarray(x, dtype=np.float64).reshape(3, self.n) for x in (pos, mm, ea)]
        self.L.orc_set_state(self.h, *(_p(x) for x in a), t)
        if reset_observables:
            self.L.orc_reset_observables(self.h)

    def get_state(self):
        a = [np.zeros((3, self.n)) for _ in range(3)]
        t = C.c_double()
        self.L.orc_get_state(self.h, *(_p(x) for x in a), C.byref(t))
        return a[0], a[1], a[2], t.value

    def set_thermal_force_zero(self):
        z = np.zeros((3, 3, self.n))
        self.L.orc_thermal(self.h, 1e-12, 0, None, 0, _p(z[0]), _p(z[1]), _p(z[2]))

    def compute_interactions(self):
        B, F, P = np.zeros((3, self.n)), np.zeros((3, self.n)), np.zeros(3)
        self.L.orc_compute_interactions(self.h, _p(B), _p(F), _p(P))
        return B, F, P

    def compute_field(self, mm):
        mm = np.ascontiguousarray(mm, dtype=np.float64)
        B = np.zeros((3, self.n))
        self.L.orc_compute_field(self.h, _p(mm), _p(B))
        return B

    def step(self, dt, noise_mode=0, xi=None, seed=0, dump=False):
        o = {}
        obs = np.zeros(8)
        if dump:
            o["B1"], o["F1"], o["B2"] = (np.zeros((3, self.n)) for _ in range(3))
        xi_p = None
        if xi is not None:
            xi = np.ascontiguousarray(xi, dtype=np.float64)
            xi_p = _p(xi)
        self.L.orc_step(self.h, dt, noise_mode, xi_p, seed, _p(o.get("B1")), _p(o.get("F1")), _p(o.get("B2")),
                        _p(obs))
        o["obs"] = obs
        return o

    def step_adaptive(self, solver, dt, absTol, dtMin, dtMax, noise_mode=0, xi=None, seed=0):
        """One accepted step with the reference's adaptive solver and time-step
        control; returns (next trial dt, dt used, attempts, obs)."""
        ad = Adapt(int(solver), float(absTol), float(dtMin), float(dtMax))
        dtv, used, att = C.c_double(dt), C.c_double(), C.c_int()
        obs = np.zeros(8)
        xi_p = None
        if xi is not None:
            xi = np.ascontiguousarray(xi, dtype=np.float64)
            xi_p = _p(xi)
        self.L.orc_step_adaptive(self.h, C.byref(ad), C.byref(dtv), noise_mode, xi_p, seed, _p(obs), C.byref(used),
                                 C.byref(att))
        return dtv.value, used.value, att.value, obs

    def set_threads(self, t):
        """Threads of the pair list and the Ewald sums (t > 1 needs overlap_mode 1)."""
        if self.L.orc_set_threads(self.h, int(t)) != 0:
            raise ValueError(f"orc_set_threads({t}) refused")

    def last_seconds(self):
        return self.L.orc_last_seconds(self.h)

    def pairs(self):
        return self.L.orc_pairs(self.h)


def philox_block(ctr, key):
    """One Philox4x32-10 block: four 32-bit counter words, two key words."""
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [int(v) for v in o]


def philox_normals(seed, step, n):
    xi = np.zeros((3, 3, n))
    lib().orc_philox_normals(seed, step, n, _p(xi))
    return xi


def noise_scales(d, rMag, rHydr, dt, vis):
    """sqrt scale factors of DefThermFluct (simulation.cpp:567, 582, 594) -> (3, N)."""
    pi = d["my_pi"]
    rMag, rHydr = np.asarray(rMag), np.asarray(rHydr)
    zr = 8.0 * pi * vis * rHydr ** 3.0
    zt = 6.0 * pi * vis * rHydr
    vm = 4.0 / 3.0 * pi * rMag ** 3.0
    kT2 = 2.0 * d["kB"] * d["temp"] / dt
    sT = np.sqrt(kT2 * zr)
    sB = np.sqrt(2.0 * d["kB"] * d["temp"] * d["magDamp"] / (d["gyroMr"] * d["satMag"] * dt) * (1.0 / vm))
    sF = np.sqrt(kT2 * zt)
    return sT, sB, sF


# ------------------------------------------------------- initial states


def random_state(n, lBox, rHydr, rng, min_gap=0.0, rot=2):
    """Seeded random-sequential-addition positions (no core or shell overlap,
    periodic distances, optional extra gap) and uniform orientations; the same
    construction as InitCoordsFromSketch (simulation.cpp:241-264, 304-337)
    with numpy's generator instead of EigenRand's."""
    pos = np.zeros((n, 3))
    rH = np.asarray(rHydr)
    for i in range(n):
        for _ in range(100000):
            x = rng.uniform(-1, 1, 3) * (lBox / 2.0 - rH[i])
            if i == 0:
                break
            d = pos[:i] - x
            d -= lBox * np.round(d / lBox)
            if np.all(np.sqrt((d * d).sum(1)) >= rH[i] + rH[:i] + min_gap):
                break
        else:
            raise RuntimeError("placement failed")
        pos[i] = x
    az = rng.uniform(0, 1, n) * 2 * math.pi
    el = 2.0 * np.arcsin(np.sqrt(rng.uniform(0, 1, n)))
    ea = np.stack([np.sin(el) * np.cos(az), np.sin(el) * np.sin(az), np.cos(el)])
    if rot == 2:
        mm = ea.copy()
    else:
        az2 = rng.uniform(0, 1, n) * 2 * math.pi
        el2 = 2.0 * np.arcsin(np.sqrt(rng.uniform(0, 1, n)))
        mm = np.stack([np.sin(el2) * np.cos(az2), np.sin(el2) * np.sin(az2), np.cos(el2)])
    return np.ascontiguousarray(pos.T), mm, ea


def rsa_fast(n, lBox, rHydr, seed, max_tries=100000):
    """(3, N) positions by random sequential addition in index order (the C
    restatement orc_rsa of InitCoordsFromSketch, simulation.cpp:241-264)."""
    rH = np.ascontiguousarray(rHydr, dtype=np.float64)
    pos = np.zeros((3, n))
    if lib().orc_rsa(n, lBox, _p(rH), int(seed), int(max_tries), _p(pos)) != 0:
        raise RuntimeError("random sequential addition failed: volume fraction too high")
    return pos


def rsa_philox(n, lBox, rHydr, seed, order=None, max_tries=2000000):
    """(3, N) positions and each particle's accepted attempt: random
    sequential addition with a Philox stream per particle (orc_rsa_philox, the
    restatement of the GPU placement md_place_rsa); order: placement order
    (None: index order, as the reference)."""
    rH = np.ascontiguousarray(rHydr, dtype=np.float64)
    pos = np.zeros((3, n))
    tries = np.zeros(n, dtype=np.int64)
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    st = lib().orc_rsa_philox(n, lBox, _p(rH), int(seed), None if o is None else o.ctypes.data_as(C.c_void_p),
                              int(max_tries), _p(pos), tries.ctypes.data_as(C.c_void_p))
    if st != 0:
        raise RuntimeError("random sequential addition failed: volume fraction too high")
    return pos, tries


def cost_model_rc(d, rMag, rHydr, lBox, kc_tc=25):
    """The Ewald split the library's cost model picks (restated for the CPU
    arm of the benchmark, which must not load the library): every rc = 0.08 L
    .. 0.5 L in steps of 0.005 L, alpha and kc from the reference's error
    model (ewald_for_rc), cost = N (9.5 n_pairs + c_k n_k) with c_k = 1.7 for
    kc <= kc_tc (tensor-core k space) else 2.5.  Returns (alpha, rc, kc)."""
    n = len(rMag)
    best = None
    for q in range(85):
        x = 0.08 + 0.005 * q
        try:
            a, kc, _ = ewald_for_rc(d, rMag, rHydr, lBox, x * lBox)
        except ValueError:
            continue
        if kc > 64:
            continue
        nr = n * 4.0 / 3.0 * math.pi * x ** 3
        nk = 2.0 * math.pi / 3.0 * kc ** 3
        cost = n * (9.5 * nr + (1.7 if kc <= kc_tc else 2.5) * nk)
        if best is None or cost < best[0]:
            best = (cost, a, x * lBox, kc)
    return best[1:]
