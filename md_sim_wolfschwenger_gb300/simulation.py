"""Python mirror of the reference's entry points over the C ABI.

`Configuration` mirrors the reference's Configuration singleton
(src/configuration.h:12-180 of MD_Sim_Wolfschwenger): the same INI keys and
getter names.  `Simulation` holds one particle system on the GPU and exposes
the reference's step functions by their names (CompInteractions,
CompDemagField, ...) on top of libmd_gb300.so.  Arrays are (3, N) float64
C-contiguous, i.e. the column-major N x 3 layout of the reference's Eigen
arrays (x block, y block, z block).
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

from ._lib import (MD_NOISE_OFF, MD_NOISE_PHILOX, MD_NOISE_UPLOADED, MD_PREC_FP64, MD_PREC_MIXED, MdConfig,
                   check, lib)

_P = lambda a: None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _plain(x, size):
    """A C-contiguous float64 ndarray of `size` values (its address can be
    handed to the library as it is)."""
    return type(x) is np.ndarray and x.dtype == np.float64 and x.flags.c_contiguous and x.size == size


def _getter_map():
    # getter name -> field (src/configuration.h:98-175)
    m = {"getNumbPart": "numbPart", "getInitConfigRot": "INIT_CONFIG_ROT",
         "getInitConfigTrans": "INIT_CONFIG_TRANS", "getReadFromFile": "READ_FROM_FILE",
         "getSizeDist": "SIZE_DIST", "getEnableMobilization": "ENABLE_MOBILIZATION",
         "getEnableThermField": "ENABLE_THERM_FIELD", "getEnableThermTorque": "ENABLE_THERM_TORQUE",
         "getEnableThermForce": "ENABLE_THERM_FORCE", "getSeed": "seed",
         "getEnableCoatingPot": "ENABLE_COATING_POT", "getSolver": "SOLVER", "getDeltaTInit": "deltaTinit",
         "getDeltaTMin": "deltaTmin", "getDeltaTMax": "deltaTmax", "getNPCoords": "npCoords",
         "getZValency": "z_valency", "getEpsilonR": "epsilon_r", "getGamma0": "gamma_0", "getKB": "kB",
         "getEpsilon0": "epsilon_0", "getMu0": "mu0", "getMyPi": "my_pi", "getIrPi": "irPi",
         "getTEnd": "tEnd", "getTMag": "tMag", "getTRelax": "tRelax"}
    for f, _ in MdConfig._fields_:
        m.setdefault("get" + f[0].upper() + f[1:], f)
    return m


_GETTERS = _getter_map()


class Configuration:
    """configuration.ini keys + derived constants (Configuration, src/configuration.cpp:6-93)."""

    def __init__(self, cfg: MdConfig | None = None):
        self.c = cfg if cfg is not None else MdConfig()
        if cfg is None:
            check(lib().md_config_default(C.byref(self.c)))

    @classmethod
    def from_ini(cls, path):
        c = MdConfig()
        check(lib().md_config_load_ini(str(path).encode(), C.byref(c)))
        return cls(c)

    @classmethod
    def default(cls):
        return cls()

    def set(self, **kw):
        """Sets fields (INI key names) and recomputes the derived constants."""
        for k, v in kw.items():
            if not hasattr(self.c, k):
                raise KeyError(k)
            setattr(self.c, k, v)
        check(lib().md_config_derive(C.byref(self.c)))
        return self

    def numb_part(self):
        return lib().md_config_numb_part(C.byref(self.c))

    def __getattr__(self, name):
        if name.startswith("get") and name in _GETTERS:
            f = _GETTERS[name]
            return lambda: getattr(self.c, f)
        raise AttributeError(name)

    def as_dict(self):
        return self.c.as_dict()


def select_device(device: int):
    """Current CUDA device of the library's runtime for the calling thread."""
    check(lib().md_select_device(int(device)))


def calibrate_fp32():
    """Measured FP32 FMA throughput of the current device in TFLOP/s."""
    v = C.c_double()
    check(lib().md_calibrate_fp32(C.byref(v)))
    return v.value


class Simulation:
    """One simulation instance on the GPU (the reference's WorkingVar_S and
    its step functions).  precision: MD_PREC_MIXED (default) or MD_PREC_FP64."""

    def __init__(self, config: Configuration, n: int | None = None, precision: int = MD_PREC_MIXED,
                 rMag=None, rHydr=None):
        self.L = lib()
        self.config = config
        self.n = int(n if n is not None else config.numb_part())
        self.precision = precision
        h = C.c_void_p()
        check(self.L.md_ctx_create(C.byref(config.c), self.n, precision, C.byref(h)))
        self.h = h
        if rMag is not None:
            self.set_particles(rMag, rHydr)

    def close(self):
        if getattr(self, "h", None):
            self.L.md_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        check(st, self.h)

    # ------------------------------------------------------------ setup
    def set_particles(self, rMag, rHydr=None):
        """InitParticleProps with given radii; returns the box length."""
        self._rMag = np.ascontiguousarray(rMag, dtype=np.float64)
        self._rHydr = None if rHydr is None else np.ascontiguousarray(rHydr, dtype=np.float64)
        self._ck(self.L.md_set_particles(self.h, _P(self._rMag), _P(self._rHydr)))
        return self.lBox

    @property
    def lBox(self):
        v = C.c_double()
        self._ck(self.L.md_get_box(self.h, C.byref(v)))
        return v.value

    def set_box(self, lBox):
        self._ck(self.L.md_set_box(self.h, lBox))

    def set_state(self, pos, mm, ea, reset=True):
        a = [np.ascontiguousarray(x, dtype=np.float64).reshape(3, self.n) for x in (pos, mm, ea)]
        self._ck(self.L.md_state_upload(self.h, *(_P(x) for x in a), int(reset)))

    def get_state(self, out=None):
        """(pos, mm, ea); `out` may be three (3, N) float64 arrays to fill."""
        a = out if out is not None else [np.empty((3, self.n)) for _ in range(3)]
        self._ck(self.L.md_state_download(self.h, *(_P(x) for x in a)))
        return tuple(a)

    def checkpoint_save(self, path):
        """Binary snapshot of the state (see md_checkpoint_save)."""
        self._ck(self.L.md_checkpoint_save(self.h, os.fsencode(str(path))))

    def checkpoint_load(self, path):
        """Restores a snapshot into this context (same N and precision)."""
        self._ck(self.L.md_checkpoint_load(self.h, os.fsencode(str(path))))

    def set_time(self, t, step=0):
        self._ck(self.L.md_set_time(self.h, t, step))

    def get_time(self):
        t, s = C.c_double(), C.c_int64()
        self._ck(self.L.md_get_time(self.h, C.byref(t), C.byref(s)))
        return t.value, s.value

    # ------------------------------------------------------------- Ewald
    def ewald_params(self, rc=None):
        """CompEwaldParams error model: (alpha, rc, kc, errF, errT)."""
        a, r, k, ef, et = C.c_double(), C.c_double(), C.c_int64(), C.c_double(), C.c_double()
        self._ck(self.L.md_ewald_params(self.h, -1.0 if rc is None else float(rc), C.byref(a), C.byref(r),
                                        C.byref(k), C.byref(ef), C.byref(et)))
        return a.value, r.value, k.value, ef.value, et.value

    def set_ewald(self, alpha, rc, kc):
        """InitEwaldConst with the given parameters."""
        self._ck(self.L.md_set_ewald(self.h, float(alpha), float(rc), int(kc)))
        self.ewald = (float(alpha), float(rc), int(kc))

    def set_kspace_engine(self, engine):
        """Reciprocal-space engine of the mixed path: "auto", "simt" or "tc"."""
        code = {"auto": 0, "simt": 1, "tc": 2}[engine]
        self._ck(self.L.md_set_kspace_engine(self.h, code))

    def set_kspace_tiling(self, ring=-1, waves=1):
        """Tensor-core structure factor tiling: ring option (-1: deepest that
        fits) and the chunk-count multiple (1..4)."""
        self._ck(self.L.md_set_kspace_tiling(self.h, int(ring), int(waves)))

    def kspace_tiling(self):
        """(ring, waves, particles per structure-factor chunk)."""
        r, w, ch = C.c_int(), C.c_int(), C.c_int()
        self._ck(self.L.md_get_kspace_tiling(self.h, C.byref(r), C.byref(w), C.byref(ch)))
        return r.value, w.value, ch.value

    def kspace_tensor_cores(self):
        """True when the current Ewald parameters run the k space on the tensor cores."""
        v = C.c_int()
        self._ck(self.L.md_kspace_engine_active(self.h, C.byref(v)))
        return bool(v.value)

    def autotune_ewald(self, ncand=5):
        a, r, k, ms = C.c_double(), C.c_double(), C.c_int64(), C.c_double()
        self._ck(self.L.md_autotune_ewald(self.h, ncand, C.byref(a), C.byref(r), C.byref(k), C.byref(ms)))
        self.ewald = (a.value, r.value, k.value)
        return a.value, r.value, k.value, ms.value

    # ------------------------------------------------------ interactions
    def CompInteractions(self):
        """EvalSinCos + CompInteractions: (B [T], F [N] without thermal force, P3)."""
        B, F, P = np.empty((3, self.n)), np.empty((3, self.n)), np.empty(3)
        self._ck(self.L.md_compute_interactions(self.h, _P(B), _P(F), _P(P)))
        return B, F, P

    def CompDemagField(self, mm):
        """CompDemagField for the given moment directions."""
        mm = np.ascontiguousarray(mm, dtype=np.float64).reshape(3, self.n)
        B = np.empty((3, self.n))
        self._ck(self.L.md_compute_field(self.h, _P(mm), _P(B)))
        return B

    # ---------------------------------------------------------- stepping
    def set_noise(self, mode, seed=None):
        self._ck(self.L.md_set_noise(self.h, int(mode), int(self.config.c.seed if seed is None else seed)))

    def step(self, nsteps=1, dt=None, xi=None):
        """nsteps of the RunSimulation loop body with a fixed dt."""
        dt = float(self.config.c.deltaTinit if dt is None else dt)
        xp = None
        if xi is not None:
            xi = np.ascontiguousarray(xi, dtype=np.float64)
            if xi.size != 9 * self.n * nsteps:
                raise ValueError("xi must hold 9N normals per step")
            xp = _P(xi)
        self._ck(self.L.md_step(self.h, int(nsteps), dt, xp))

    def step_io(self, state, nsteps=1, dt=None, out=None):
        """State (pos, mm, ea) in, nsteps of step(), state out, in one call
        and one synchronisation (md_step_io); `out` may be three (3, N)
        float64 arrays to fill.  Pinned host arrays copy fastest."""
        dt = float(self.config.c.deltaTinit if dt is None else dt)
        n3 = 3 * self.n
        a = [x if _plain(x, n3) else np.ascontiguousarray(x, dtype=np.float64).reshape(3, self.n) for x in state]
        if out is None:
            o = [np.empty((3, self.n)) for _ in range(3)]
        else:
            o = out
            if not all(_plain(x, n3) for x in o):
                raise ValueError("out must be three C-contiguous float64 arrays of 3N values")
        self._ck(self.L.md_step_io(self.h, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data, int(nsteps), dt,
                                   o[0].ctypes.data, o[1].ctypes.data, o[2].ctypes.data))
        return tuple(o)

    def step_adaptive(self, max_steps, dt, t_end=float("inf"), xi=None):
        """Accepted steps of RunSimulation's loop with the configuration's
        SOLVER (0 Heun-Euler, 1 Bogacki-Shampine, 2 Dormand-Prince) and the
        reference's step control, while t <= t_end; returns (next trial dt,
        steps done)."""
        d = C.c_double(float(dt))
        k = C.c_int64()
        xp = None
        if xi is not None:
            xi = np.ascontiguousarray(xi, dtype=np.float64)
            if xi.size != 9 * self.n * max_steps:
                raise ValueError("xi must hold 9N normals per step")
            xp = _P(xi)
        self._ck(self.L.md_step_adaptive(self.h, int(max_steps), float(t_end), C.byref(d), xp, C.byref(k)))
        return d.value, k.value

    def records(self, first=0, count=None):
        """Per-step {t, mz, MSDx, MSDy, MSDz, Pxy, Pxz, Pyz} rows."""
        n = C.c_int64()
        self._ck(self.L.md_num_records(self.h, C.byref(n)))
        count = n.value - first if count is None else count
        out = np.empty((count, 8))
        self._ck(self.L.md_records(self.h, first, count, _P(out)))
        return out

    def clear_records(self):
        self._ck(self.L.md_clear_records(self.h))

    def sync(self):
        self._ck(self.L.md_sync(self.h))

    # -------------------------------------------------------- test hooks
    def debug_cells(self):
        nc, ncx = C.c_int64(), C.c_int64()
        self._ck(self.L.md_debug_cells(self.h, C.byref(nc), C.byref(ncx), None, None))
        cs = np.empty(nc.value + 1, dtype=np.int32)
        perm = np.empty(self.n, dtype=np.int32)
        self._ck(self.L.md_debug_cells(self.h, C.byref(nc), C.byref(ncx), cs.ctypes.data_as(C.POINTER(C.c_int32)),
                                       perm.ctypes.data_as(C.POINTER(C.c_int32))))
        return ncx.value, cs, perm

    def debug_structure_factor(self):
        nk = C.c_int64(0)
        self._ck(self.L.md_debug_structure_factor(self.h, C.byref(nk), None))
        out = np.empty((nk.value, 5))
        self._ck(self.L.md_debug_structure_factor(self.h, C.byref(nk), _P(out)))
        return out

    def rdf(self, bins=500, range_mag=8.0, r_mag0=None, include_last=False):
        """g(r) of the current frame on the device (mFiles/radial_dist_fun.m):
        returns (x in units of 2 r_mag0 at the bin centres, g, counts)."""
        r0 = float(self._rMag[0] if r_mag0 is None else r_mag0)
        g = np.empty(int(bins))
        cnt = np.empty(int(bins), dtype=np.uint64)
        self._ck(self.L.md_rdf(self.h, int(bins), range_mag * r0, r0, int(bool(include_last)), _P(g),
                               cnt.ctypes.data_as(C.POINTER(C.c_uint64))))
        x = (np.arange(bins) + 0.5) * (range_mag * r0 / bins) / (2 * r0)
        return x, g, cnt

    def debug_real_part(self):
        """Real-space (B, F) alone of the last CompInteractions, (3, N) SI."""
        B, F = np.empty((3, self.n)), np.empty((3, self.n))
        self._ck(self.L.md_debug_real_part(self.h, _P(B), _P(F)))
        return B, F

    def launches(self):
        v = C.c_int64()
        self._ck(self.L.md_debug_launches(self.h, C.byref(v)))
        return v.value

    def pairs(self):
        """In-range pairs (unordered) of the last full real-space evaluation."""
        v = C.c_int64()
        self._ck(self.L.md_debug_pairs(self.h, C.byref(v)))
        return v.value

    def set_neighbor_skin(self, skin_frac):
        """Skin of the real-space neighbour list as a fraction of rc."""
        self._ck(self.L.md_set_neighbor_skin(self.h, float(skin_frac)))

    def set_strong_pairs(self, theta):
        """Mixed path: pairs above theta contact forces of the smallest
        particles ((|mu_i||mu_j|/mu_min^2)(2 rHydr_min/r)^4) are evaluated in
        FP64 (default 3; 0 turns it off)."""
        self._ck(self.L.md_set_strong_pairs(self.h, float(theta)))

    def strong_pairs(self):
        """Entries of the strong-pair list of the last build (0: off, -1: not in use)."""
        v = C.c_int64()
        self._ck(self.L.md_debug_strong_pairs(self.h, C.byref(v)))
        return v.value

    def neighbor_capacity(self, cap=0):
        """Entries of the last neighbour list; cap > 0 caps the capacity (test hook)."""
        used = C.c_int64()
        self._ck(self.L.md_debug_neighbor_capacity(self.h, int(cap), C.byref(used)))
        return used.value

    def profile(self, enable=True):
        self._ck(self.L.md_profile(self.h, int(enable)))

    def profile_read(self):
        """Milliseconds per kernel segment of the last step."""
        from ._lib import SEGMENTS
        ms = np.zeros(len(SEGMENTS))
        self._ck(self.L.md_profile_read(self.h, _P(ms)))
        return dict(zip(SEGMENTS, ms))

    def device_bytes(self):
        v = C.c_int64()
        self._ck(self.L.md_ctx_device_bytes(self.h, C.byref(v)))
        return v.value

    def stream(self):
        v = C.c_void_p()
        self._ck(self.L.md_ctx_stream(self.h, C.byref(v)))
        return v.value
