"""Packed stepping of independent systems and request serving over the C ABI
(md_batch_*, md_serve_run in include/md_gb300.h), plus host-side initial
systems (md_init_system).

`Batch` advances several `Simulation` objects (mixed precision, Philox or no
noise) with one launch per kernel for all of them; each system's results
equal those of `Simulation.step` on it alone.  `serve` runs a request stream
with continuous batching under a device-memory budget (the loop itself is
C++ inside the library)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import MdRequest, MdRequestResult, MdServeOpts, MdServeStats, check, lib
from .simulation import Configuration, Simulation

_P = lambda a: None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def init_system(config: Configuration, n: int, seed: int):
    """(rMag, rHydr, pos, mm, ea, lBox) of a new system (InitParticleProps +
    InitCoordsFromSketch with the configuration's keys)."""
    n = int(n)
    rMag, rHydr = np.empty(n), np.empty(n)
    pos, mm, ea = np.empty((3, n)), np.empty((3, n)), np.empty((3, n))
    L = C.c_double()
    check(lib().md_init_system(C.byref(config.c), n, int(seed), _P(rMag), _P(rHydr), _P(pos), _P(mm), _P(ea),
                               C.byref(L)))
    return rMag, rHydr, pos, mm, ea, L.value


def place_rsa(rHydr, lBox: float, seed: int, largest_first: bool = False):
    """(3, N) positions by random sequential addition on the GPU
    (md_place_rsa): index order as the reference (or largest radius first),
    a Philox stream per particle."""
    rH = np.ascontiguousarray(rHydr, dtype=np.float64)
    pos = np.empty((3, len(rH)))
    check(lib().md_place_rsa(len(rH), float(lBox), _P(rH), int(seed), int(bool(largest_first)), _P(pos)))
    return pos


def autotune_ewald_cached(sim: Simulation, volFrac: float):
    """Ewald parameters from the per-(N, volume fraction) tuning cache:
    (alpha, rc, kc, hit)."""
    a, r, k, h = C.c_double(), C.c_double(), C.c_int64(), C.c_int()
    check(lib().md_autotune_ewald_cached(sim.h, float(volFrac), C.byref(a), C.byref(r), C.byref(k), C.byref(h)),
          sim.h)
    sim.ewald = (a.value, r.value, k.value)
    return a.value, r.value, k.value, bool(h.value)


def tune_cache_save(path):
    check(lib().md_tune_cache_save(str(path).encode()))


def tune_cache_load(path):
    check(lib().md_tune_cache_load(str(path).encode()))


def tune_cache_clear():
    check(lib().md_tune_cache_clear())


class Batch:
    """Systems advanced together by packed launches (md_batch_*)."""

    def __init__(self, capacity: int):
        self.L = lib()
        h = C.c_void_p()
        check(self.L.md_batch_create(int(capacity), C.byref(h)))
        self.h = h
        self.members = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.md_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, sim: Simulation, nsteps: int, dt: float):
        i = C.c_int64()
        check(self.L.md_batch_add(self.h, sim.h, int(nsteps), float(dt), C.byref(i)))
        self.members[i.value] = sim
        return i.value

    def remove(self, sid: int):
        check(self.L.md_batch_remove(self.h, int(sid)))
        self.members.pop(sid, None)

    def run(self, max_steps: int):
        k = C.c_int64()
        check(self.L.md_batch_run(self.h, int(max_steps), C.byref(k)))
        return k.value

    def launch(self, max_steps: int):
        k = C.c_int64()
        check(self.L.md_batch_launch(self.h, int(max_steps), C.byref(k)))
        return k.value

    def wait(self):
        check(self.L.md_batch_wait(self.h))

    def remaining(self, sid: int):
        left, st = C.c_int64(), C.c_int()
        check(self.L.md_batch_remaining(self.h, int(sid), C.byref(left), C.byref(st)))
        return left.value, st.value

    def info(self):
        """(systems, particles, launches per packed step, GPU ms of the last round)."""
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        check(self.L.md_batch_info(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return a.value, b.value, c.value, d.value


def serve(config: Configuration, requests, hbm_budget=150e9, max_systems=256, round_steps=100, realtime=True,
          autotune=False):
    """Runs the request stream (dicts with n, volFrac, steps, dt, fieldKind,
    fieldAmp, fieldFreq, seed, arrival); returns (results, stats) as lists of
    dicts / a dict."""
    nreq = len(requests)
    arr = (MdRequest * max(nreq, 1))()
    for i, q in enumerate(requests):
        for k, _ in MdRequest._fields_:
            setattr(arr[i], k, q[k])
    res = (MdRequestResult * max(nreq, 1))()
    opts = MdServeOpts(float(hbm_budget), int(max_systems), int(round_steps), int(bool(realtime)),
                       int(bool(autotune)))
    st = MdServeStats()
    check(lib().md_serve_run(C.byref(config.c), arr, nreq, C.byref(opts), res, C.byref(st)))
    out = [{k: getattr(res[i], k) for k, _ in MdRequestResult._fields_} for i in range(nreq)]
    return out, {k: getattr(st, k) for k, _ in MdServeStats._fields_}
