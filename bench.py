"""Benchmark of the coupled LLG + Brownian-dynamics step on GB300.

Workload (one "step" = one Heun time step of the whole system): the single
large instance of the benchmark suite -- N = 32768 magnetite particles with
log-normal core diameters (median 20 nm, sigma 0.2), 5 nm shell, volume
fraction 0.10, static 20 mT field, dt = 1e-12 s, Philox thermal noise,
Ewald parameters for 1e-5 relative force error (timed autotune over the
error model), mixed precision.  Synthetic, seeded inputs (log-normal radii,
random sequential addition, uniform orientations).

Prints one JSON line (see the keys below).  `--impl reference` times the
reference's CPU algorithm (the C restatement in oracle/, single-threaded per
replica, all host threads as independent replicas) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from md_sim_wolfschwenger_gb300.workloads import WORKLOADS  # noqa: E402  (plain data, no library load)

W = dict(WORKLOADS["large"])

# Algorithmic FLOPs (FMA = 2) per unit of work, counted from the formulas.
FLOPS_PAIR_FULL = 113.0   # per unordered pair: erfc/exp terms, field on both, force, pressure
FLOPS_PAIR_FIELD = 58.0   # per unordered pair: field on both particles
FLOPS_KSF = 11.0          # per (k, particle): phase step (6), weight (1), two accumulations (4)
FLOPS_KSCAT_FULL = 21.0   # per (k, particle): phase step, field (6), force (9)
FLOPS_KSCAT_FIELD = 12.0  # per (k, particle): phase step, field


def tc_mma_flops(n, kc):
    """Executed tensor-core FLOPs (3 passes, padding included) per launch of
    the tensor-core structure factor (FP16 operands) and scatter (TF32
    operands) of md_ktc.cu for kc: the same row / tile shapes as
    kspace_tc_shape."""
    rows = sum(1 for nz in range(kc + 1) for ny in range(-kc, kc + 1)
               if ny * ny + nz * nz <= kc * kc and (nz > 0 or ny > 0)) + 1  # + the (0, 0) row (nx > 0)
    ns = (2 * (2 * kc + 1) + 15) // 16 * 16
    kp = (2 * (2 * kc + 1) + 7) // 8 * 8
    mt = (rows + 63) // 64
    npad = (n + 15) // 16 * 16
    sf = 3 * 2.0 * (mt * 128) * ns * (2 * npad)
    nb = (n + 127) // 128 * 128
    nt_full, nt_field = (rows + 19) // 20, (rows + 31) // 32
    return sf, 3 * 2.0 * nb * (nt_full * 128) * kp, 3 * 2.0 * nb * (nt_field * 128) * kp
BYTES_CELLS = 60.0        # per particle (+8 per cell)
BYTES_HEUN1 = 252.0       # per particle
BYTES_HEUN2 = 404.0       # per particle


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    p.add_argument("--workload", choices=sorted(WORKLOADS), default="large")
    p.add_argument("--n", type=int, default=0, help="override the workload's particle count")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true", help="skip the plain-FP64 comparison")
    p.add_argument("--sweep-replicas", type=int, default=256, help="field-sweep sample: replicas (0 skips it)")
    p.add_argument("--sweep-steps", type=int, default=1000, help="field-sweep sample: steps per replica")
    p.add_argument("--serve-requests", type=int, default=4096, help="served stream: requests (0 skips it)")
    p.add_argument("--serve-step-scale", type=float, default=0.02,
                   help="served-stream sample: factor on the drawn step counts (1e3..1e5 log-uniform)")
    p.add_argument("--stress-steps", type=int, default=20, help="stress-instance sample: steps (0 skips it)")
    p.add_argument("--autotune", type=int, default=0, help="candidate cutoffs timed (0: the cost-model choice, the same one the reference arm uses)")
    return p.parse_args()


def workload_config(n, seed):
    from md_sim_wolfschwenger_gb300 import workloads
    return workloads.config(dict(W, n=n), seed)


def workload_state(n, seed):
    """Initial system from the library's InitParticleProps + InitCoordsFromSketch
    (md_init_system: log-normal radii, random sequential addition placed
    largest first, moments and easy axes independent and uniform)."""
    from md_sim_wolfschwenger_gb300 import workloads
    return workloads.state(dict(W, n=n), seed)


def bench_config(n, ws):
    """The `config` object of the JSON line: the workload alone, identical in
    both arms (per-run quantities such as the box length and the Ewald split
    of the drawn system are reported under "system")."""
    return {"workload": W["desc"], "n": n, "replicas_per_gpu": 1,
            "parallelism": f"replicas x{ws}" if ws > 1 else "single instance",
            "l2": "GPU arm: L2 flushed between timed steps (256 MiB write), step time from CUDA events on the "
                  "library's stream; CPU arm: wall clock per step"}


def oracle_ini(n, seed):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_io
    return ref_io.ini_dict(volFrac=W["phi"], magFluxDens=W["B0"], tMag=1.0, seed=seed)


# ------------------------------------------------------------ clocks


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.02)
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# -------------------------------------------------------------- dist


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(v, ws):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------- cpu arms


def cpu_baseline_port(n, sysd, ewald, seed, threads=1, steps=1):
    """The oracle's restatement of the reference step (all-pairs list,
    sequential overlap push, FP64) timed on host cores; `threads` independent
    replicas run concurrently (ctypes releases the GIL)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    rMag, rHydr, L, pos, mm, ea = sysd
    alpha, rc, kc = ewald
    d = O.derive(oracle_ini(n, seed))
    d["vis"] = 1e-3
    d["ENABLE_THERM_TORQUE"] = d["ENABLE_THERM_FIELD"] = d["ENABLE_THERM_FORCE"] = True
    d["magDamp"], d["satMag"], d["anisEn"] = 0.1, 4.8e5, 1.1e4
    reps = []
    for t in range(threads):
        o = O.Oracle(d, rMag, rHydr, L, alpha, rc, kc, vis=1e-3, overlap_mode=0)
        o.set_state(pos, mm, ea)
        reps.append(o)
    times = []
    for s in range(steps):
        ths = [threading.Thread(target=r.step, args=(1e-12, 2, None, seed + i)) for i, r in enumerate(reps)]
        t0 = time.perf_counter()
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        times.append(time.perf_counter() - t0)
    per = [r.last_seconds() for r in reps]
    for r in reps:
        r.close()
    return times, per


def run_reference(args):
    """The reference's algorithm on the host cores: the C restatement of its
    step (oracle/md_oracle.c: all-pairs list, FP64 real- and k-space Ewald
    sums in the reference's loops, Heun step), one instance of the workload
    with the pair list and Ewald sums spread over every host thread.  The
    system (seeded log-normal radii, random sequential addition in index
    order, uniform orientations) and the Ewald split (the library's cost
    model over the reference's error model, restated in oracle.py) come from
    oracle code only: this arm loads nothing of the CUDA library."""
    rank, ws, _ = dist_init()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    n, seed = args.n, 1
    rng = np.random.default_rng(1000 + seed)
    rMag = W["median"] * np.exp(W["sigma"] * rng.standard_normal(n)) if W["sigma"] > 0 else np.full(n, W["median"])
    rHydr = rMag + 5e-9
    d = O.derive(oracle_ini(n, seed))
    d["vis"] = 1e-3
    d["ENABLE_THERM_TORQUE"] = d["ENABLE_THERM_FIELD"] = d["ENABLE_THERM_FORCE"] = True
    d["magDamp"], d["satMag"], d["anisEn"] = 0.1, 4.8e5, 1.1e4
    L = O.box_length(rHydr, W["phi"], d["my_pi"])
    t0 = time.perf_counter()
    pos = O.rsa_fast(n, L, rHydr, 7 + seed)
    mm = rng.standard_normal((3, n))
    mm /= np.linalg.norm(mm, axis=0)
    ea = rng.standard_normal((3, n))
    ea /= np.linalg.norm(ea, axis=0)
    alpha, rc, kc = O.cost_model_rc(d, rMag, rHydr, L)
    setup_s = time.perf_counter() - t0
    threads = max(1, os.cpu_count() or 1)
    o = O.Oracle(d, rMag, rHydr, L, alpha, rc, kc, vis=1e-3, overlap_mode=1)
    o.set_threads(threads)
    o.set_state(pos, mm, ea)
    for _ in range(args.warmup):
        o.step(1e-12, 2, None, seed)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(1e-12, 2, None, seed)
    total = time.perf_counter() - t0
    pairs = o.pairs()
    o.close()
    value = n * args.steps / total
    sample = (f"{args.steps} timed steps (+{args.warmup} warm-up) of one N={n} instance, the pair list and the Ewald "
              f"sums spread over {threads} host threads; all-pairs list and FP64 Ewald in the reference's loops")
    line = {"impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded log-normal radii, random sequential addition, moments and easy axes "
                    "independent and uniform on the sphere)",
            "config": bench_config(n, ws),
            "system": {"lBox_m": L, "ewald": {"alpha_L": alpha * L, "rc_over_L": rc / L, "kc": kc, "pairs": pairs},
                       "setup_s": setup_s},
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------ secondary workloads


def _pct(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    lo, hi = int(math.floor(k)), int(math.ceil(k))
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


def contact_scales(cfg, rMag, rHydr):
    """Contact force, field and torque of the smallest particles
    (CompEwaldParams / CheckEwaldSum, src/interaction.cpp:180-181, 743-753):
    the scales of the reference's relative error."""
    mu0, pi, ms = cfg.c.mu0, cfg.c.my_pi, cfg.c.satMag
    mmin = float(np.min(ms * 4.0 / 3.0 * pi * np.asarray(rMag) ** 3))
    rh = float(np.min(rHydr))
    return (3 * mu0 * mmin ** 2 / (2 * pi * (2 * rh) ** 4), mu0 * mmin / (2 * pi * (2 * rh) ** 3),
            mmin ** 2 * mu0 / (16 * pi * rh ** 3))


def rms_rel(a, b, scale):
    d = np.asarray(a) - np.asarray(b)
    return math.sqrt(float((d * d).sum()) / d.shape[-1]) / scale


def fp64_plain(n, sysd, ewald, seed, steps=4, warm=1):
    """The same system and Ewald parameters on the plain FP64 path
    (MD_PREC_FP64, one instance): particle-steps/s from CUDA events on the
    library's stream; and the mixed path's error against it on the initial
    state (CompInteractions: field, force, torque mu x B; contact-normalised
    RMS over particles, the reference's error metric)."""
    import torch
    from md_sim_wolfschwenger_gb300 import MD_NOISE_PHILOX, MD_PREC_FP64, MD_PREC_MIXED, Simulation
    from md_sim_wolfschwenger_gb300 import workloads
    rMag, rHydr, L, pos, mm, ea = sysd
    cfg = workload_config(n, seed)
    err, _ = workloads.mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, ewald)
    err["metric"] = ("RMS over particles of |mixed - fp64| / contact value (CheckEwaldSum's metric); the "
                     "Ewald truncation budget is 1e-5")
    sim = Simulation(cfg, n, MD_PREC_FP64, rMag=rMag, rHydr=rHydr)
    sim.set_state(pos, mm, ea)
    sim.set_ewald(*ewald)
    sim.set_noise(MD_NOISE_PHILOX, seed)
    sim.step(warm, 1e-12)
    sim.sync()
    ext = torch.cuda.ExternalStream(sim.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(ext):
        e0.record()
    sim.step(steps, 1e-12)
    with torch.cuda.stream(ext):
        e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    sim.close()
    return {"value": n / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms, "steps": steps,
            "dtype": "f64", "note": "same system and Ewald parameters, plain FP64 path, one instance",
            "mixed_error_vs_fp64": err}


def segment_rooflines(seg_mean, n, kc, pairs, nk_real, tensor_cores, peak_fp32, hbm_peak):
    """Per-segment achieved rates of a profiled pass (ms per kernel segment):
    algorithmic FLOPs or bytes per unit (the constants above) over the
    segment's time, against the FP32 FMA-chain peak, the HBM copy peak or the
    measured tensor rate; returns the segments and their work table."""
    work = {"real_full": ("fp32", pairs * FLOPS_PAIR_FULL), "real_field": ("fp32", pairs * FLOPS_PAIR_FIELD),
            "ksf_full": ("fp32", nk_real * n * FLOPS_KSF), "ksf_field": ("fp32", nk_real * n * FLOPS_KSF),
            "kscat_full": ("fp32", nk_real * n * FLOPS_KSCAT_FULL),
            "kscat_field": ("fp32", nk_real * n * FLOPS_KSCAT_FIELD),
            "cells": ("hbm", n * BYTES_CELLS), "heun1": ("hbm", n * BYTES_HEUN1), "heun2": ("hbm", n * BYTES_HEUN2)}
    peak_tf32 = peak_f16 = None
    if tensor_cores:
        # the tensor-core k space: the structure factor's executed 3-pass FP16
        # MMA work against the measured bf16 rate (the same rate), the
        # scatter's 3-pass TF32 work against half of it (nominal 1:2)
        sf_fl, scf_fl, scd_fl = tc_mma_flops(n, kc)
        work.update(ksf_full=("tensor16", sf_fl), ksf_field=("tensor16", sf_fl), kscat_full=("tensor", scf_fl),
                    kscat_field=("tensor", scd_fl))
        try:
            peak_f16 = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"]
        except Exception:
            peak_f16 = 1900.0
        peak_tf32 = peak_f16 / 2
    segs = {}
    for k, ms in seg_mean.items():
        ent = {"ms": ms}
        if k in work and ms > 0:
            kind, amount = work[k]
            if kind == "fp32":
                ach = amount / (ms * 1e-3) / 1e12
                ent.update(bound="fp32", achieved=ach, unit="TFLOP/s", peak=peak_fp32, frac=ach / peak_fp32)
            elif kind == "tensor":
                ach = amount / (ms * 1e-3) / 1e12
                ent.update(bound="tensor", achieved=ach, unit="TFLOP/s", peak=peak_tf32, frac=ach / peak_tf32,
                           note="3-pass TF32 MMAs executed (padding included); peak = measured bf16 / 2")
            elif kind == "tensor16":
                ach = amount / (ms * 1e-3) / 1e12
                ent.update(bound="tensor", achieved=ach, unit="TFLOP/s", peak=peak_f16, frac=ach / peak_f16,
                           note="3-pass FP16 MMAs executed (padding included); peak = measured bf16 (same rate)")
            else:
                ach = amount / (ms * 1e-3) / 1e9
                ent.update(bound="hbm", achieved=ach, unit="GB/s", peak=hbm_peak,
                           frac=(ach / hbm_peak) if hbm_peak else None)
        segs[k] = ent
    return segs, work


def stress_sample(steps, peak_fp32, hbm_peak, warm=3, fp64_steps=2, seed=1):
    """The stress instance (N = 131072, log-normal sigma 0.25, volume fraction
    0.20, 30 mT): mixed particle-steps/s from CUDA events around `steps`
    graph replays, the plain FP64 path on the same system and Ewald
    parameters, and the mixed path's error against it (B, F, torque)."""
    import torch
    from md_sim_wolfschwenger_gb300 import MD_NOISE_PHILOX, MD_PREC_FP64, MD_PREC_MIXED, Simulation, workloads
    w = workloads.spec("stress")
    n = w["n"]
    cfg = workloads.config(w, seed)
    rMag, rHydr, L, pos, mm, ea = workloads.state(w, seed)
    out = {}
    for prec, k in ((MD_PREC_MIXED, steps), (MD_PREC_FP64, fp64_steps)):
        sim = Simulation(cfg, n, prec, rMag=rMag, rHydr=rHydr)
        sim.set_state(pos, mm, ea)
        if prec == MD_PREC_MIXED:
            alpha, rc, kc, errF, errT = sim.ewald_params()
        sim.set_ewald(alpha, rc, kc)
        sim.set_noise(MD_NOISE_PHILOX, seed)
        sim.step(warm if prec == MD_PREC_MIXED else 1, 1e-12)
        sim.sync()
        ext = torch.cuda.ExternalStream(sim.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            e0.record()
        sim.step(k, 1e-12)
        with torch.cuda.stream(ext):
            e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / k
        extra = {}
        if prec == MD_PREC_MIXED:
            extra = {"pairs": sim.pairs(), "strong_pair_entries_fp64": sim.strong_pairs(),
                     "kspace_tensor_cores": sim.kspace_tensor_cores()}
            # per-kernel segments: a profiled pass (kernels one after another)
            sim.profile(True)
            sim.step(1, 1e-12)
            acc = None
            for _ in range(3):
                sim.step(1, 1e-12)
                sg = sim.profile_read()
                acc = sg if acc is None else {a: acc[a] + b for a, b in sg.items()}
            sim.profile(False)
            seg_mean = {a: b / 3 for a, b in acc.items()}
            segs, _ = segment_rooflines(seg_mean, n, kc, extra["pairs"], len(sim.debug_structure_factor()),
                                        sim.kspace_tensor_cores(), peak_fp32, hbm_peak)
            kspace = [q for q in seg_mean if q.startswith("k")]
            extra_segs = {"segments": segs,
                          "kspace_share_of_serialised_step": sum(seg_mean[q] for q in kspace) / sum(seg_mean.values()),
                          "fp64_accumulation_ms": seg_mean.get("kred_full", 0.0) + seg_mean.get("kred_field", 0.0),
                          "fp64_accumulation_note": "the structure factor's exact chunk sums (TwoSum FP32 pairs, "
                                                    "then FP64), S and e S in FP64 and the scatter operand image: "
                                                    "the reduction segments, ms per step"}
        sim.close()
        out[prec] = (ms, k, extra)
        if prec == MD_PREC_MIXED:
            out["segs"] = extra_segs
    err, _ = workloads.mixed_vs_fp64(cfg, rMag, rHydr, pos, mm, ea, (alpha, rc, kc))
    ms, k, extra = out[MD_PREC_MIXED]
    ms64, k64, _ = out[MD_PREC_FP64]
    return {"value": n / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms, "steps": k,
            "workload": w["desc"], "n": n, "lBox_m": L,
            "ewald": {"alpha_L": alpha * L, "rc_over_L": rc / L, "kc": kc, "pred_force_err_rel_contact": errF,
                      "pred_torque_err_rel_contact": errT, **extra},
            "fp64_plain": {"value": n / (ms64 * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms64,
                           "steps": k64},
            "mixed_over_fp64_plain": ms64 / ms,
            "mixed_error_vs_fp64": err,
            **out["segs"],
            "note": "graph replays back to back (no L2 flush; the working set exceeds the 129 MB L2); torque "
                    "error is the FP32 k-space floor for a moment ratio of ~700 (below the parameters' own "
                    "Ewald truncation error pred_torque_err_rel_contact)"}


def sweep_sample(replicas, steps, seed=3):
    """Field sweep (magnetisation curve): `replicas` independent systems with
    N uniform in 256..8192, monodisperse 20/30 nm, volume fraction 0.05,
    static fields evenly spaced 0..50 mT, advanced together by packed
    launches (md_batch_*); `steps` steps each (the full sweep runs 5e4)."""
    import md_sim_wolfschwenger_gb300 as m
    rng = np.random.default_rng(seed)
    ns = rng.integers(256, 8193, replicas)
    fields = np.linspace(0.0, 0.05, replicas)
    t0 = time.perf_counter()
    sims = []
    for i, (n, b0) in enumerate(zip(ns, fields)):
        cfg = m.Configuration.default().set(numbPartOverride=int(n), volFrac=0.05, rMagMean=1e-8, dShell=5e-9,
                                            visOverride=1e-3, INIT_CONFIG_ROT=4, SIZE_DIST=0, magFluxDens=float(b0),
                                            tMag=1.0, errTolEwald=1e-5)
        rMag, rHydr, pos, mm, ea, L = m.init_system(cfg, int(n), 100 + i)
        sim = m.Simulation(cfg, int(n), m.MD_PREC_MIXED, rMag=rMag)
        a, r, k, _, _ = sim.ewald_params()
        sim.set_ewald(a, r, k)
        sim.set_state(pos, mm, ea)
        sim.set_noise(m.MD_NOISE_PHILOX, 100 + i)
        sims.append(sim)
    setup_s = time.perf_counter() - t0
    b = m.Batch(replicas)
    for sim in sims:
        b.add(sim, steps + 2, 1e-12)
    b.run(2)  # warm-up: graph capture and first launches
    gpu_ms, t0 = 0.0, time.perf_counter()
    left = steps
    while left > 0:
        k = b.run(left)
        gpu_ms += b.info()[3]
        left -= k
    wall = time.perf_counter() - t0
    _, parts, lps, _ = b.info()
    mz = [float(sim.records()[-1, 1]) for sim in sims]
    b.close()
    for sim in sims:
        sim.close()
    total = float(ns.sum()) * steps
    return {"value": total / wall, "unit": "particle-steps/s", "gpu_value": total / (gpu_ms * 1e-3),
            "replicas": replicas, "particles": int(ns.sum()), "steps": steps, "launches_per_step": lps,
            "setup_s": setup_s,
            "mz_at_0_25_50_mT": [mz[0], mz[len(mz) // 2], mz[-1]],
            "sample": f"{replicas} replicas, N uniform 256..8192 (seeded), monodisperse 20/30 nm, volume fraction "
                      f"0.05, static fields 0..50 mT, {steps} steps each (the full sweep runs 5e4), one packed "
                      f"launch per kernel per step for all replicas under a captured CUDA graph"}


def serve_stream(nreq, step_scale, seed=4):
    """Requests of the served stream: Poisson arrivals at 200/s; N log-uniform
    in 128..16384; volume fraction uniform in 0.02..0.15; steps log-uniform in
    1e3..1e5 (times step_scale); sinusoidal field, amplitude uniform in
    10..30 mT, frequency uniform in 10..100 kHz."""
    rng = np.random.default_rng(seed)
    arr = np.cumsum(rng.exponential(1.0 / 200.0, nreq))
    out = []
    for i in range(nreq):
        n = int(round(math.exp(rng.uniform(math.log(128), math.log(16384)))))
        phi = float(rng.uniform(0.02, 0.15))
        st = max(1, int(round(math.exp(rng.uniform(math.log(1e3), math.log(1e5))) * step_scale)))
        amp, freq = float(rng.uniform(0.01, 0.03)), float(rng.uniform(1e4, 1e5))
        out.append(dict(n=n, volFrac=phi, steps=st, dt=1e-12, fieldKind=1, fieldAmp=amp, fieldFreq=freq,
                        seed=5000 + i, arrival=float(arr[i])))
    return out


def serve_base_config():
    import md_sim_wolfschwenger_gb300 as m
    return m.Configuration.default().set(rMagMean=1e-8, dShell=5e-9, visOverride=1e-3, INIT_CONFIG_ROT=4,
                                         SIZE_DIST=0, errTolEwald=1e-5)


def serve_sample(nreq, step_scale, plain_sample=8):
    """The served stream through md_serve_run (continuous batching under a
    150 GB device-memory budget, real-time arrivals), and the plain FP64
    single-instance path timed on a seeded subsample of the same requests
    (each alone, back to back) for the ratio."""
    import md_sim_wolfschwenger_gb300 as m
    reqs = serve_stream(nreq, step_scale)
    cfg = serve_base_config()
    res, st = m.serve(cfg, reqs, hbm_budget=150e9, max_systems=256, round_steps=100, realtime=True)
    ok = [r for r in res if r["status"] == 0]
    lat = [r["latency"] for r in ok]
    value = st["particle_steps"] / st["wall"]
    # plain FP64 single instance on a subsample of the same requests
    rng = np.random.default_rng(11)
    idx = sorted(rng.choice(nreq, size=min(plain_sample, nreq), replace=False).tolist())
    ps, secs = 0.0, 0.0
    for i in idx:
        q = reqs[i]
        c = serve_base_config().set(numbPartOverride=q["n"], volFrac=q["volFrac"], seed=q["seed"], fieldKind=1,
                                    fieldAmp=q["fieldAmp"], fieldFreq=q["fieldFreq"])
        rMag, rHydr, pos, mm, ea, L = m.init_system(c, q["n"], q["seed"])
        sim = m.Simulation(c, q["n"], m.MD_PREC_FP64, rMag=rMag)
        a, r, k, _, _ = sim.ewald_params()
        sim.set_ewald(a, r, k)
        sim.set_state(pos, mm, ea)
        sim.set_noise(m.MD_NOISE_PHILOX, q["seed"])
        sim.step(1, 1e-12)
        sim.sync()
        k = max(2, min(q["steps"], 6))
        t0 = time.perf_counter()
        sim.step(k, 1e-12)
        sim.sync()
        secs += time.perf_counter() - t0
        ps += q["n"] * k
        sim.close()
    plain = ps / secs if secs > 0 else None
    return {"value": value, "unit": "particle-steps/s", "requests": nreq, "completed": len(ok),
            "p50_latency_s": _pct(lat, 0.5), "p99_latency_s": _pct(lat, 0.99), "wall_s": st["wall"],
            "gpu_ms": st["gpu_ms"], "admit_ms": st["admit_ms"], "rounds": st["rounds"],
            "peak_systems": st["peak_systems"], "peak_bytes": st["peak_bytes"],
            "plain_fp64_single_instance": {"value": plain, "unit": "particle-steps/s",
                                           "sample": f"{len(idx)} requests of the stream, each alone on the "
                                                     f"FP64 path (MD_PREC_FP64), a few steps each"},
            "vs_plain_fp64": (value / plain) if plain else None,
            "sample": f"{'all' if nreq >= 4096 else 'first'} {nreq} requests of the stream (Poisson 200/s; N log-uniform 128..16384; volume "
                      f"fraction 0.02..0.15; steps log-uniform 1e3..1e5 scaled by {step_scale}; sinusoidal "
                      f"field 10..30 mT, 10..100 kHz); 150 GB budget, realtime admission, mixed precision"}


# ----------------------------------------------------------- our arm


def run_ours(args):
    rank, ws, local = dist_init()
    import torch
    from md_sim_wolfschwenger_gb300 import (MD_NOISE_PHILOX, MD_PREC_FP64, MD_PREC_MIXED, Simulation,
                                            calibrate_fp32, select_device)
    select_device(local)
    torch.cuda.set_device(local)
    n = args.n
    prec = MD_PREC_FP64 if args.precision == "fp64" else MD_PREC_MIXED
    seed = 1 + rank
    cfg = workload_config(n, seed)
    rMag, rHydr, L, pos, mm, ea = sysd = workload_state(n, seed)
    sim = Simulation(cfg, n, prec, rMag=rMag, rHydr=rHydr)
    sim.set_state(pos, mm, ea)
    if args.autotune > 0:
        alpha, rc, kc, _ = sim.autotune_ewald(args.autotune)
    else:
        alpha, rc, kc, _, _ = sim.ewald_params()
        sim.set_ewald(alpha, rc, kc)
    _, _, _, errF, errT = sim.ewald_params(rc)
    sim.set_noise(MD_NOISE_PHILOX, seed)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sim.step(args.warmup, 1e-12)
    sim.sync()
    launches_per_step = sim.launches() // max(1, args.warmup)
    ext = torch.cuda.ExternalStream(sim.stream())
    clocks = ClockSampler(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    # timed steps: the production graph (real- and k-space branches
    # concurrent), CUDA events on the library's stream around each step,
    # L2 flushed before each
    evs = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            e0.record()
        sim.step(1, 1e-12)
        with torch.cuda.stream(ext):
            e1.record()
        evs.append((e0, e1))
    torch.cuda.synchronize()
    barrier(ws)
    total_ms = sum(a.elapsed_time(b) for a, b in evs)
    total_ms = allmax(total_ms, ws)
    value = ws * n * args.steps / (total_ms * 1e-3)

    # continuous run (graph replays back to back, no flush) for reference
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(ext):
        e0.record()
    sim.step(args.steps, 1e-12)
    with torch.cuda.stream(ext):
        e1.record()
    torch.cuda.synchronize()
    cont_ms = e0.elapsed_time(e1) / args.steps

    # per-kernel durations: a profiled pass, kernels one after another with
    # CUDA events between them (inside the replayed graph), L2 flushed per step
    sim.profile(True)
    sim.step(1, 1e-12)
    seg_sum, psteps = None, max(5, min(args.steps, 50))
    for _ in range(psteps):
        flush.zero_()
        torch.cuda.synchronize()
        sim.step(1, 1e-12)
        seg = sim.profile_read()
        seg_sum = seg if seg_sum is None else {k: seg_sum[k] + v for k, v in seg.items()}
    sim.profile(False)
    seg_mean = {k: v / psteps for k, v in seg_sum.items()}
    serial_ms = sum(seg_mean.values())
    pairs = sim.pairs()
    strong = sim.strong_pairs()
    ring, waves, chunk = sim.kspace_tiling()
    kspace = {"tensor_cores": bool(sim.kspace_tensor_cores()), "sf_ring_option": ring, "sf_chunk_waves": waves,
              "sf_chunk_particles": chunk, "chosen_by": "autotuner" if args.autotune > 0 else "defaults"}
    nk_real = len(sim.debug_structure_factor())
    clk = clocks.stop()  # sampled over both timed runs

    # end to end through the C ABI with pinned host buffers, copies timed:
    # each step the state goes in from host memory and comes back
    # (md_step_io: upload, step, download, one synchronisation)
    host_in = [torch.empty((3, n), dtype=torch.float64).pin_memory().numpy() for _ in range(3)]
    host_out = [torch.empty((3, n), dtype=torch.float64).pin_memory().numpy() for _ in range(3)]
    st = sim.get_state(out=host_in)
    ksteps = max(3, min(args.steps, 10))
    e2e_s = 0.0
    for _ in range(ksteps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.step_io(host_in, 1, 1e-12, out=host_out)
        e2e_s += time.perf_counter() - t0
        for a_, b_ in zip(host_in, host_out):
            a_[...] = b_
    e2e_s = allmax(e2e_s, ws)
    e2e = {"value": ws * n * ksteps / e2e_s, "unit": "particle-steps/s", "h2d_bytes_per_step": 3 * 24 * n,
           "d2h_bytes_per_step": 3 * 24 * n, "steps": ksteps}
    del st

    # roofline of every segment; the dominant one is reported
    peak_fp32 = calibrate_fp32()
    hbm_peak = None
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except Exception:
        pass
    segs, work = segment_rooflines(seg_mean, n, kc, pairs, nk_real, sim.kspace_tensor_cores(), peak_fp32, hbm_peak)
    dom = max((k for k in segs if k in work), key=lambda k: segs[k]["ms"])
    traffic = None  # from the ncu capture of this workload, when there is one
    try:
        for ln in open(os.path.join(ROOT, "profiles", "traffic.txt")):
            f = ln.split()
            if len(f) == 4 and not ln.startswith("#") and f[0] == args.workload and int(f[1]) == n and f[2] == dom:
                traffic = float(f[3])
    except (OSError, ValueError):
        pass
    d = segs[dom]
    roofline = {"kernel": dom, "bound": d["bound"], "achieved": d["achieved"], "peak": d["peak"], "unit": d["unit"],
                "frac": d["frac"], "traffic": traffic,
                "peak_source": ("measured FP32 FMA-chain kernel in this process (MEASURED_PEAKS.json has no FP32 "
                                "figure; this kernel class is FP32/SFU-issue bound, not HBM or tensor)"
                                if d["bound"] == "fp32" else "MEASURED_PEAKS.json hbm_gbs")}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        times, per = cpu_baseline_port(n, sysd, (alpha, rc, kc), seed, threads=1, steps=1)
        cpu = {"value": n / per[0], "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": f"1 step of the same N={n} system and Ewald parameters, single thread (the reference "
                         f"is single-threaded): all-pairs list, FP64, Philox noise; {per[0]:.1f} s"}

    fp64 = sweep = serving = stress = None
    if rank == 0 and ws == 1:
        if not args.no_fp64:
            fp64 = fp64_plain(n, sysd, (alpha, rc, kc), seed)
        if args.stress_steps > 0 and args.workload == "large":
            stress = stress_sample(args.stress_steps, peak_fp32, hbm_peak)
        if args.sweep_replicas > 0:
            sweep = sweep_sample(args.sweep_replicas, args.sweep_steps)
        if args.serve_requests > 0:
            serving = serve_sample(args.serve_requests, args.serve_step_scale)

    if rank == 0:
        line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if prec == MD_PREC_FP64 else "f32",
                "precision": ("fp64 (plain)" if prec == MD_PREC_FP64 else
                              "mixed: FP32 pair maths, phases, scatter and integrator; real-space pairs above 3 "
                              "contact forces (strong pairs) in FP64; structure-factor chunk partials summed "
                              "exactly (TwoSum FP32 pairs, then FP64), S(n) and e(n)S(n) in FP64; FP64 self/"
                              "surface terms, positions, reductions"),
                "data": "synthetic (seeded log-normal radii, random sequential addition, moments and easy axes "
                        "independent and uniform on the sphere)",
                "config": bench_config(n, ws),
                "system": {"lBox_m": L,
                           "ewald": {"alpha_L": alpha * L, "rc_over_L": rc / L, "kc": kc,
                                     "pred_force_err_rel_contact": errF, "pred_torque_err_rel_contact": errT,
                                     "pairs": pairs, "k_vectors": nk_real,
                                     "strong_pair_entries_fp64": strong},
                           "kspace": kspace},
                "e2e": e2e, "roofline": roofline, "segments": segs,
                "continuous": {"ms_per_step": cont_ms, "value": ws * n / (cont_ms * 1e-3),
                               "note": "graph replays back to back without L2 flush"},
                "serialized": {"ms_per_step": serial_ms, "steps": psteps,
                               "note": "the profiled pass: the same kernels one after another (no branch "
                                       "concurrency), the sum of the segments; per-kernel figures come from it"},
                "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches_per_step * args.steps,
                "fp64_plain": fp64, "mixed_over_fp64_plain": (value / fp64["value"]) if fp64 else None,
                "sweep": sweep, "serving": serving, "stress": stress}
        print(json.dumps(line), flush=True)
    sim.close()


def main():
    args = parse()
    W.clear()
    W.update(WORKLOADS[args.workload])
    if args.n > 0 and args.n != W["n"]:
        W["desc"] = W["desc"].replace(f"N={W['n']}", f"N={args.n}")
        W["n"] = args.n
    args.n = W["n"]
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
