"""Packed stepping and serving.  A system's results in a packed batch (one
launch per kernel for all systems) do not depend on what else is packed with
it: alone or in a mix, bit for bit.  Against the single-system kernels of
md_step, whose compiled FP32 arithmetic may round differently (FMA
contraction), packed results agree within FP32 rounding: tolerances below.
The request loop admits against its memory budget and its results do not
depend on the mix either."""
import numpy as np
import pytest

import md_sim_wolfschwenger_gb300 as m

pytestmark = pytest.mark.gpu


def _system(n, seed, phi=0.05, field=0.02, kind=m.MD_FIELD_STEP, freq=0.0, lognormal=False, rc=None):
    kw = dict(numbPartOverride=n, volFrac=phi, rMagMean=1e-8, dShell=5e-9, visOverride=1e-3, INIT_CONFIG_ROT=4,
              SIZE_DIST=1 if lognormal else 0, sigmaLog=0.2 if lognormal else 0.0, fieldKind=kind)
    if kind == m.MD_FIELD_SIN:
        kw.update(fieldAmp=field, fieldFreq=freq)
    else:
        kw.update(magFluxDens=field, tMag=1.0)
    cfg = m.Configuration.default().set(**kw)
    rMag, rHydr, pos, mm, ea, L = m.init_system(cfg, n, seed)
    sim = m.Simulation(cfg, n, m.MD_PREC_MIXED, rMag=rMag)
    a, r, k, _, _ = sim.ewald_params(None if rc is None else rc * sim.lBox)  # rc: box fraction
    sim.set_ewald(a, r, k)
    sim.set_state(pos, mm, ea)
    sim.set_noise(m.MD_NOISE_PHILOX, 1000 + seed)
    return sim


SPECS = [  # n, seed, phi, field, kind, freq, lognormal, rc (None: error model)
    (256, 1, 0.05, 0.00, m.MD_FIELD_STEP, 0.0, False, None),
    (700, 2, 0.10, 0.02, m.MD_FIELD_SIN, 5e4, True, None),
    (1500, 3, 0.05, 0.05, m.MD_FIELD_STEP, 0.0, False, None),
    (3000, 4, 0.15, 0.01, m.MD_FIELD_SIN, 2e4, False, None),
    (2048, 5, 0.05, 0.03, m.MD_FIELD_STEP, 0.0, True, 0.45),
]


# md_step vs packed after a few dozen steps: moment directions (unit
# vectors) within a few FP32 ulps growing with the steps, positions (box
# units) within FP32 rounding of the displacements, records likewise.
TOL_M, TOL_POS, TOL_REC = 2e-6, 1e-10, 2e-6


def _run_alone(spec, steps, dt, packed=True):
    """The system stepped by itself: in a batch of one (packed kernels) or by md_step."""
    sim = _system(*spec)
    if packed:
        b = m.Batch(1)
        b.add(sim, steps, dt)
        while b.run(11):
            pass
    else:
        sim.step(steps, dt)
    out = sim.get_state(), sim.records()
    sim.close()
    return out


def test_packed_equals_alone_bit_for_bit():
    dt = 1e-12
    steps = [30, 12, 30, 21, 5]  # uneven: systems leave the batch mid-way (re-packs)
    alone = [_run_alone(s, k, dt) for s, k in zip(SPECS, steps)]
    sims = [_system(*s) for s in SPECS]
    b = m.Batch(8)
    ids = [b.add(sm, k, dt) for sm, k in zip(sims, steps)]
    rounds = 0
    while True:
        k = b.run(7)
        if k == 0:
            break
        rounds += 1
        for sid, sm in zip(ids, sims):
            if sid in b.members and b.remaining(sid)[0] == 0:
                b.remove(sid)
    assert rounds >= 5
    for sm, (st, rec), k in zip(sims, alone, steps):
        p, mm, ea = sm.get_state()
        assert np.array_equal(p, st[0]) and np.array_equal(mm, st[1]) and np.array_equal(ea, st[2])
        r = sm.records()
        assert r.shape == (k, 8)
        assert np.array_equal(r, rec)


def test_packed_matches_single_system_kernels():
    dt = 1e-12
    for spec in SPECS:
        (p0, m0, e0), r0 = _run_alone(spec, 25, dt, packed=False)
        (p1, m1, e1), r1 = _run_alone(spec, 25, dt, packed=True)
        sim = _system(*spec)
        L = sim.lBox
        d = np.abs(p1 - p0)
        d = np.minimum(d, L - d)
        assert d.max() / L < TOL_POS
        assert np.abs(m1 - m0).max() < TOL_M and np.abs(e1 - e0).max() < TOL_M
        assert np.abs(r1[:, 1] - r0[:, 1]).max() < TOL_REC


def test_batch_info_and_launch_count():
    sims = [_system(*s) for s in SPECS[:3]]
    b = m.Batch(4)
    for sm in sims:
        b.add(sm, 5, 1e-12)
    assert b.run(5) == 5
    nsys, npart, lps, ms = b.info()
    assert nsys == 3 and npart == sum(s[0] for s in SPECS[:3])
    # one launch per kernel for all systems: at most 28 with both k-space
    # engines in the batch (CUDA-core and tensor-core systems)
    assert 10 <= lps <= 28
    assert ms > 0


def test_batch_grows_overflowing_neighbour_list():
    sims = [_system(*s) for s in SPECS[:2]]
    ref = _run_alone(SPECS[1], 6, 1e-12)  # the list fits: list-order sums
    sims[1].neighbor_capacity(cap=50)  # the next build overflows: direct scan, then growth
    b = m.Batch(2)
    for sm in sims:
        b.add(sm, 6, 1e-12)
    b.run(3)
    assert sims[1].neighbor_capacity() > 50
    b.run(3)
    p, mm, ea = sims[1].get_state()
    L = sims[1].lBox
    # the overflow step summed in cell-scan order: FP32 rounding differs
    assert np.abs(p - ref[0][0]).max() / L < TOL_POS and np.abs(mm - ref[0][1]).max() < TOL_M


def test_batch_rejects_unsupported_systems():
    sim = _system(256, 9)
    fp = m.Simulation(sim.config, 256, m.MD_PREC_FP64, rMag=np.full(256, 1e-8))
    b = m.Batch(1)
    with pytest.raises(m.MdError):
        b.add(fp, 3, 1e-12)          # no state / FP64
    b.add(sim, 3, 1e-12)
    with pytest.raises(m.MdError):
        b.add(_system(256, 10), 3, 1e-12)   # capacity 1


def _requests(k, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        out.append(dict(n=int(rng.integers(128, 2500)), volFrac=float(rng.uniform(0.02, 0.15)),
                        steps=int(rng.integers(10, 60)), dt=1e-12, fieldKind=m.MD_FIELD_SIN,
                        fieldAmp=float(rng.uniform(0.01, 0.03)), fieldFreq=float(rng.uniform(1e4, 1e5)),
                        seed=100 + i, arrival=0.002 * i))
    return out


def test_serve_results_same_alone_and_in_mix():
    cfg = m.Configuration.default().set(rMagMean=1e-8, dShell=5e-9, visOverride=1e-3, INIT_CONFIG_ROT=4)
    reqs = _requests(8)
    res, st = m.serve(cfg, reqs, hbm_budget=40e9, max_systems=16, round_steps=16, realtime=True)
    assert all(r["status"] == 0 for r in res)
    assert st["peak_systems"] >= 2 and st["rounds"] >= 3
    assert st["particle_steps"] == sum(q["n"] * q["steps"] for q in reqs)
    for q, r in zip(reqs, res):
        assert r["steps_done"] == q["steps"]
        assert r["latency"] >= 0 and r["finished"] >= r["admitted"] >= 0
    for i in (0, 3, 7):
        solo, _ = m.serve(cfg, [dict(reqs[i], arrival=0.0)], hbm_budget=40e9, max_systems=1, round_steps=5,
                          realtime=False)
        assert solo[0]["checksum"] == res[i]["checksum"]
        assert solo[0]["mz"] == res[i]["mz"]


def test_serve_respects_memory_budget():
    cfg = m.Configuration.default().set(rMagMean=1e-8, dShell=5e-9, visOverride=1e-3)
    reqs = _requests(6, seed=1)
    for q in reqs:
        q["arrival"] = 0.0
    res, st = m.serve(cfg, reqs, hbm_budget=40e9, max_systems=16, round_steps=8, realtime=False)
    assert all(r["status"] == 0 for r in res)
    held = [r["device_bytes"] for r in res]
    assert st["peak_bytes"] <= 40e9
    # a budget below what all six hold together: admission must hold some back
    budget = max(1.05 * max(held), 0.5 * sum(held))
    assert budget < sum(held)
    res2, st2 = m.serve(cfg, reqs, hbm_budget=budget, max_systems=16, round_steps=8, realtime=False)
    assert all(r["status"] == 0 for r in res2)
    assert st2["peak_bytes"] <= budget
    assert [r["checksum"] for r in res2] == [r["checksum"] for r in res]


def test_serve_reports_oversized_request():
    cfg = m.Configuration.default().set(rMagMean=1e-8, dShell=5e-9, visOverride=1e-3)
    reqs = _requests(2, seed=2)
    reqs[0]["n"] = 100000
    res, _ = m.serve(cfg, reqs, hbm_budget=30e6, max_systems=4, round_steps=8, realtime=False)
    assert res[0]["status"] == 3 and res[1]["status"] == 0


def test_autotune_cache_hit_for_same_bucket(tmp_path):
    m.tune_cache_clear()
    a = _system(1024, 21)
    r1 = m.autotune_ewald_cached(a, 0.05)
    assert not r1[3]
    b = _system(1100, 22)
    r2 = m.autotune_ewald_cached(b, 0.05)
    assert r2[3]
    assert abs(r2[1] / b.lBox - r1[1] / a.lBox) < 1e-12
    p = tmp_path / "tune.txt"
    m.tune_cache_save(p)
    m.tune_cache_clear()
    m.tune_cache_load(p)
    assert m.autotune_ewald_cached(_system(1050, 23), 0.05)[3]


def test_autotune_single_candidate_is_the_cost_model_choice():
    """With one candidate the autotuner times only the cost model's split
    and keeps it: the same (alpha, rc, kc) as md_ewald_params."""
    a = _system(2048, 31, phi=0.08, lognormal=True)
    al, rc, kc, _, _ = a.ewald_params()
    ta, trc, tkc, ms = a.autotune_ewald(1)
    assert (ta, trc, tkc) == (al, rc, kc) and ms > 0
