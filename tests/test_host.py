"""Host-side checks that need no GPU: the library loads and exports every
declared entry point, configuration handling matches the reference's
Configuration, the Ewald error model matches the reference's search."""
import ctypes as C
import math
import os
import tempfile

import numpy as np
import pytest

import oracle as O
import ref_io
from helpers import md_config


def test_library_loads_and_exports_every_symbol():
    import md_sim_wolfschwenger_gb300 as m
    L = m.lib()
    names = m.exported_symbols()
    assert len(names) >= 30
    for nm in names:
        assert hasattr(L, nm), nm
    assert L.md_config_size() == C.sizeof(m.MdConfig)
    assert b"sm_103a" in L.md_version()


def test_status_strings():
    import md_sim_wolfschwenger_gb300 as m
    L = m.lib()
    for s in range(8):
        assert L.md_strerror(s)
    assert L.md_strerror(99) == b"unknown status"


def test_ctx_create_rejects_bad_arguments():
    import md_sim_wolfschwenger_gb300 as m
    L = m.lib()
    cfg = m.Configuration.default()
    h = C.c_void_p()
    assert L.md_ctx_create(C.byref(cfg.c), 1, 1, C.byref(h)) == 1
    assert L.md_ctx_create(C.byref(cfg.c), 64, 7, C.byref(h)) == 1


@pytest.mark.parametrize("overrides", [{}, {"npDim": 5, "temp": 310.0, "magDamp": 0.05, "conc": 20},
                                       {"ENABLE_COATING_POT": "true", "SOLVER": 1}])
def test_ini_loader_matches_reference_derivations(overrides):
    ini = ref_io.ini_dict(**overrides)
    cfg = md_config(ini)
    d = O.derive(ini)
    c = cfg.c
    for key in ("magDamp", "temp", "satMag", "anisEn", "rMagMean", "dShell", "volFrac", "tMag", "deltaTinit",
                "magFluxDens", "errTolEwald", "my_pi", "kB", "gyroMr", "facEwald", "effLenSurfMol", "mu0",
                "velMmConst", "anisConst", "sterRepFac", "gamma", "epsilon", "kappa", "electrostatRepFac", "irPi",
                "vis", "sigma", "tEnd"):
        assert getattr(c, key) == pytest.approx(d[key], rel=1e-15, abs=0), key
    for key in ("INIT_CONFIG_ROT", "INIT_CONFIG_TRANS", "SIZE_DIST", "seed", "SOLVER", "npDim", "numbPart"):
        assert getattr(c, key) == d[key], key
    for key in ("ENABLE_MOBILIZATION", "ENABLE_THERM_FIELD", "ENABLE_THERM_TORQUE", "ENABLE_THERM_FORCE",
                "ENABLE_COATING_POT"):
        assert bool(getattr(c, key)) == d[key], key
    assert cfg.getNumbPart() == d["numbPart"]
    assert cfg.getVis() == c.vis


def test_ini_loader_semantics():
    """inih dialect: inline ';' comments, case-insensitive keys, missing keys
    default to -1/false, garbage numbers fall back to the default."""
    import md_sim_wolfschwenger_gb300 as m
    text = ("; comment\n[Particle_Properties]\nNPDIM = 3 ; three\nmagDamp: 0.2\ntemp = abc\n"
            "[gb300]\nNUMB_PART = 30\nvis = 1e-3\n")
    with tempfile.NamedTemporaryFile("w", suffix=".ini", delete=False) as f:
        f.write(text)
    try:
        cfg = m.Configuration.from_ini(f.name)
    finally:
        os.unlink(f.name)
    assert cfg.c.npDim == 3 and cfg.c.magDamp == 0.2 and cfg.c.temp == -1
    assert cfg.c.satMag == -1 and cfg.c.ENABLE_MOBILIZATION == 0
    assert cfg.numb_part() == 30 and cfg.c.visOverride == 1e-3


def test_missing_ini_is_an_error():
    import md_sim_wolfschwenger_gb300 as m
    with pytest.raises(m.MdError) as e:
        m.Configuration.from_ini("/nonexistent/configuration.ini")
    assert e.value.status == 5


def test_default_config_is_the_shipped_ini():
    """md_config_default equals the reference's shipped configuration.ini
    (checked against the file itself when the reference is mounted)."""
    import md_sim_wolfschwenger_gb300 as m
    import ref_io
    root = ref_io.reference_root()
    path = os.path.join(root, "src", "configuration.ini") if root else ""
    if not os.path.exists(path):
        pytest.skip("reference sources not mounted")
    a = m.Configuration.default().as_dict()
    b = m.Configuration.from_ini(path).as_dict()
    for k in a:
        if k in ("precision", "noise"):
            continue
        assert a[k] == b[k], k


@pytest.mark.parametrize("n,phi,rc_frac,lognormal", [(64, 0.05, 0.45, False), (512, 0.05, 0.3, False),
                                                      (4096, 0.1, 0.25, True), (512, 0.2, 0.4, True)])
def test_ewald_error_model_matches_reference_search(n, phi, rc_frac, lognormal):
    """alpha and kc of md_ewald_params_host against the reference's scan +
    interpolation (restated in the oracle, interaction.cpp:190-257)."""
    import md_sim_wolfschwenger_gb300 as m
    ini = ref_io.ini_dict(volFrac=phi, errTolEwald=1e-5)
    cfg = md_config(ini, vis=1e-3, n=n)
    d = O.derive(ini)
    rng = np.random.default_rng(n)
    rMag = 1e-8 * np.exp(0.2 * rng.standard_normal(n)) if lognormal else np.full(n, 1e-8)
    rHydr = rMag + 5e-9
    L = O.box_length(rHydr, phi, d["my_pi"])
    a_ref, kc_ref, kraw_ref = O.ewald_for_rc(d, rMag, rHydr, L, rc_frac * L)
    a, r, k, ef, et, lb = (C.c_double(), C.c_double(), C.c_int64(), C.c_double(), C.c_double(), C.c_double())
    P = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    st = m.lib().md_ewald_params_host(C.byref(cfg.c), n, P(rMag), P(rHydr), rc_frac * L, C.byref(a), C.byref(r),
                                      C.byref(k), C.byref(ef), C.byref(et), C.byref(lb))
    assert st == 0
    assert lb.value == pytest.approx(L, rel=1e-15)
    # the reference's grid step is 2e8/9999 in alpha; linear interpolation
    assert a.value == pytest.approx(a_ref, rel=2e-4)
    assert abs(k.value - kraw_ref) <= 0.5 + 1e-6
    # the chosen parameters meet the tolerance of the reference's model
    assert ef.value < 1.5e-5


def test_cost_model_cutoff_is_valid():
    import md_sim_wolfschwenger_gb300 as m
    n = 32768
    ini = ref_io.ini_dict(volFrac=0.1, errTolEwald=1e-5)
    cfg = md_config(ini, vis=1e-3, n=n)
    rng = np.random.default_rng(3)
    rMag = 1e-8 * np.exp(0.2 * rng.standard_normal(n))
    a, r, k, ef, et, lb = (C.c_double(), C.c_double(), C.c_int64(), C.c_double(), C.c_double(), C.c_double())
    P = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    assert m.lib().md_ewald_params_host(C.byref(cfg.c), n, P(rMag), None, -1.0, C.byref(a), C.byref(r), C.byref(k),
                                        C.byref(ef), C.byref(et), C.byref(lb)) == 0
    assert 0.08 * lb.value <= r.value <= 0.5 * lb.value
    assert 2 <= k.value <= 64
    assert ef.value < 2e-5 and math.isfinite(et.value)


def _init(n, seed, **kw):
    import md_sim_wolfschwenger_gb300 as m
    cfg = m.Configuration.default().set(numbPartOverride=n, **kw)
    return m.init_system(cfg, n, seed)


@pytest.mark.parametrize("kw", [dict(volFrac=0.05, rMagMean=1e-8),
                                dict(volFrac=0.2, SIZE_DIST=1, sigmaLog=0.25, rMagMean=1.25e-8),
                                dict(volFrac=0.1, SIZE_DIST=1, rMagMean=1e-8)])
def test_init_system_places_non_overlapping_spheres(kw):
    rMag, rHydr, pos, mm, ea, L = _init(3000, 5, **kw)
    c = kw["rMagMean"]
    if kw.get("SIZE_DIST"):
        assert rMag.std() > 0
    else:
        assert np.all(rMag == c)
    assert L == pytest.approx((np.sum(4 / 3 * 3.14159265359 * rHydr ** 3) / kw["volFrac"]) ** (1 / 3), rel=1e-12)
    # inside [-(L/2 - r_h), L/2 - r_h] and no overlap of hydrodynamic spheres
    assert np.all(np.abs(pos) <= L / 2 - rHydr[None, :] + 1e-20)
    from scipy.spatial import cKDTree
    t = cKDTree(pos.T)
    for i, j in t.query_pairs(2 * rHydr.max()):
        assert np.linalg.norm(pos[:, i] - pos[:, j]) >= rHydr[i] + rHydr[j]
    assert np.allclose((mm ** 2).sum(0), 1) and np.allclose((ea ** 2).sum(0), 1)


def test_init_system_orientations_and_grid():
    _, _, pos, mm, ea, L = _init(512, 3, volFrac=0.05, INIT_CONFIG_TRANS=2, INIT_CONFIG_ROT=1)
    xs = np.unique(np.round(pos[0] / L, 12))
    assert xs.size == 8 and np.allclose(np.diff(xs), 1 / 8)
    assert np.all(mm[2] == 1) and np.all(mm[:2] == 0)
    assert abs(ea[2].mean()) < 0.1 and abs((ea[2] ** 2).mean() - 1 / 3) < 0.05   # uniform on the sphere
    _, _, _, mm3, ea3, _ = _init(64, 3, volFrac=0.05, INIT_CONFIG_ROT=3)
    assert np.all(ea3[2] == 1) and np.array_equal(mm3, ea3)
    _, _, _, mm4, ea4, _ = _init(4000, 4, volFrac=0.05, INIT_CONFIG_ROT=4)
    assert abs(np.mean((mm4 * ea4).sum(0))) < 0.05   # independent directions
    a = _init(100, 9, volFrac=0.05)
    b = _init(100, 9, volFrac=0.05)
    assert all(np.array_equal(x, y) for x, y in zip(a[:5], b[:5]))


def test_init_system_reports_jammed_packing():
    import md_sim_wolfschwenger_gb300 as m
    with pytest.raises(m.MdError):
        _init(2000, 1, volFrac=0.6)


def test_tune_cache_file_round_trip(tmp_path):
    import md_sim_wolfschwenger_gb300 as m
    p = tmp_path / "t.txt"
    p.write_text("# header\n24 5 0.25\n26 10 0.3125\n")
    m.tune_cache_clear()
    m.tune_cache_load(p)
    q = tmp_path / "u.txt"
    m.tune_cache_save(q)
    assert q.read_text().splitlines()[1:] == ["24 5 0.25", "26 10 0.3125"]
    m.tune_cache_clear()


def test_tune_cache_file_round_trip(tmp_path):
    """The tuning cache file keeps, per (N, volume fraction) bucket, the
    cut-off and the k-space choices (engine, ring option, chunk waves); a line
    with the cut-off only (an older file) loads with default choices."""
    import md_sim_wolfschwenger_gb300 as m
    src = tmp_path / "in.txt"
    src.write_text("# header\n30 5 0.245 1 3 2\n28 10 0.3\n26 12 0.9 0 0 1\n")
    m.tune_cache_clear()
    m.tune_cache_load(src)
    out = tmp_path / "out.txt"
    m.tune_cache_save(out)
    m.tune_cache_clear()
    rows = [ln.split() for ln in out.read_text().splitlines() if not ln.startswith("#")]
    got = {(int(r[0]), int(r[1])): (float(r[2]), int(r[3]), int(r[4]), int(r[5])) for r in rows}
    assert got == {(30, 5): (0.245, 1, 3, 2), (28, 10): (0.3, 0, -1, 1)}  # rc > 0.5 L is refused


def test_step_io_hands_over_only_plain_arrays():
    """md_step_io receives the state arrays' addresses as they are: only
    C-contiguous float64 arrays of 3N values qualify (others are copied,
    or refused as outputs, by Simulation.step_io)."""
    from md_sim_wolfschwenger_gb300.simulation import _plain
    n3 = 3 * 10
    assert _plain(np.zeros((3, 10)), n3)
    assert _plain(np.zeros(n3), n3)
    assert not _plain(np.zeros((3, 10), dtype=np.float32), n3)
    assert not _plain(np.asfortranarray(np.zeros((3, 10))), n3)
    assert not _plain(np.zeros((3, 20))[:, ::2], n3)
    assert not _plain(np.zeros((3, 11)), n3)
    assert not _plain([0.0] * n3, n3)
