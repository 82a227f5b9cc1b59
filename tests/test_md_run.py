"""The drop-in executable md_run (InitSimulation + RunSimulation of the
reference, src/simulation.cpp:24-537, with the step on the GPU): command line
and errors on CPU; on the GPU, the output files it writes equal those written
from the same system stepped through the Python API, byte for byte, with the
fixed step and with the adaptive solvers."""
import os
import subprocess

import numpy as np
import pytest

import ref_io
from helpers import ROOT

EXE = os.path.join(ROOT, "md_sim_wolfschwenger_gb300", "_lib", "md_run")


def _run(args, cwd, timeout=600):
    return subprocess.run([EXE] + args, cwd=cwd, capture_output=True, text=True, timeout=timeout)


def test_help_and_bad_arguments(tmp_path):
    r = _run(["--help"], tmp_path)
    assert r.returncode == 0 and "usage: md_run" in r.stdout
    r = _run(["--bogus"], tmp_path)
    assert r.returncode == 2 and "unknown option" in r.stderr
    r = _run(["--precision", "half"], tmp_path)
    assert r.returncode == 2


def test_missing_configuration_is_reported(tmp_path):
    run = tmp_path / "run"
    run.mkdir()
    r = _run([], run)  # ../configuration.ini does not exist
    assert r.returncode == 1 and "md_config_load_ini" in r.stderr


def _frames(path):
    """coords.txt frames (lists of rows) and their time labels."""
    frames, cur = [], []
    for line in open(path):
        vals = line.split()
        if not vals:
            if cur:
                frames.append(np.array(cur, dtype=float))
            cur = []
            continue
        cur.append([float(v) for v in vals])
    if cur:
        frames.append(np.array(cur, dtype=float))
    return frames


@pytest.mark.gpu
def test_outputs_equal_python_api_run(tmp_path):
    import md_sim_wolfschwenger_gb300 as m
    from md_sim_wolfschwenger_gb300 import outputs
    ini = ref_io.ini_dict(npDim=4, tMag=1e-10, tRelax=5e-11, deltaTinit=1e-12, magFluxDens=0.02, seed=7,
                          INIT_CONFIG_ROT=2, volFrac=0.05)
    ini["output_settings"]["npCoords"] = 10
    ref_io.write_ini(tmp_path / "configuration.ini", ini)
    run = tmp_path / "run"
    run.mkdir()
    r = _run(["--precision", "mixed", "--chunk", "37", "--quiet", "--fixed-dt"], run)
    assert r.returncode == 0, r.stderr
    assert "simulation ended successfully" in r.stdout
    names = sorted(os.listdir(run))
    assert names == sorted(["data.txt", "coords.txt", "dtMean.txt", "Pxy.txt", "Pxz.txt", "Pyz.txt", "MSDx.txt",
                            "MSDy.txt", "MSDz.txt", "mz.txt", "t.txt"])

    # the same run through the Python API
    cfg = m.Configuration.from_ini(tmp_path / "configuration.ini")
    n = cfg.numb_part()
    rMag, rHydr, pos, mm, ea, L = m.init_system(cfg, n, 7)
    sim = m.Simulation(cfg, n, m.MD_PREC_MIXED, rMag=rMag, rHydr=rHydr)
    sim.set_state(pos, mm, ea)
    a, rc, kc, _, _ = sim.ewald_params()
    sim.set_ewald(a, rc, kc)
    sim.set_noise(m.MD_NOISE_PHILOX, 7)
    t, steps, nframes = 0.0, 0, 0
    while t <= cfg.c.tEnd:  # RunSimulation's loop and frame test, src/simulation.cpp:466-494
        if np.floor(t / cfg.c.tEnd * cfg.c.npCoords) == nframes:
            nframes += 1
        t += cfg.c.deltaTinit
        steps += 1
    sim.step(steps, cfg.c.deltaTinit)
    rec = sim.records()
    p, mm2, ea2 = sim.get_state()
    sim.close()
    ref = tmp_path / "api"
    ref.mkdir()
    outputs.export_records(str(ref), rec, t, steps)
    outputs.write_data(ref / "data.txt", cfg, rMag, rHydr, L)
    for nm in ("dtMean.txt", "Pxy.txt", "Pxz.txt", "Pyz.txt", "MSDx.txt", "MSDy.txt", "MSDz.txt", "mz.txt", "t.txt",
               "data.txt"):
        assert (run / nm).read_bytes() == (ref / nm).read_bytes(), nm
    # coords: the loop's frames plus the final one; the last equals the API's final state
    fr = _frames(run / "coords.txt")
    assert nframes >= 10 and len(fr) == nframes + 1 and all(f.shape == (n, 10) for f in fr)
    assert fr[0][0, 9] == 0.0 and fr[-1][0, 9] == float(f"{t:g}")
    outputs.write_coords(ref / "final.txt", p, mm2, ea2, 0.0)
    last = _frames(ref / "final.txt")[0]
    np.testing.assert_array_equal(fr[-1][:, :9], last[:, :9])
    assert len(np.loadtxt(run / "mz.txt")) == steps


@pytest.mark.gpu
@pytest.mark.parametrize("solver", [0, 2])
def test_adaptive_outputs_equal_python_api_run(tmp_path, solver):
    import md_sim_wolfschwenger_gb300 as m
    from md_sim_wolfschwenger_gb300 import outputs
    ini = ref_io.ini_dict(npDim=4, tMag=2e-11, tRelax=1e-11, deltaTinit=1e-12, magFluxDens=0.02, seed=9,
                          SOLVER=solver, absTol=1e-4, volFrac=0.05)
    ini["output_settings"]["npCoords"] = 5
    ref_io.write_ini(tmp_path / "configuration.ini", ini)
    run = tmp_path / "run"
    run.mkdir()
    r = _run(["--precision", "fp64", "--quiet"], run)
    assert r.returncode == 0, r.stderr
    cfg = m.Configuration.from_ini(tmp_path / "configuration.ini")
    n = cfg.numb_part()
    rMag, rHydr, pos, mm, ea, L = m.init_system(cfg, n, 9)
    sim = m.Simulation(cfg, n, m.MD_PREC_FP64, rMag=rMag, rHydr=rHydr)
    sim.set_state(pos, mm, ea)
    a, rc, kc, _, _ = sim.ewald_params()
    sim.set_ewald(a, rc, kc)
    sim.set_noise(m.MD_NOISE_PHILOX, 9)
    _, steps = sim.step_adaptive(100000, cfg.c.deltaTinit, t_end=cfg.c.tEnd)
    rec = sim.records()
    t_end = sim.get_time()[0]
    sim.close()
    assert steps >= 3 and len(np.atleast_1d(np.loadtxt(run / "t.txt"))) == steps
    ref = tmp_path / "api"
    ref.mkdir()
    outputs.export_records(str(ref), rec, t_end, steps)
    for nm in ("dtMean.txt", "Pxy.txt", "MSDx.txt", "MSDz.txt", "mz.txt", "t.txt"):
        assert (run / nm).read_bytes() == (ref / nm).read_bytes(), nm
    assert np.all(np.diff(rec[:, 0]) > 0)


def _ckpt_state(path, n):
    raw = np.fromfile(path, dtype=np.uint8)
    assert bytes(raw[:8]) == b"MDCKPT01"
    vals = raw[8 + 6 * 8 + 4 * 8:].view(np.float64)
    return vals[2 * n:2 * n + 9 * n].reshape(3, 3, n), raw[8:8 + 48].view(np.int64)


@pytest.mark.gpu
def test_resume_from_checkpoint_continues_the_run(tmp_path):
    # no applied field: the field program (on while t < tMag) would differ
    # between the two configurations, which end at different times
    ini = ref_io.ini_dict(npDim=4, tMag=6e-11, tRelax=0.0, deltaTinit=1e-12, magFluxDens=0.0, seed=3,
                          volFrac=0.05)
    ini["output_settings"]["npCoords"] = 4
    full = tmp_path / "full"
    full.mkdir()
    ref_io.write_ini(full / "configuration.ini", ini)
    (full / "run").mkdir()
    r = _run(["--precision", "fp64", "--quiet", "--fixed-dt", "--checkpoint", str(full / "end.ckpt")], full / "run")
    assert r.returncode == 0, r.stderr
    half = tmp_path / "half"
    half.mkdir()
    ini_h = ref_io.ini_dict(npDim=4, tMag=3e-11, tRelax=0.0, deltaTinit=1e-12, magFluxDens=0.0, seed=3,
                            volFrac=0.05)
    ini_h["output_settings"]["npCoords"] = 4
    ref_io.write_ini(half / "configuration.ini", ini_h)
    (half / "run").mkdir()
    r = _run(["--precision", "fp64", "--quiet", "--fixed-dt", "--checkpoint", str(half / "mid.ckpt")], half / "run")
    assert r.returncode == 0, r.stderr
    r = _run([str(full / "configuration.ini"), "--precision", "fp64", "--quiet", "--fixed-dt", "--resume",
              str(half / "mid.ckpt"), "--checkpoint", str(half / "end.ckpt")], half / "run")
    assert r.returncode == 0, r.stderr
    assert "resumed from" in r.stdout
    a, ha = _ckpt_state(full / "end.ckpt", 64)
    b, hb = _ckpt_state(half / "end.ckpt", 64)
    assert ha[5] == hb[5]  # same number of steps
    np.testing.assert_allclose(b[1:], a[1:], rtol=0, atol=1e-11)          # moments, easy axes
    np.testing.assert_allclose(b[0], a[0], rtol=0, atol=1e-12 * np.abs(a[0]).max())
