"""Output files: the library's writers (md_write_*_txt, md_export_records_txt)
against the text files the reference's own writers (saveData,
WriteCoords2TXT, WriteData2TXT, ExportDiffVis; src/postprocessing.cpp) wrote
from the same numbers (tests/golden/n64_outputs_txt/, made by
tests/golden/make_golden.py).  Byte-for-byte.  CPU only."""
import os

import numpy as np

from helpers import GOLDEN, load_golden, md_config
from md_sim_wolfschwenger_gb300 import outputs

REF_TXT = os.path.join(GOLDEN, "n64_outputs_txt")


def _same(a, b):
    with open(a, "rb") as fa, open(b, "rb") as fb:
        x, y = fa.read(), fb.read()
    assert x == y, (os.path.basename(a), x[:200], y[:200])


def _final_time(g):
    t = 0.0
    for _ in range(g["nsteps"]):
        t += g["dt"]  # RunSimulation's tInt += deltaTused
    return t


def test_output_files_match_reference_writers(tmp_path):
    ini, g = load_golden("n64_outputs")
    cfg = md_config(ini, vis=g["vis"], n=g["n"])
    cfg.set(absTol=1e300)  # the harness's override (every step accepted)
    t_end = _final_time(g)
    outputs.write_data(tmp_path / "data.txt", cfg, g["rMag"], g["rHydr"], g["lBox"])
    outputs.write_coords(tmp_path / "coords.txt", g["ref_posF"], g["ref_mmF"], g["ref_eaF"], 0.0)
    outputs.write_coords(tmp_path / "coords.txt", g["ref_posF"], g["ref_mmF"], g["ref_eaF"], t_end)
    outputs.export_records(str(tmp_path), g["ref_obs"], t_end, g["nsteps"])
    names = sorted(os.listdir(REF_TXT))
    assert names == sorted(os.listdir(tmp_path))
    for nm in names:
        _same(os.path.join(REF_TXT, nm), tmp_path / nm)


def test_zero_label_truncates_and_other_labels_append(tmp_path):
    p = tmp_path / "m.txt"
    outputs.write_matrix(p, np.array([[1.0, -2.5], [3e-9, 40.0]]), 1.0)
    outputs.write_matrix(p, np.array([[5.0]]), 0.0)
    assert p.read_text() == "5\n\n"
    outputs.write_matrix(p, np.array([1.0, 123456789.0, -0.5]), 2.0)
    assert p.read_text() == "5\n\n          1\n1.23457e+08\n       -0.5\n\n"
