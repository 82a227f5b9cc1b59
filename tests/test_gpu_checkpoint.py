"""Checkpoint / resume (md_checkpoint_save/load): a context restored from
the file continues exactly like the saving run, bit for bit, in both
precisions; mismatched or truncated files are refused."""
import numpy as np
import pytest

import md_sim_wolfschwenger_gb300 as m
from helpers import gpu_system, random_system

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_resume_continues_bit_for_bit(tmp_path, prec):
    ini, g = random_system(700, seed=81, rc_frac=0.3, noise=True, B0=0.02, lognormal=True)
    a = gpu_system(ini, g, prec, noise=m.MD_NOISE_PHILOX, seed=5)
    a.step(7, g["dt"])
    path = tmp_path / "state.ckpt"
    a.checkpoint_save(path)
    a.clear_records()
    a.step(6, g["dt"])
    sa, ra, ta = a.get_state(), a.records(), a.get_time()
    b = gpu_system(ini, g, prec)  # fresh context, same configuration and particle count
    b.checkpoint_load(path)
    b.step(6, g["dt"])
    sb, rb, tb = b.get_state(), b.records(), b.get_time()
    for x, y in zip(sa, sb):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(ra, rb)
    assert ta == tb and ta[1] == 13


def test_refuses_foreign_or_truncated_files(tmp_path):
    ini, g = random_system(300, seed=82, rc_frac=0.3)
    a = gpu_system(ini, g, 1)
    path = tmp_path / "s.ckpt"
    a.checkpoint_save(path)
    other = random_system(301, seed=83, rc_frac=0.3)
    b = gpu_system(*other, 1)
    with pytest.raises(m.MdError):
        b.checkpoint_load(path)
    c = gpu_system(ini, g, 0)  # other precision
    with pytest.raises(m.MdError):
        c.checkpoint_load(path)
    data = path.read_bytes()
    (tmp_path / "cut.ckpt").write_bytes(data[: len(data) // 2])
    with pytest.raises(m.MdError):
        a.checkpoint_load(tmp_path / "cut.ckpt")
    (tmp_path / "junk.ckpt").write_bytes(b"not a checkpoint at all" * 10)
    with pytest.raises(m.MdError):
        a.checkpoint_load(tmp_path / "junk.ckpt")
