"""md_step_io (the state in, nsteps, the state out, one synchronisation)
against the separate calls it combines: md_state_upload (reset = 0),
md_step and md_state_download give the same trajectory bit for bit, with
the drawn noise on and both precisions; uploaded noise is refused."""
import numpy as np
import pytest

from helpers import gpu_system, random_system
from md_sim_wolfschwenger_gb300 import MdError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_step_io_matches_separate_calls(prec):
    ini, g = random_system(700, seed=31, rc_frac=0.3, noise=True)
    a = gpu_system(ini, g, prec, noise=2, seed=5)  # Philox noise
    b = gpu_system(ini, g, prec, noise=2, seed=5)
    state = (g["pos"].copy(), g["mm"].copy(), g["ea"].copy())
    sa = tuple(x.copy() for x in state)
    sb = tuple(x.copy() for x in state)
    for _ in range(4):
        sa = a.step_io(sa, 2, 1e-12)
        b.set_state(*sb, reset=False)
        b.step(2, 1e-12)
        sb = b.get_state()
        for x, y in zip(sa, sb):
            np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a.records(), b.records())
    assert np.abs(sa[0] - state[0]).max() > 0  # the particles moved


def test_step_io_refuses_uploaded_noise():
    ini, g = random_system(64, seed=2, rc_frac=0.4)
    sim = gpu_system(ini, g, 1, noise=1)  # uploaded normals
    with pytest.raises(MdError):
        sim.step_io((g["pos"], g["mm"], g["ea"]), 1, 1e-12)
