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


def test_step_io_output_arrays_checked():
    """Output arrays are written through their addresses: a strided view
    or another dtype is refused before the call; strided inputs are copied."""
    ini, g = random_system(64, seed=4, rc_frac=0.4)
    sim = gpu_system(ini, g, 1)
    state = (g["pos"], g["mm"], g["ea"])
    wide = np.zeros((3, 2 * g["n"]))
    with pytest.raises(ValueError):
        sim.step_io(state, 1, 1e-12, out=[wide[:, ::2], np.zeros((3, g["n"])), np.zeros((3, g["n"]))])
    with pytest.raises(ValueError):
        sim.step_io(state, 1, 1e-12, out=[np.zeros((3, g["n"]), dtype=np.float32)] * 3)
    ref = gpu_system(ini, g, 1)
    strided = [np.asfortranarray(x) for x in state]
    out = sim.step_io(strided, 1, 1e-12)
    exp = ref.step_io(state, 1, 1e-12)
    for x, y in zip(out, exp):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("prec", [0, 1])
def test_step_io_with_mapped_host_buffers(prec):
    """Page-locked host buffers, which the device addresses directly: the
    state goes in and out through kernels instead of copies, with the same
    trajectory as the separate calls on pageable arrays, including a move of
    every particle beyond half the list's skin between two calls (the input
    kernel's displacement check must force the rebuild)."""
    torch = pytest.importorskip("torch")
    ini, g = random_system(700, seed=37, rc_frac=0.3, noise=True)
    a = gpu_system(ini, g, prec, noise=2, seed=5)
    b = gpu_system(ini, g, prec, noise=2, seed=5)
    keep = []

    def pinned(x):
        t = torch.empty(x.shape, dtype=torch.float64).pin_memory()
        keep.append(t)
        v = t.numpy()
        v[...] = x
        return v

    sin = [pinned(x) for x in (g["pos"], g["mm"], g["ea"])]
    sout = [pinned(np.zeros_like(x)) for x in sin]
    sb = [x.copy() for x in (g["pos"], g["mm"], g["ea"])]
    L = g["lBox"]
    rng = np.random.default_rng(3)
    for it in range(4):
        if it == 2:
            p = sin[0] + 0.02 * g["rc"] * rng.standard_normal(sin[0].shape)
            p -= L * np.round(p / L)
            sin[0][...] = p
            sb[0] = p.copy()
        a.step_io(sin, 2, 1e-12, out=sout)
        b.set_state(*sb, reset=False)
        b.step(2, 1e-12)
        sb = list(b.get_state())
        for x, y in zip(sout, sb):
            np.testing.assert_array_equal(x, y)
        for x, y in zip(sin, sout):
            x[...] = y
    np.testing.assert_array_equal(a.records(), b.records())


def test_step_io_partly_registered_buffer_is_refused():
    """A host array page-locked over its first part only is not handed to
    the transfer kernels (both ends must lie in one mapping); the copy
    engines refuse a range that straddles a registration, so the call
    reports MD_ERR_CUDA, and the context goes on with proper arrays."""
    torch = pytest.importorskip("torch")
    rt = torch.cuda.cudart()
    ini, g = random_system(700, seed=41, rc_frac=0.3, noise=True)
    a = gpu_system(ini, g, 1, noise=2, seed=5)
    b = gpu_system(ini, g, 1, noise=2, seed=5)
    n = g["n"]
    raw = np.empty(3 * n + 1024)
    off = ((-raw.ctypes.data) % 4096) // 8
    pos = raw[off:off + 3 * n].reshape(3, n)
    pos[...] = g["pos"]
    part = (3 * n * 8 // 2) // 4096 * 4096
    assert part > 0
    torch.cuda.check_error(rt.cudaHostRegister(pos.ctypes.data, part, 2))  # cudaHostRegisterMapped
    try:
        with pytest.raises(MdError):
            a.step_io((pos, g["mm"], g["ea"]), 2, 1e-12)
    finally:
        torch.cuda.check_error(rt.cudaHostUnregister(pos.ctypes.data))
    out = a.step_io((pos, g["mm"], g["ea"]), 2, 1e-12)
    b.set_state(g["pos"], g["mm"], g["ea"], reset=False)
    b.step(2, 1e-12)
    for x, y in zip(out, b.get_state()):
        np.testing.assert_array_equal(x, y)
