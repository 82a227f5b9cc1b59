"""md_structure_factor_noalloc: the structure factor for callers that cannot
call cudaMalloc (a framework that owns all device memory, a loop that must
not allocate after start-up).  Its result must equal the structure factor of
the context-based path (md_compute_interactions + md_debug_structure_factor)
for the same particles, on two calls in a row that share the library's one
static scratch array.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import TOL_FP64, gpu_system, random_system

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_structure_factor_matches_context_path():
    torch = pytest.importorskip("torch")
    import md_sim_wolfschwenger_gb300 as m
    L = m.lib()
    ini, g = random_system(512, seed=41, rc_frac=0.3)
    n, kc = g["n"], g["kc"]
    assert kc <= 16
    d = O.derive(ini)
    magmom = d["satMag"] * 4.0 / 3.0 * d["my_pi"] * g["rMag"] ** 3.0
    sim = gpu_system(ini, g, 0)  # FP64 context path: the existing entry points
    rng = np.random.default_rng(3)
    out = torch.zeros((20000, 5), dtype=torch.float64, device="cuda")
    for call in range(2):
        mm = g["mm"] if call == 0 else g["mm"] + 0.3 * rng.standard_normal(g["mm"].shape)
        if call:
            mm = mm / np.linalg.norm(mm, axis=0)
        sim.set_state(g["pos"], mm, g["ea"])
        sim.CompInteractions()
        S_ref = sim.debug_structure_factor()
        pos_d = torch.tensor(g["pos"], dtype=torch.float64, device="cuda").contiguous()
        mom_d = torch.tensor(mm * magmom[None, :], dtype=torch.float64, device="cuda").contiguous()
        nk = C.c_int64(0)
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        st = L.md_structure_factor_noalloc(_ptr(pos_d), _ptr(mom_d), n, g["lBox"], kc, d["my_pi"], _ptr(out),
                                           C.byref(nk), stream)
        assert st == 0
        torch.cuda.synchronize()
        S_new = out[:nk.value].cpu().numpy()
        lut = {tuple(int(v) for v in r[:3]): r[3:] for r in S_new}
        assert len(lut) == nk.value
        scale = np.abs(mm * magmom[None, :]).max() * np.sqrt(n) * kc
        got = np.array([lut[tuple(int(v) for v in r[:3])] for r in S_ref])
        assert np.abs(got - S_ref[:, 3:]).max() < TOL_FP64 * scale, call


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import md_sim_wolfschwenger_gb300 as m
    L = m.lib()
    nk = C.c_int64(0)
    one = C.c_void_p(1)  # never dereferenced: the size check comes first
    assert L.md_structure_factor_noalloc(one, one, 10, 1e-6, 17, 3.14159265359, one, C.byref(nk), None) == 1
    # particle count beyond 2^30 (the documented limit; indexing is 64-bit below it)
    assert L.md_structure_factor_noalloc(one, one, (1 << 30) + 1, 1e-6, 8, 3.14159265359, one, C.byref(nk),
                                         None) == 1
    assert L.md_noalloc_scratch_bytes() == 2430592
