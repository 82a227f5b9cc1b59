"""The bounded-wait error path of the tensor-core kernels.  Every mbarrier
wait there gives up after a limit of SM clock cycles (md_set_wait_limit);
the kernel then records the failure, frees its tensor memory and returns,
and the call reports MD_ERR_CUDA.  The probe (md_debug_wait_probe) takes
those steps on an mbarrier that nothing signals, with a short limit, so the
wait runs out without any fault; the context must then keep working."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import TOL_MIXED, gpu_system, load_golden, oracle_system, scales

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_is_reported_and_the_context_recovers():
    import md_sim_wolfschwenger_gb300 as m
    L = m.lib()
    ini, g = load_golden("n64_noiseoff")
    sim = gpu_system(ini, g, 1)
    # signalled barrier: the wait succeeds
    assert L.md_debug_wait_probe(sim.h, 1, 2_000_000) == 0
    # nothing arrives: the wait gives up after ~1 ms of SM cycles
    st = L.md_debug_wait_probe(sim.h, 0, 2_000_000)
    assert st == 2
    buf = C.create_string_buffer(512)
    L.md_last_error(sim.h, buf, len(buf))
    assert b"wait gave up" in buf.value
    # the error word was cleared and the tensor memory freed: normal work goes on
    assert L.md_debug_wait_probe(sim.h, 1, 2_000_000) == 0
    fAl, bAl, _ = scales(ini, g)
    B, F, _ = sim.CompInteractions()
    Bo, Fo, _ = oracle_system(ini, g).compute_interactions()
    assert O.rms_rel(B, Bo, bAl) < TOL_MIXED and O.rms_rel(F, Fo, fAl) < TOL_MIXED


def test_wait_limit_is_a_runtime_parameter():
    import md_sim_wolfschwenger_gb300 as m
    L = m.lib()
    ini, g = load_golden("n64_noiseoff")
    sim = gpu_system(ini, g, 1)
    assert L.md_set_wait_limit(sim.h, 10) == 1  # below the floor: rejected
    assert L.md_set_wait_limit(sim.h, 500_000_000) == 0
    B, F, _ = sim.CompInteractions()  # tensor-core k space under the new limit
    assert np.all(np.isfinite(B)) and np.all(np.isfinite(F))
