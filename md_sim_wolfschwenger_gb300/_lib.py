"""ctypes binding of the C ABI in include/md_gb300.h (libmd_gb300.so).

The library is the only compute path: if it is missing or fails to load,
every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "md_gb300.h")
LIB_PATH = os.path.join(HERE, "_lib", "libmd_gb300.so")

MD_OK = 0
STATUS = {0: "MD_OK", 1: "MD_ERR_INVALID", 2: "MD_ERR_CUDA", 3: "MD_ERR_NOMEM", 4: "MD_ERR_NONFINITE",
          5: "MD_ERR_CONFIG", 6: "MD_ERR_UNSUPPORTED", 7: "MD_ERR_NO_DEVICE"}
MD_PREC_FP64, MD_PREC_MIXED = 0, 1
MD_NOISE_OFF, MD_NOISE_UPLOADED, MD_NOISE_PHILOX = 0, 1, 2
MD_FIELD_STEP, MD_FIELD_SIN = 0, 1
SEGMENTS = ["cells", "real_full", "ksf_full", "kred_full", "kscat_full", "heun1", "real_field", "ksf_field",
            "kred_field", "kscat_field", "heun2", "obs"]


class MdError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def _config_fields():
    """Fields of md_config, parsed from the C header so the mirror cannot drift."""
    src = open(HEADER).read()
    body = src[src.index("typedef struct md_config {"):src.index("} md_config;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for m in re.finditer(r"\b(int64_t|double)\s+([^;]+);", body):
        ty = C.c_int64 if m.group(1) == "int64_t" else C.c_double
        for name in m.group(2).split(","):
            fields.append((name.strip(), ty))
    return fields


class MdConfig(C.Structure):
    _fields_ = _config_fields()

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MdRequest(C.Structure):
    _fields_ = [("n", C.c_int64), ("volFrac", C.c_double), ("steps", C.c_int64), ("dt", C.c_double),
                ("fieldKind", C.c_int64), ("fieldAmp", C.c_double), ("fieldFreq", C.c_double),
                ("seed", C.c_uint64), ("arrival", C.c_double)]


class MdRequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("admitted", C.c_double), ("finished", C.c_double), ("latency", C.c_double),
                ("mz", C.c_double), ("checksum", C.c_double), ("steps_done", C.c_int64),
                ("device_bytes", C.c_int64)]


class MdServeOpts(C.Structure):
    _fields_ = [("hbm_budget", C.c_double), ("max_systems", C.c_int64), ("round_steps", C.c_int64),
                ("realtime", C.c_int), ("autotune", C.c_int)]


class MdServeStats(C.Structure):
    _fields_ = [("wall", C.c_double), ("particle_steps", C.c_double), ("gpu_ms", C.c_double),
                ("admit_ms", C.c_double), ("rounds", C.c_int64), ("repacks", C.c_int64),
                ("peak_systems", C.c_int64), ("peak_bytes", C.c_double)]


_lib = None


def lib():
    """Loads libmd_gb300.so (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} not built; run md_sim_wolfschwenger_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    P = C.POINTER(C.c_double)
    I64 = C.c_int64
    PI64 = C.POINTER(C.c_int64)
    V = C.c_void_p
    sig = {
        "md_strerror": (C.c_char_p, [C.c_int]),
        "md_last_error": (C.c_int, [V, C.c_char_p, C.c_size_t]),
        "md_version": (C.c_char_p, []),
        "md_config_load_ini": (C.c_int, [C.c_char_p, C.POINTER(MdConfig)]),
        "md_config_default": (C.c_int, [C.POINTER(MdConfig)]),
        "md_config_derive": (C.c_int, [C.POINTER(MdConfig)]),
        "md_config_numb_part": (I64, [C.POINTER(MdConfig)]),
        "md_config_size": (C.c_size_t, []),
        "md_select_device": (C.c_int, [C.c_int]),
        "md_ctx_create": (C.c_int, [C.POINTER(MdConfig), I64, C.c_int, C.POINTER(V)]),
        "md_ctx_destroy": (C.c_int, [V]),
        "md_ctx_stream": (C.c_int, [V, C.POINTER(V)]),
        "md_ctx_device_bytes": (C.c_int, [V, PI64]),
        "md_set_particles": (C.c_int, [V, P, P]),
        "md_get_box": (C.c_int, [V, P]),
        "md_set_box": (C.c_int, [V, C.c_double]),
        "md_state_upload": (C.c_int, [V, P, P, P, C.c_int]),
        "md_state_download": (C.c_int, [V, P, P, P]),
        "md_set_time": (C.c_int, [V, C.c_double, I64]),
        "md_checkpoint_save": (C.c_int, [V, C.c_char_p]),
        "md_checkpoint_load": (C.c_int, [V, C.c_char_p]),
        "md_get_time": (C.c_int, [V, P, PI64]),
        "md_ewald_params": (C.c_int, [V, C.c_double, P, P, PI64, P, P]),
        "md_set_ewald": (C.c_int, [V, C.c_double, C.c_double, I64]),
        "md_set_kspace_engine": (C.c_int, [V, C.c_int]),
        "md_kspace_engine_active": (C.c_int, [V, C.POINTER(C.c_int)]),
        "md_set_kspace_tiling": (C.c_int, [V, C.c_int, C.c_int]),
        "md_get_kspace_tiling": (C.c_int, [V, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "md_ewald_params_host": (C.c_int, [C.POINTER(MdConfig), I64, P, P, C.c_double, P, P, PI64, P, P, P]),
        "md_autotune_ewald": (C.c_int, [V, C.c_int, P, P, PI64, P]),
        "md_compute_interactions": (C.c_int, [V, P, P, P]),
        "md_compute_field": (C.c_int, [V, P, P]),
        "md_set_noise": (C.c_int, [V, C.c_int, C.c_uint64]),
        "md_step": (C.c_int, [V, I64, C.c_double, P]),
        # the state arrays as plain addresses (the per-step call is kept lean)
        "md_step_io": (C.c_int, [V, V, V, V, I64, C.c_double, V, V, V]),
        "md_step_adaptive": (C.c_int, [V, I64, C.c_double, P, P, PI64]),
        "md_records": (C.c_int, [V, I64, I64, P]),
        "md_num_records": (C.c_int, [V, PI64]),
        "md_clear_records": (C.c_int, [V]),
        "md_sync": (C.c_int, [V]),
        "md_debug_cells": (C.c_int, [V, PI64, PI64, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "md_debug_structure_factor": (C.c_int, [V, PI64, P]),
        "md_debug_launches": (C.c_int, [V, PI64]),
        "md_debug_pairs": (C.c_int, [V, PI64]),
        "md_debug_real_part": (C.c_int, [V, P, P]),
        "md_set_neighbor_skin": (C.c_int, [V, C.c_double]),
        "md_set_wait_limit": (C.c_int, [V, I64]),
        "md_debug_wait_probe": (C.c_int, [V, C.c_int, I64]),
        "md_set_strong_pairs": (C.c_int, [V, C.c_double]),
        "md_debug_strong_pairs": (C.c_int, [V, PI64]),
        "md_debug_neighbor_capacity": (C.c_int, [V, I64, PI64]),
        "md_profile": (C.c_int, [V, C.c_int]),
        "md_profile_read": (C.c_int, [V, P]),
        "md_calibrate_fp32": (C.c_int, [P]),
        "md_init_system": (C.c_int, [C.POINTER(MdConfig), I64, C.c_uint64, P, P, P, P, P, P]),
        "md_place_rsa": (C.c_int, [I64, C.c_double, P, C.c_uint64, C.c_int, P]),
        "md_autotune_ewald_cached": (C.c_int, [V, C.c_double, P, P, PI64, C.POINTER(C.c_int)]),
        "md_tune_cache_save": (C.c_int, [C.c_char_p]),
        "md_tune_cache_load": (C.c_int, [C.c_char_p]),
        "md_tune_cache_clear": (C.c_int, []),
        "md_batch_create": (C.c_int, [I64, C.POINTER(V)]),
        "md_batch_destroy": (C.c_int, [V]),
        "md_batch_add": (C.c_int, [V, V, I64, C.c_double, PI64]),
        "md_batch_remove": (C.c_int, [V, I64]),
        "md_batch_launch": (C.c_int, [V, I64, PI64]),
        "md_batch_wait": (C.c_int, [V]),
        "md_batch_run": (C.c_int, [V, I64, PI64]),
        "md_batch_remaining": (C.c_int, [V, I64, PI64, C.POINTER(C.c_int)]),
        "md_batch_info": (C.c_int, [V, PI64, PI64, PI64, P]),
        "md_serve_run": (C.c_int, [C.POINTER(MdConfig), C.POINTER(MdRequest), I64, C.POINTER(MdServeOpts),
                                   C.POINTER(MdRequestResult), C.POINTER(MdServeStats)]),
        "md_write_matrix_txt": (C.c_int, [C.c_char_p, P, I64, I64, C.c_int, C.c_double]),
        "md_write_coords_txt": (C.c_int, [C.c_char_p, I64, P, P, P, C.c_double]),
        "md_write_data_txt": (C.c_int, [C.c_char_p, C.POINTER(MdConfig), I64, P, P, C.c_double]),
        "md_export_records_txt": (C.c_int, [C.c_char_p, P, I64, C.c_double, I64]),
        "md_rdf": (C.c_int, [V, I64, C.c_double, C.c_double, C.c_int, P, C.POINTER(C.c_uint64)]),
        "md_noalloc_scratch_bytes": (C.c_size_t, []),
        "md_structure_factor_noalloc": (C.c_int, [V, V, I64, C.c_double, I64, C.c_double, V, PI64, V]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if L.md_config_size() != C.sizeof(MdConfig):
        raise OSError(f"md_config size mismatch: C {L.md_config_size()} vs ctypes {C.sizeof(MdConfig)}")
    _lib = L
    return L


def exported_symbols():
    """Every function name declared in include/md_gb300.h."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(md_[a-z0-9_]+)\s*\(", src)))


def check(status, ctx=None):
    if status != MD_OK:
        buf = C.create_string_buffer(1024)
        lib().md_last_error(ctx, buf, len(buf))
        raise MdError(status, buf.value.decode(errors="replace"))
