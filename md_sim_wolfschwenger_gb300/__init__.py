"""GB300 implementation of the coupled LLG + Brownian-dynamics time step for
magnetic nanoparticle suspensions (drop-in for the hot path of
MD_Sim_Wolfschwenger).  The compute path is libmd_gb300.so (hand-written
CUDA for sm_103a) behind the C ABI in include/md_gb300.h."""
from ._lib import (MD_FIELD_SIN, MD_FIELD_STEP, MD_NOISE_OFF, MD_NOISE_PHILOX, MD_NOISE_UPLOADED, MD_PREC_FP64,
                   MD_PREC_MIXED, MdConfig, MdError, exported_symbols, lib)
from .simulation import Configuration, Simulation, calibrate_fp32, select_device
from . import outputs
from .batch import (Batch, autotune_ewald_cached, init_system, place_rsa, serve, tune_cache_clear, tune_cache_load,
                    tune_cache_save)

__all__ = ["Configuration", "Simulation", "Batch", "outputs", "serve", "init_system", "place_rsa", "autotune_ewald_cached",
           "tune_cache_save", "tune_cache_load", "tune_cache_clear", "calibrate_fp32", "select_device", "MdConfig",
           "MdError", "lib",
           "exported_symbols", "MD_PREC_FP64",
           "MD_PREC_MIXED", "MD_NOISE_OFF", "MD_NOISE_UPLOADED", "MD_NOISE_PHILOX", "MD_FIELD_STEP", "MD_FIELD_SIN"]
