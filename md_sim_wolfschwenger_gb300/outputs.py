"""The reference's text output files (saveData, WriteCoords2TXT,
WriteData2TXT, ExportDiffVis in src/postprocessing.cpp of
MD_Sim_Wolfschwenger) written by the library's C writers from host arrays.
A time label of exactly 0 truncates a file, any other value appends."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import check, lib
from .simulation import Configuration


def _P(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _arr(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def write_matrix(path, a, t_int=0.0):
    """saveData: a 2-D array (or a vector, written as one column)."""
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a[:, None]
    a = np.ascontiguousarray(a)
    check(lib().md_write_matrix_txt(os.fsencode(path), _P(a), a.shape[0], a.shape[1], 0, float(t_int)))


def write_coords(path, pos, mm, ea, t_int):
    """WriteCoords2TXT: one frame of (3, N) positions, moments, easy axes."""
    pos = _arr(pos)
    n = pos.size // 3
    mm, ea = _arr(mm, (3, n)), _arr(ea, (3, n))
    check(lib().md_write_coords_txt(os.fsencode(path), n, _P(pos), _P(mm), _P(ea), float(t_int)))


def write_data(path, config: Configuration, rMag, rHydr, lBox):
    """WriteData2TXT: radii and the run's settings."""
    rMag, rHydr = _arr(rMag), _arr(rHydr)
    check(lib().md_write_data_txt(os.fsencode(path), C.byref(config.c), rMag.size, _P(rMag), _P(rHydr),
                                  float(lBox)))


def export_records(directory, records, t_int, steps):
    """ExportDiffVis + mz.txt + t.txt from (count, 8) per-step records."""
    r = _arr(records)
    count = r.size // 8
    check(lib().md_export_records_txt(os.fsencode(directory or ""), _P(r), count, float(t_int), int(steps)))
