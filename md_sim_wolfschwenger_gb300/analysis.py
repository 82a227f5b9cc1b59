"""Post-processing of a run's records and frames: the reference's MATLAB
analysis scripts (mFiles/ of MD_Sim_Wolfschwenger) restated with numpy, plus
the ensemble statistics used to compare noisy runs.

* `einstein_diffusion` -- mFiles/eval_diffusion.m:25-56: D = slope / 2 of a
  least-squares line through MSD(t) between 30 % and 99 % of the record.
* `radial_distribution` -- mFiles/radial_dist_fun.m:19-66: 500 bins up to
  8 r_mag, minimum image, distances below contact clamped to 2 r_mag,
  normalised by L^3 / (2 pi dr^3 N^2) / (k - 1/2)^2.  The script's inner
  loop stops at particle N - 1 (`for j2 = j1 + 1 : numbPart - 1`), so pairs
  with the last particle are left out; `include_last=True` counts them.
* `orientation_autocorrelation` -- mean over particles of u_i(t) . u_i(0),
  for moments or easy axes (the reference computes no rotational
  coefficient; this is the quantity its coords frames allow).
"""
from __future__ import annotations

import math

import numpy as np


def einstein_diffusion(msd, dt, lo=0.3, hi=0.99):
    """(D, slope, intercept) of MSD(t) = slope t + intercept, t = s dt."""
    msd = np.asarray(msd, dtype=np.float64)
    t = np.arange(msd.size) * dt
    i1, i2 = int(math.floor(msd.size * lo)), int(math.floor(msd.size * hi))
    # MATLAB's time(idx1:idx2) is 1-based and inclusive
    sl = slice(max(i1 - 1, 0), i2)
    k, d = np.polyfit(t[sl], msd[sl], 1)
    return k / 2.0, k, d


def radial_distribution(pos, lBox, rMag0, bins=500, range_mag=8.0, include_last=False):
    """g(r) histogram of one frame; pos is (3, N).  Returns (x, g) with x in
    units of the core diameter 2 rMag0 at the bin centres."""
    pos = np.asarray(pos, dtype=np.float64)
    n = pos.shape[1]
    rng = range_mag * rMag0
    bw = rng / bins
    hist = np.zeros(bins)
    last = n if include_last else n - 1
    for j1 in range(n):
        d = pos[:, j1 + 1:last] - pos[:, j1:j1 + 1]
        d = np.where(d > lBox / 2, d - lBox, d)
        d = np.where(d < -lBox / 2, d + lBox, d)
        r = np.sqrt((d * d).sum(0))
        r = np.maximum(r, 2 * rMag0)
        r = r[r < rng]
        np.add.at(hist, np.floor(r / bw).astype(int), 1)
    norm = lBox ** 3 / (2 * math.pi * bw ** 3 * n * n)
    k = np.arange(1, bins + 1)
    g = hist * norm / (k - 0.5) ** 2
    x = (k - 0.5) * bw / (2 * rMag0)
    return x, g


def orientation_autocorrelation(u_t, u_0):
    """mean_i u_i(t) . u_i(0) for (3, N) unit vectors."""
    return float(np.mean(np.sum(np.asarray(u_t) * np.asarray(u_0), axis=0)))


def ensemble_mean(samples):
    """(mean, standard error of the mean) over the first axis."""
    a = np.asarray(samples, dtype=np.float64)
    m = a.mean(axis=0)
    se = a.std(axis=0, ddof=1) / math.sqrt(a.shape[0]) if a.shape[0] > 1 else np.zeros_like(m)
    return m, se


def agree(mean_a, se_a, mean_b, se_b, z=4.0, floor=0.0):
    """Two-sample test per entry: |a - b| <= z sqrt(se_a^2 + se_b^2) + floor."""
    diff = np.abs(np.asarray(mean_a) - np.asarray(mean_b))
    tol = z * np.sqrt(np.asarray(se_a) ** 2 + np.asarray(se_b) ** 2) + floor
    return bool(np.all(diff <= tol)), diff, tol
