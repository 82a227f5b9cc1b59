"""Initial particle systems on the host (InitParticleProps size draws and
InitCoordsFromSketch, src/simulation.cpp:118-351 of MD_Sim_Wolfschwenger),
with numpy's seeded generator in place of EigenRand's Mersenne Twister.

`rsa_positions` is the reference's random sequential addition (uniform
candidate in [-(L/2 - r_h), L/2 - r_h]^3, rejected if it overlaps any placed
hydrodynamic sphere) with a cell grid so that it runs in O(N) instead of
O(N^2)."""
from __future__ import annotations

import math

import numpy as np


def lognormal_radii(n, median, sigma_ln, rng):
    """Core radii with ln(r) ~ N(ln(median), sigma_ln)."""
    return median * np.exp(sigma_ln * rng.standard_normal(n))


def box_length(rHydr, volFrac, my_pi=3.14159265359):
    """L = (sum V_hydr / volFrac)^(1/3) (simulation.cpp:56)."""
    vh = 4.0 / 3.0 * my_pi * np.asarray(rHydr, dtype=np.float64) ** 3.0
    return math.pow(float(vh.sum()) / volFrac, 1.0 / 3.0)


def rsa_positions(L, rHydr, rng, max_tries=100000, largest_first=None):
    """(3, N) positions, non-overlapping hydrodynamic spheres.  Particles are
    placed in index order like the reference; with largest_first (default:
    when the radii are not all equal) they are placed in order of decreasing
    radius, which keeps dense polydisperse systems from jamming on the last
    large particles.  Each particle keeps its own index either way."""
    rH = np.asarray(rHydr, dtype=np.float64)
    n = rH.size
    if largest_first is None:
        largest_first = bool(rH.max() > rH.min())
    order = np.argsort(-rH, kind="stable") if largest_first else np.arange(n)
    cs = 2.0 * rH.max()
    nc = max(1, int(L // cs))
    cs = L / nc
    cells = {}
    pos = np.zeros((n, 3))
    for i in order:
        for _ in range(max_tries):
            x = rng.uniform(-1.0, 1.0, 3) * (L / 2.0 - rH[i])
            c = np.minimum(((x + L / 2) / cs).astype(int), nc - 1)
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in cells.get(((c[0] + dx), (c[1] + dy), (c[2] + dz)), ()):
                            d = pos[j] - x
                            if d @ d < (rH[i] + rH[j]) ** 2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                break
        else:
            raise RuntimeError("random sequential addition failed: volume fraction too high")
        pos[i] = x
        cells.setdefault((c[0], c[1], c[2]), []).append(i)
    return np.ascontiguousarray(pos.T)


def uniform_directions(n, rng):
    """Unit vectors uniform on the sphere (simulation.cpp:304-312)."""
    az = rng.uniform(0.0, 1.0, n) * 2 * math.pi
    el = 2.0 * np.arcsin(np.sqrt(rng.uniform(0.0, 1.0, n)))
    return np.ascontiguousarray(np.stack([np.sin(el) * np.cos(az), np.sin(el) * np.sin(az), np.cos(el)]))
