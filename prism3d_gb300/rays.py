"""Ray set and per-ray external field of the FUV transfer (host side, NumPy).

No device code and no library load: the benchmark's CPU reference arm and the
workload builders use these without touching libprism3d_gb300.so.
"""
from __future__ import annotations

import numpy as np


def healpix_directions(nside=2):
    """Fibonacci-spiral ray set of the reference (radiative_transfer/fuv_rt.py:19-57).

    Evaluated with NumPy in the reference's operation order, so the ray
    directions (and hence every ds and dominant axis) equal the reference's.
    """
    n = 12 * nside ** 2
    d = np.zeros((n, 3))
    w = np.full(n, 4.0 * np.pi / n)
    ga = np.pi * (3.0 - np.sqrt(5.0))
    for i in range(n):
        ct = 1.0 - 2.0 * (i + 0.5) / n
        st = np.sqrt(1.0 - ct ** 2)
        ph = ga * i
        d[i, 0] = st * np.cos(ph)
        d[i, 1] = st * np.sin(ph)
        d[i, 2] = ct
    return d, w


def directional_G0(G0, source_direction, nside=1, background=0.0):
    """Per-ray G0 for a distant source (radiative_transfer/fuv_rt_3d.py:21-71)."""
    d, w = healpix_directions(nside)
    src = np.asarray(source_direction, dtype=np.float64)
    src = src / np.linalg.norm(src)
    cos = d @ src
    lit = cos > 0
    ws = np.sum(np.where(lit, cos * w, 0.0))
    g = np.where(lit, G0 * cos * (4.0 * np.pi) / ws, 0.0) if ws > 0 else np.full(len(d), G0)
    return g + background
