"""Seeded synthetic inputs for the five benchmark workloads.

No public dataset exists for these workloads; each generator draws from
``numpy.random.default_rng(seed)`` with the shapes, means and log-normal
widths the workloads name.  Cell size is 0.005 pc throughout.

    lognormal_cube  white noise -> periodic Gaussian smoothing (sigma = 2
                    cells) -> standardise -> n = mean exp(sigma_ln g - sigma_ln^2/2)
    orion_bar_slab  log10 n_base = lo + (hi - lo) (1 + tanh((x - L/4)/w)) / 2
                    (w = 0.0125 pc, so the ramp spans ~0.05 pc) times a
                    mean-one log-normal perturbation
    cored_slab      orion_bar_slab plus seeded Gaussian cores (peak n_core,
                    FWHM 3 cells)
"""
from __future__ import annotations

import numpy as np

from .constants import pc_cm

CELL_PC = 0.005
CELL_CM = CELL_PC * pc_cm


def _smooth_periodic(g, sigma_cells):
    """Gaussian filter with periodic boundaries, via FFT."""
    out = np.fft.fftn(g)
    for ax, n in enumerate(g.shape):
        k = np.fft.fftfreq(n)
        shape = [1] * g.ndim
        shape[ax] = n
        out *= np.exp(-2.0 * (np.pi * sigma_cells * k) ** 2).reshape(shape)
    return np.real(np.fft.ifftn(out))


def lognormal_field(shape, sigma_ln, seed, smooth=2.0):
    rng = np.random.default_rng(seed)
    g = _smooth_periodic(rng.standard_normal(shape), smooth)
    g = (g - g.mean()) / g.std()
    return np.exp(sigma_ln * g - 0.5 * sigma_ln ** 2)


def lognormal_cube(n, mean, sigma_ln, seed=1):
    return mean * lognormal_field((n, n, n), sigma_ln, seed)


def orion_bar_slab(n, lo=1e3, hi=1e5, sigma_ln=0.8, seed=1, width_pc=0.0125):
    L = n * CELL_PC
    x = (np.arange(n) + 0.5) * CELL_PC
    ramp = 0.5 * (1.0 + np.tanh((x - 0.25 * L) / width_pc))
    base = 10.0 ** (np.log10(lo) + (np.log10(hi) - np.log10(lo)) * ramp)
    return base[:, None, None] * lognormal_field((n, n, n), sigma_ln, seed)


def cored_slab(n, lo=1e3, hi=3e5, sigma_ln=1.2, seed=1, n_cores=None, n_core=1e6):
    dens = orion_bar_slab(n, lo, hi, sigma_ln, seed)
    rng = np.random.default_rng(seed + 1000)
    if n_cores is None:
        n_cores = max(1, n // 16)
    sig = 3.0 / (2.0 * np.sqrt(2.0 * np.log(2.0)))
    idx = np.arange(n)
    for _ in range(n_cores):
        c = rng.uniform(n * 0.3, n, 3) if n > 4 else rng.uniform(0, n, 3)
        lo_i = np.maximum((c - 6 * sig).astype(int), 0)
        hi_i = np.minimum((c + 6 * sig).astype(int) + 1, n)
        sl = tuple(slice(a, b) for a, b in zip(lo_i, hi_i))
        gx, gy, gz = np.meshgrid(idx[sl[0]], idx[sl[1]], idx[sl[2]], indexing="ij")
        r2 = (gx + 0.5 - c[0]) ** 2 + (gy + 0.5 - c[1]) ** 2 + (gz + 0.5 - c[2]) ** 2
        dens[sl] = np.maximum(dens[sl], n_core * np.exp(-0.5 * r2 / sig ** 2))
    return dens


# name -> (density builder, G0, nside, zeta_CR_0)
WORKLOADS = {
    "cube16": (lambda seed=1: lognormal_cube(16, 1e4, 1.0, seed), 1e4, 1, 2e-16),
    "cube64": (lambda seed=1: lognormal_cube(64, 1e4, 1.5, seed), 1e3, 2, 2e-16),
    "slab128": (lambda seed=1: orion_bar_slab(128, seed=seed), 2.6e4, 2, 2e-16),
    "cube32": (lambda seed=1: lognormal_cube(32, 3e4, 1.0, seed), 1e4, 1, 2e-16),
    "slab256": (lambda seed=1: cored_slab(256, seed=seed), 2.6e4, 2, 5e-16),
    # the 128^3 slab's recipe on 96^3 cells: state (~0.27 GB) above L2, small
    # enough for a profiler capture
    "slab96": (lambda seed=1: orion_bar_slab(96, seed=seed), 2.6e4, 2, 2e-16),
}


# name -> one-line description (bench config)
WORKLOAD_DESC = {
    "cube16": "16^3 log-normal cube, mean n_H 1e4, sigma_ln 1.0, G0 1e4 on -x, 12 rays",
    "cube64": "64^3 log-normal cube, mean n_H 1e4, sigma_ln 1.5, G0 1e3 on -x, 48 rays",
    "slab128": "128^3 tanh-ramp slab 1e3->1e5 x lognormal 0.8, G0=2.6e4 on -x, 48 rays",
    "cube32": "32^3 log-normal cube, mean n_H 3e4, sigma_ln 1.0, G0 1e4 on -x, 12 rays",
    "slab256": "256^3 tanh-ramp slab 1e3->3e5 x lognormal 1.2 + Gaussian cores (1e6), "
               "G0=2.6e4 on -x, 48 rays, zeta 5e-16",
    "slab96": "96^3 tanh-ramp slab 1e3->1e5 x lognormal 0.8, G0=2.6e4 on -x, 48 rays",
}


def network_cells(n, seed=1):
    """Per-cell conditions (n, 7: n_H, T, G0, A_V, zeta, f_sh_H2, f_sh_CO) for
    the full-network benchmark: log-uniform n_H 10-3e6 cm^-3, T 10-1e4 K, G0
    0.1-1e5, uniform A_V 0-20, zeta 1e-17-1e-15 s^-1, f_sh_H2 1e-8-1,
    f_sh_CO 1e-6-1 (the span of the PDR cells the network is solved on)."""
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(np.stack(
        [10 ** rng.uniform(1, 6.5, n), 10 ** rng.uniform(1, 4, n), 10 ** rng.uniform(-1, 5, n),
         rng.uniform(0, 20, n), 10 ** rng.uniform(-17, -15, n), 10 ** rng.uniform(-8, 0, n),
         10 ** rng.uniform(-6, 0, n)], axis=1))


def workload(name, seed=1):
    """(density, G0_rays (per-ray array, source on -x), nside, zeta0, cell_size)."""
    from .rays import directional_G0
    build, g0, nside, zeta = WORKLOADS[name]
    dens = build(seed)
    return dens, directional_G0(g0, [-1.0, 0.0, 0.0], nside), nside, zeta, CELL_CM
