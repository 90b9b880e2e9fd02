"""Column-density maps on the device: the GPU counterparts of
``integrate_column`` and ``column_density_maps``
(prism3d/observations/jwst_pipeline.py:109-180), same arguments and keys.

``solver`` is a PDRSolverGPU (its device state is used in place) or any
object with the reference solver's attributes (density, x_H2, x_CO, x_Cp,
x_e as (nx, ny, nz) float64 arrays, cell_size).
"""
from __future__ import annotations

import numpy as np

from . import _lib as L

MAP_KEYS = ("N_H", "N_H2", "N_CO", "N_Cp", "N_e", "A_V_total")


def _map_shape(shape, los_axis):
    return tuple(n for a, n in enumerate(shape) if a != los_axis)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def column_density_maps(solver, los_axis=2, inclination_deg=0.0):
    """N_H, N_H2, N_CO, N_Cp, N_e [cm^-2] and A_V_total along los_axis;
    |inclination_deg| >= 0.01 shears the cube as the reference does."""
    from .solver import PDRSolverGPU
    shape = tuple(np.shape(solver.density))
    if len(shape) != 3:
        raise ValueError("density must be (nx, ny, nz)")
    mshape = _map_shape(shape, los_axis) if los_axis in (0, 1, 2) else (0,)
    out = np.empty((6,) + mshape)
    if isinstance(solver, PDRSolverGPU):
        L.call("p3d_steady_column_maps", solver._h, float(solver.cell_size), int(los_axis),
               float(inclination_deg), L.dptr(out))
    else:
        f = [_f64(getattr(solver, k)) for k in ("density", "x_H2", "x_CO", "x_Cp", "x_e")]
        if any(a.shape != shape for a in f):
            raise ValueError("all fields must have the density's shape")
        L.call("p3d_column_maps", *shape, *[L.dptr(a) for a in f], float(solver.cell_size),
               int(los_axis), float(inclination_deg), L.dptr(out))
    return {k: out[i] for i, k in enumerate(MAP_KEYS)}


def integrate_column(solver, quantity, los_axis=2):
    """Sum of a 3-D quantity (attribute name or array) along los_axis times
    the cell size."""
    data = getattr(solver, quantity) if isinstance(quantity, str) else quantity
    data = _f64(data)
    if data.ndim != 3:
        raise ValueError("quantity must be a 3-D array")
    out = np.empty(_map_shape(data.shape, los_axis) if los_axis in (0, 1, 2) else (0,))
    L.call("p3d_integrate_column", *data.shape, L.dptr(data), float(solver.cell_size),
           int(los_axis), L.dptr(out))
    return out
