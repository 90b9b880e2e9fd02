"""Column-density maps: oracle pinned to the reference (CPU), GPU kernels
against the reference's own maps (gpu marker)."""
import os
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

G = np.load(os.path.join(ROOT, "tests", "golden", "maps.npz"))
KEYS = ("N_H", "N_H2", "N_CO", "N_Cp", "N_e", "A_V_total")


def _fields():
    s = types.SimpleNamespace(**{k: G[k] for k in ("density", "x_H2", "x_CO", "x_Cp", "x_e",
                                                  "T_gas")})
    s.cell_size = float(G["cell_size"])
    return s


def _cases():
    return [(los, j, float(inc)) for los in range(3) for j, inc in enumerate(G["inclinations"])]


def test_oracle_maps_match_reference():
    s = _fields()
    for los, j, inc in _cases():
        m = O.column_density_maps(s.density, s.x_H2, s.x_CO, s.x_Cp, s.x_e, s.cell_size, los,
                                  inc)
        for k in KEYS:
            np.testing.assert_allclose(m[k], G[f"{k}_{los}_{j}"], rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_gpu_maps_match_reference():
    from prism3d_gb300.observations import column_density_maps, integrate_column
    s = _fields()
    for los, j, inc in _cases():
        m = column_density_maps(s, los_axis=los, inclination_deg=inc)
        for k in KEYS:
            np.testing.assert_allclose(m[k], G[f"{k}_{los}_{j}"], rtol=1e-13, atol=0)
    for los in range(3):
        np.testing.assert_allclose(integrate_column(s, "T_gas", los_axis=los),
                                   G[f"int_T_{los}"], rtol=1e-13, atol=0)


@pytest.mark.gpu
def test_gpu_maps_of_steady_state():
    from prism3d_gb300 import fields
    from prism3d_gb300.observations import column_density_maps
    from prism3d_gb300.solver import PDRSolverGPU
    dens, g0, nside, zeta, cell = fields.workload("cube16", seed=1)
    s = PDRSolverGPU(dens, cell * 16, G0_external=g0, zeta_CR_0=zeta, nside_rt=nside,
                     T_init=100.0)
    s.run(max_iterations=20, convergence_tol=1e-300, mixed=True, n_allow=0)
    for los, inc in ((0, 0.0), (2, 4.0)):
        m = column_density_maps(s, los_axis=los, inclination_deg=inc)
        ref = O.column_density_maps(s.density, s.x_H2, s.x_CO, s.x_Cp, s.x_e, s.cell_size, los,
                                    inc)
        for k in KEYS:
            np.testing.assert_allclose(m[k], ref[k], rtol=1e-13, atol=0)
    s.close()


@pytest.mark.gpu
def test_gpu_maps_argument_errors():
    from prism3d_gb300 import _lib as L
    from prism3d_gb300.observations import column_density_maps
    s = _fields()
    with pytest.raises(L.P3DError):
        column_density_maps(s, los_axis=3)
    with pytest.raises(L.P3DError):
        column_density_maps(s, inclination_deg=90.0)
