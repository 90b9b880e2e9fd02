"""Dust steps inside the device steady-state driver: the reference's
two-level loop (prism3d/solver_3d.py:239-249), one THEMIS grain step
(_evolve_dust_state, :465-507) on every cell before each inner convergence
but the first.

Checked on the 16^3 cube with three dust steps: the per-cell grain state
after two grain steps equals the oracle's restatement of the grain step
applied twice to the device's G0 (the ray march fixes G0, so the grain
state does not depend on the gas); the converged state after the last step
is a fixed point of the oracle's outer map with that per-cell grain state
(abundances within 1e-6, T within 1e-4 or on a jump of the outer map); and
it differs from the one-step steady state (the grain state matters)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
SPECIES = ("x_HI", "x_H2", "x_Cp", "x_C", "x_CO")


@pytest.mark.parametrize("mixed", [True, False])
def test_dust_steps_reach_the_grain_state_fixed_point(mixed):
    from prism3d_gb300 import fields
    from prism3d_gb300.solver import PDRSolverGPU
    dens, g0, nside, zeta, cell = fields.workload("cube16", 1)
    s = PDRSolverGPU(dens, cell * 16, G0_external=g0, zeta_CR_0=zeta, nside_rt=nside,
                     T_init=100.0)
    assert s.run(max_iterations=3000, convergence_tol=1e-9, mixed=mixed, n_allow=0)
    one = {k: s.get(k) for k in SPECIES + ("T_gas",)}
    np.testing.assert_array_equal(s.get("f_nano"), 1.0)
    np.testing.assert_array_equal(s.get("E_g"), 0.1)
    s.reset()
    assert s.run(max_iterations=3000, convergence_tol=1e-9, mixed=mixed, n_allow=0,
                 dust_steps=3)
    G0 = s.get("G0")
    fn, eg = np.ones_like(G0), np.full_like(G0, 0.1)
    for _ in range(2):
        fn, eg = O.evolve_dust_state(G0, dens, fn, eg)
    np.testing.assert_allclose(s.get("f_nano"), fn, rtol=1e-13)
    np.testing.assert_allclose(s.get("E_g"), eg, rtol=1e-13)
    st = {k: s.get(k) for k in SPECIES + ("x_O", "x_e", "T_gas")}
    st["f_nano"], st["E_g"] = s.get("f_nano"), s.get("E_g")
    assert np.all(s.get("change") <= 1e-9)
    x_star, G, _, _ = O.map_residual(st, dens, g0, cell, nside, zeta)
    for k in SPECIES:
        m = st[k] > 1e-20
        rel = np.abs(x_star[k] - st[k])[m] / st[k][m]
        assert rel.max() <= 1e-6, (k, rel.max())
    T = st["T_gas"]
    off = np.abs(G - T) / T > 1e-4
    assert np.mean(off) < 0.01, int(off.sum())
    moved = max(np.max(np.abs(st[k] - one[k]) / np.abs(one[k])) for k in SPECIES)
    assert moved > 1e-3
    s.close()
