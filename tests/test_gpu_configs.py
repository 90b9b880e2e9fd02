"""Steady-state parity at the benchmark configurations (GB300).

* 64^3 log-normal cube (sigma_ln 1.5, G0 1e3 on -x, 48 rays): the plain FP64
  path's first outer iterations against the oracle's FP64 restatement of the
  method, cell by cell; and the converged mixed-precision state against the
  converged plain FP64 one, cell by cell.
* 128^3 Orion-Bar-like slab (the headline workload): converged mixed against
  converged plain FP64, cell by cell.

Tolerances are those of the headline metric: abundances (relative to n_H)
within 1e-6 relative where the plain value is above 1e-20, T_gas within 1e-4
relative.  A solve counts as converged when at most n_allow = max(8, 1e-5 n)
cells still change by more than tol (1e-8) per iteration; those cells (the
'change' field above tol in either solve) are reported and excluded, and
there are at most n_allow of them per solve.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
KEYS = ("T_gas", "x_HI", "x_H2", "x_Cp", "x_C", "x_CO", "x_O", "x_e")
TOL = 1e-8


def _solve(name, mixed):
    from prism3d_gb300 import fields
    from prism3d_gb300.solver import PDRSolverGPU
    dens, g0, nside, zeta, cell = fields.workload(name, 1)
    s = PDRSolverGPU(dens, cell * dens.shape[0], G0_external=g0, zeta_CR_0=zeta,
                     nside_rt=nside, T_init=100.0)
    n_allow = max(8, int(1e-5 * dens.size))
    ok = s.run(max_iterations=4000, convergence_tol=TOL, mixed=mixed, n_allow=n_allow,
               w_chem=0.1)
    st = {k: s.get(k) for k in KEYS + ("change",)}
    s.close()
    return ok, n_allow, st


def _compare(mixed, plain):
    moving = (mixed["change"] > TOL) | (plain["change"] > TOL)
    worst = {}
    bad = np.zeros(moving.shape, bool)
    for k in KEYS:
        a, b = mixed[k], plain[k]
        m = np.abs(b) > 1e-20
        rel = np.zeros(a.shape)
        rel[m] = np.abs(a - b)[m] / np.abs(b)[m]
        off = rel > (1e-4 if k == "T_gas" else 1e-6)
        bad |= off
        worst[k] = float(rel[~moving].max())
    return bad, moving, worst


@pytest.mark.parametrize("name", ["cube64", "slab128"])
def test_converged_mixed_matches_plain(name):
    okp, n_allow, plain = _solve(name, False)
    okm, _, mixed = _solve(name, True)
    assert okp and okm
    bad, moving, worst = _compare(mixed, plain)
    assert int(np.sum(mixed["change"] > TOL)) <= n_allow
    assert int(np.sum(plain["change"] > TOL)) <= n_allow
    assert not np.any(bad & ~moving), (int(np.sum(bad & ~moving)), worst)


def test_cube64_plain_first_iterations_match_oracle():
    """Three plain FP64 outer iterations on the 64^3 cube against the
    oracle's FP64 steady method (oracle.steady_run), cell by cell."""
    from prism3d_gb300 import fields
    from prism3d_gb300.solver import PDRSolverGPU
    dens, g0, nside, zeta, cell = fields.workload("cube64", 1)
    s = PDRSolverGPU(dens, cell * dens.shape[0], G0_external=g0, zeta_CR_0=zeta,
                     nside_rt=nside, T_init=100.0)
    s.run(max_iterations=3, convergence_tol=1e-300, mixed=False, n_allow=0, w_chem=0.1)
    assert s.iterations == 3
    ref, _ = O.steady_run(dens, g0, cell, nside=nside, zeta0=zeta, max_outer=3, tol=0.0,
                          w_chem=0.1)
    assert np.array_equal(s.selected_ray(), ref["ray"])
    np.testing.assert_array_equal(s.get("A_V"), ref["A_V"])
    np.testing.assert_array_equal(s.get("N_H"), ref["N_H"])
    np.testing.assert_allclose(s.get("G0"), ref["G0"], rtol=1e-12)
    for key in KEYS:
        a, b = s.get(key), ref[key]
        m = np.abs(b) > 1e-20
        rel = np.abs(a - b)[m] / np.abs(b)[m]
        assert rel.max() <= 1e-8, (key, rel.max(), int(np.sum(rel > 1e-8)))
    s.close()
