"""GPU steady-state driver against the FP64 CPU restatement of the method.

The oracle's steady_run (oracle/oracle.py) and the device driver iterate the
same outer map to a relative change below 1e-10; their fixed points must
agree to 1e-6 relative for every species above 1e-20 of n_H and 1e-4 for
T_gas (the spec bar), and the mixed-precision path must agree with the
plain FP64 path to the same bar.  Bit-exact: the selected ray per cell.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
SPECIES = ("x_HI", "x_H2", "x_Cp", "x_C", "x_CO")


def _cmp(a, b, rel, floor):
    m = np.abs(b) > floor
    err = np.abs(a - b)[m] / np.abs(b)[m]
    return float(np.max(err)) if err.size else 0.0, int(np.sum(np.abs(a - b)[m] > rel * np.abs(b)[m]))


def _run_gpu(name, mixed, tol=1e-10, seed=1):
    from prism3d_gb300 import fields
    from prism3d_gb300.solver import PDRSolverGPU
    dens, g0, nside, zeta, cell = fields.workload(name, seed)
    s = PDRSolverGPU(dens, cell * dens.shape[0], G0_external=g0, zeta_CR_0=zeta, nside_rt=nside,
                     T_init=100.0)
    ok = s.run(max_iterations=3000, convergence_tol=tol, mixed=mixed)
    return s, ok


@pytest.fixture(scope="module")
def cube16_oracle():
    from prism3d_gb300 import fields
    dens, g0, nside, zeta, cell = fields.workload("cube16")
    st, hist = O.steady_run(dens, g0, cell, nside=nside, zeta0=zeta, max_outer=3000, tol=1e-10)
    assert hist[-1]["dmax"] < 1e-10
    return st


def test_steady_plain_matches_oracle(cube16_oracle):
    s, ok = _run_gpu("cube16", mixed=False)
    assert ok, s.last_change
    ref = cube16_oracle
    assert np.array_equal(s.selected_ray(), ref["ray"])
    for k in ("G0", "A_V", "N_H"):
        np.testing.assert_allclose(s.get(k), ref[k], rtol=1e-12)
    np.testing.assert_array_equal(s.get("A_V"), ref["A_V"])
    errs = {k: _cmp(s.get(k), ref[k], 1e-6, 1e-20) for k in SPECIES}
    errs["T_gas"] = _cmp(s.get("T_gas"), ref["T_gas"], 1e-4, 0.0)
    for k, (mx, nbad) in errs.items():
        assert nbad == 0, (k, mx, nbad, errs)


def test_steady_mixed_matches_plain():
    sp, okp = _run_gpu("cube16", mixed=False)
    sm, okm = _run_gpu("cube16", mixed=True)
    assert okp and okm
    for k in SPECIES:
        mx, nbad = _cmp(sm.get(k), sp.get(k), 1e-6, 1e-20)
        assert nbad == 0, (k, mx, nbad)
    mx, nbad = _cmp(sm.get("T_gas"), sp.get("T_gas"), 1e-4, 0.0)
    assert nbad == 0, ("T_gas", mx, nbad)


def test_steady_state_is_fixed_point_of_reference_iteration(cube16_oracle):
    """One more outer iteration with the oracle from the GPU state changes
    nothing beyond the tolerance (chemistry at its steady state, thermal root
    at its root)."""
    s, ok = _run_gpu("cube16", mixed=True)
    assert ok
    st = dict(cube16_oracle)
    for k in SPECIES + ("T_gas",):
        st[k] = s.get(k)
    h = st["x_HI"] + 2 * st["x_H2"]
    np.testing.assert_allclose(h, 1.0, atol=1e-12)
    c = st["x_Cp"] + st["x_C"] + st["x_CO"]
    np.testing.assert_allclose(c, O.X_C, rtol=1e-12)
