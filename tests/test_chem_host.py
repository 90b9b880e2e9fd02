"""The steady driver's per-cell chemistry, built for the host, against the
oracle's FP64 restatement of the method (no GPU).

tests/host_chem.cpp compiles prism3d_gb300/csrc/p3d_newton.cuh with g++.
The inputs are those the oracle's steady method hands its chemistry solve
(oracle.chem_steady) in outer iterations 0 and 5 on a 24^3 cut of the
Orion-Bar-like slab: rates, shielding columns, Doppler width and the start
abundances.  Both builds converge to the oracle's steady state (the
mixed one factorises in FP32 but iterates on FP64 residuals to the same
rtol 1e-12, with the shielding factors in the mixed kernel's forms):
measured ~1e-15 (FP64) and ~1.4e-14 (mixed), asserted 1e-12 and 1e-10 for
every species above 1e-20 of n_H.
The device build of the same source runs in the -m gpu tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from hostbuild import build
from hostbuild import ptr as _p

SPECIES = ("x_HI", "x_H2", "x_Cp", "x_C", "x_CO")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    return build("host_chem.cpp", tmp_path_factory.mktemp("hostchem"))


@pytest.fixture(scope="module")
def calls(monkeypatch_module):
    """(inputs, oracle outputs) of the oracle's chemistry solve at outer
    iterations 0 and 5."""
    from prism3d_gb300 import fields
    from prism3d_gb300.core import directional_G0
    dens = fields.orion_bar_slab(24, seed=1)
    g0 = directional_G0(2.6e4, [-1.0, 0.0, 0.0], 2)
    seen = []
    real = O.chem_steady

    def spy(*args, **kw):
        k = len(seen)
        keep = k in (0, 5)
        inp = [np.array(a, dtype=np.float64, copy=True) if isinstance(a, np.ndarray) else a
               for a in args] if keep else None
        out = real(*args, **kw)
        if keep:
            res = [np.array(a, copy=True) for a in args[8:15]]
            seen.append((inp, dict(kw), res, out))
        else:
            seen.append(None)
        return out
    monkeypatch_module.setattr(O, "chem_steady", spy)
    O.steady_run(dens, g0, fields.CELL_CM, nside=2, zeta0=2e-16, T_init=100.0, max_outer=6,
                 tol=1e-300, w_chem=0.1)
    return [c for c in seen if c is not None]


@pytest.fixture(scope="module")
def monkeypatch_module():
    mp = pytest.MonkeyPatch()
    yield mp
    mp.undo()


def _host_solve(L, inp, kw, mixed):
    (n_h, kpd0, kci, acp, kco0, rh2, rcr, x_c_total, x_hi, x_h2, x_cp, x_c, x_co, _x_o, _x_e,
     x_hcop) = inp
    kco_cr, u_h2, u_co, _ds, b_dop = kw["selfshield"]
    hcop = np.ravel(x_hcop)
    assert np.all(hcop == hcop[0])  # the driver takes one x_HCO+
    n = np.ravel(n_h).size
    y = np.ascontiguousarray(np.stack([np.ravel(a) for a in (x_hi, x_h2, x_cp, x_c, x_co)],
                                      axis=1))
    f64 = [np.ascontiguousarray(np.ravel(a), dtype=np.float64) for a in
           (n_h, kpd0, kci, acp, kco0, rh2, rcr)]
    ss = [np.ascontiguousarray(np.ravel(a), dtype=np.float64) for a in (kco_cr, u_h2, u_co)]
    fh2 = np.zeros(n)
    it = np.zeros(n, np.int32)
    st = np.zeros(n, np.int32)
    L.hc_chem_steady(ctypes.c_long(n), *[_p(a) for a in f64], ctypes.c_double(x_c_total),
                     ctypes.c_double(hcop[0]), *[_p(a) for a in ss], ctypes.c_double(b_dop),
                     ctypes.c_int(int(mixed)), ctypes.c_int(kw.get("max_iter", 200)),
                     ctypes.c_double(kw.get("rtol", 1e-12)), _p(y), _p(fh2), _p(it), _p(st))
    return y, fh2, st


@pytest.mark.parametrize("mixed,tol", [(False, 1e-12), (True, 1e-10)])
def test_host_chemistry_matches_oracle(lib, calls, mixed, tol):
    assert len(calls) == 2
    for inp, kw, res, (_, _, status, fsh) in calls:
        assert not kw.get("h2_implicit") and not kw.get("co_implicit")
        y, fh2, st = _host_solve(lib, inp, kw, mixed)
        ok = (st == 0) & (np.ravel(status) == 0)
        assert ok.mean() > 0.999, (int((st != 0).sum()), int((np.ravel(status) != 0).sum()))
        for c, name in enumerate(SPECIES):
            ref = np.ravel(res[c])
            m = ok & (ref > 1e-20)
            rel = np.abs(y[:, c] - ref)[m] / ref[m]
            assert rel.max() <= tol, (name, mixed, rel.max())
        np.testing.assert_allclose(fh2[ok], fsh[0][ok], rtol=max(tol, 1e-12))


def test_shielding_slope_in_doppler_width(lib):
    """The worklist wakes a settled cell when |db / b| x |d ln f_H2 / d ln b|
    exceeds its tolerance; the kept slope (closed form) against a central
    difference of f_H2 itself in ln b, and f_H2 against the oracle's
    f_shield_H2, over 1e12-1e24 cm^-2 and b 0.5-20 km/s."""
    rng = np.random.default_rng(3)
    n = 4000
    nh2 = 10 ** rng.uniform(12, 24, n)
    b = rng.uniform(0.5, 20.0, n)
    f = np.zeros(n)
    s = np.zeros(n)
    lib.hc_fsh_h2(ctypes.c_long(n), _p(nh2), _p(b), _p(f), _p(s))
    fp, fm = np.zeros(n), np.zeros(n)
    h = 1e-5
    for out, bb in ((fp, b * np.exp(h)), (fm, b * np.exp(-h))):
        junk = np.zeros(n)
        lib.hc_fsh_h2(ctypes.c_long(n), _p(nh2), _p(np.ascontiguousarray(bb)), _p(out), _p(junk))
    fd = (np.log(fp) - np.log(fm)) / (2 * h)
    assert np.all(s >= 0.0) and s.max() <= 2.0
    # (atol: the difference quotient's rounding, ~1e-16 / h)
    np.testing.assert_allclose(s, np.abs(fd), rtol=1e-5, atol=1e-9)
    # the kernel's f_H2 is the reference's f_shield_H2 with b = sqrt(2 k T / m_H2) / 1e5
    T = (b * 1e5) ** 2 * O.m_H2 / (2.0 * O.k_boltz)
    np.testing.assert_allclose(f, O.f_shield_H2(nh2, T), rtol=1e-12)


def test_analytic_jacobian_matches_fp64_differences(lib):
    """chem5_eval's analytic Jacobian (the chemistry block of the adjoint's
    per-cell Jacobian, p3d_adjoint.cuh) against central differences of the
    same FP64 residual on seeded states over the PDR range, with the
    shielding fixed by the columns and with the cell's own H2 half layer
    inside the solve.  The allowed difference is the difference quotient's
    own error: 1e-6 of the entry (truncation) plus the rounding of the
    residual's terms over the step."""
    rng = np.random.default_rng(17)
    dbl = ctypes.c_double
    worst = 0.0
    for trial in range(400):
        nh = 10 ** rng.uniform(1, 6.5)
        g0 = 10 ** rng.uniform(-1, 5)
        av = rng.uniform(0, 10)
        zeta = 10 ** rng.uniform(-17, -15)
        T = 10 ** rng.uniform(1, 4)
        kpd0 = 4.43e-11 * g0 * np.exp(-3.74 * av)
        kci = 2.56e-10 * g0 * np.exp(-3.02 * av)
        kco0 = 1.71e-10 * g0 * np.exp(-3.53 * av)
        acp = 4.67e-12 * (T / 300.0) ** -0.6
        rh2 = 10 ** rng.uniform(-18, -16) * nh * 0.5
        xh2 = rng.uniform(1e-6, 0.49)
        y = np.array([1 - 2 * xh2, xh2, 10 ** rng.uniform(-9, -4.1), 10 ** rng.uniform(-9, -4.1),
                      10 ** rng.uniform(-12, -4.1)])
        u_h2 = 10 ** rng.uniform(12, 22)
        u_co = 10 ** rng.uniform(8, 18)
        ds = 0.0 if trial % 2 == 0 else 1.5e16
        args = [dbl(v) for v in (nh, kpd0, kci, acp, kco0, rh2, 0.25 * zeta, 1.076e-4, 1e-10,
                                 6 * zeta, 1.0, u_h2, u_co, ds, 1.2)]
        f = np.zeros(5)
        J = np.zeros(25)
        lib.hc_chem5_eval(*args, _p(np.ascontiguousarray(y)), _p(f), _p(J))
        J = J.reshape(5, 5)
        terms = np.abs(J) @ np.abs(y) + np.abs(f)
        for c in range(5):
            h = 1e-6 * y[c]
            fp, fm, junk = np.zeros(5), np.zeros(5), np.zeros(25)
            yp, ym = y.copy(), y.copy()
            yp[c] += h
            ym[c] -= h
            lib.hc_chem5_eval(*args, _p(yp), _p(fp), _p(junk))
            lib.hc_chem5_eval(*args, _p(ym), _p(fm), _p(junk))
            fd = (fp - fm) / (2 * h)
            for r in range(5):
                allowed = 1e-6 * abs(J[r, c]) + 8 * 2.2e-16 * terms[r] / (2 * h)
                worst = max(worst, abs(J[r, c] - fd[r]) / allowed)
    assert worst < 1.0, worst
