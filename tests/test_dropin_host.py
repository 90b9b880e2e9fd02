"""The drop-in kernels' cell functions, built for the host
(tests/host_dropin.cpp), against the reference's own values
(tests/golden/thermal_chem.npz from tests/golden/make_golden.py) on the
reference's 8^3 parity fixture (p8) and a dense lit cube (d8): the net
heating at ten temperatures (1e-12 of the terms' size), the 10 + 3 thermal
root (1e-10), the explicit-Euler chemistry after 1, 7 and 20 substeps
(1e-12), and the reference's Rust unit tests of the chemistry (H and C
conservation, rust/src/chemistry.rs:190-238) and of the thermal root
(rust/src/thermal.rs:378-447).  The device builds run in
tests/test_gpu_dropin.py."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from hostbuild import build
from hostbuild import ptr as _p


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    from prism3d_gb300 import tables
    L = build("host_dropin.cpp", tmp_path_factory.mktemp("hostdropin"))
    lp = [np.ascontiguousarray(a, dtype=np.float64) for a in tables.line_params()]
    co = np.ascontiguousarray(tables.co_ladder(), dtype=np.float64)
    L.hd_init(*[_p(a) for a in lp], _p(co))
    return L


def _ptrs(arrays):
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in arrays]
    arr = (ctypes.c_void_p * len(keep))(*[a.ctypes.data for a in keep])
    return arr, keep


@pytest.mark.parametrize("case", ["p8", "d8"])
def test_thermal_matches_reference(lib, golden, case):
    g = golden("thermal_chem")
    ctx, keep = _ptrs(g[f"{case}_ctx"])
    n = keep[0].size
    for k, tv in enumerate(g[f"{case}_tgrid"]):
        out = np.zeros(n)
        lib.hd_net64(ctypes.c_long(n), ctx, ctypes.c_double(tv), _p(out))
        ref = g[f"{case}_net"][k]
        scale = np.abs(keep[0]) + np.abs(ref) + 1e-40
        assert np.max(np.abs(out - ref) / scale) < 1e-12, tv
    t = np.zeros(n)
    lib.hd_thermal13(ctypes.c_long(n), ctx, ctypes.c_int(10), ctypes.c_int(3), _p(t))
    np.testing.assert_allclose(t, g[f"{case}_T13"], rtol=1e-10)


@pytest.mark.parametrize("case", ["p8", "d8"])
@pytest.mark.parametrize("ns", [1, 7, 20])
def test_chemistry_euler_matches_reference(lib, golden, case, ns):
    g = golden("thermal_chem")
    st = {k[len(case) + 4:]: g[k] for k in g.files if k.startswith(case + "_st_")}
    st["zeta_CR"] = g[f"{case}_zeta"]
    rates, keep = _ptrs(O.chem_rates(st, g[f"{case}_fsh"], g[f"{case}_fco"]))
    xin = g[f"{case}_chem_in"]
    n = xin[0].size
    y = np.ascontiguousarray(np.stack([xin[i] for i in range(5)], axis=1))
    hcop = np.ascontiguousarray(np.ravel(st["x_HCOp"]), dtype=np.float64)
    lib.hd_chem_euler(ctypes.c_long(n), rates, ctypes.c_double(float(g["x_C_total"][0])),
                      _p(y), _p(hcop), ctypes.c_int(ns), ctypes.c_double(1e-4))
    ref = g[f"{case}_chem_out{ns}"]
    for i in range(5):
        np.testing.assert_allclose(y[:, i], ref[i], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(np.maximum(y[:, 2] + hcop, 1e-30), ref[5], rtol=1e-12,
                               atol=1e-300)


def test_known_answers(lib):
    # chemistry: one cell, 200 substeps (rust/src/chemistry.rs:190-238)
    rates, keep = _ptrs([np.array([v]) for v in (1e3, 1e-15, 1e-14, 4.67e-12, 1e-14,
                                                   3e-17 * 1e3 * 0.5, 2.5e-17)])
    y = np.array([[0.5, 0.25, 5e-5, 1e-5, 4e-5]])
    lib.hd_chem_euler(ctypes.c_long(1), rates, ctypes.c_double(1.076e-4), _p(y),
                      _p(np.array([1e-10])), ctypes.c_int(200), ctypes.c_double(1e-4))
    assert abs(y[0, 0] + 2 * y[0, 1] - 1.0) < 1e-10
    assert abs(y[0, 2:].sum() - 1.076e-4) / 1.076e-4 < 1e-6
    # thermal (rust/src/thermal.rs:378-447): finite net heating of a warm
    # surface cell at 500 K; a root inside [10, 1e5] K
    k, mh = O.k_boltz, O.m_H
    for n_h, gf, td, tv in ((1e4, 1e-20, 30.0, 500.0), (1e3, 1e-22, 20.0, None)):
        gg = 2.0 * 0.35 * 1e-21 * n_h * n_h * np.sqrt(8.0 * k / (np.pi * mh)) * k
        ctx, keep = _ptrs([np.array([v]) for v in (gf, gg, td, 1e-4 * n_h, 0.9 * n_h, 0.05 * n_h,
                                                   1e-6 * n_h, 1e-4 * n_h, 3e-4 * n_h,
                                                   1e-5 * n_h)])
        out = np.zeros(1)
        if tv is not None:
            lib.hd_net64(ctypes.c_long(1), ctx, ctypes.c_double(tv), _p(out))
            assert np.isfinite(out[0])
        else:
            lib.hd_thermal13(ctypes.c_long(1), ctx, ctypes.c_int(10), ctypes.c_int(3), _p(out))
            assert 10.0 <= out[0] <= 1e5
