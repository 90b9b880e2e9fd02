"""The steady driver's per-cell physics (prism3d_gb300/csrc/p3d_phys.cuh),
built for the host (tests/host_phys.cpp), against the reference's own
values (tests/golden/elementwise.npz, tests/golden/make_golden.py): H2
self-shielding at five grid-mean temperatures, CO shielding, cosmic-ray
attenuation for two zeta_0, dust temperature, the H2 formation rate and
the PE heating (condensed tables formed here as pe_condense_kernel does) on
4000 points including the branch edges.  Tolerance 1e-13 relative (FP64
pow/exp/log10 of the host library against NumPy's); the mixed path's forms
of the shielding factors and the H2 formation rate to the same values
within the tolerances in FAST_TOL."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from hostbuild import build
from hostbuild import ptr as _p


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    return build("host_phys.cpp", tmp_path_factory.mktemp("hostphys"))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# the mixed path's forms of the shielding factors and the H2 formation
# rate (FAST: one denominator, logarithms and exp64 instead of divisions,
# pow() and exp()) against the same reference values (measured: fsh_h2
# 6e-16, fsh_co 4e-14, h2_form 6e-16); their N_H2 derivatives against the plain forms', to
# 1e-13 of the largest (the CO one is a difference of two terms)
FAST_TOL = {"fsh_h2": 1e-13, "fsh_co": 1e-13, "h2_form": 1e-13}


@pytest.mark.parametrize("fast", [0, 1])
def test_shielding_and_cosmic_rays(lib, golden, fast):
    g = golden("elementwise")
    n = g["N_H2"].size
    out = np.zeros(n)
    d = np.zeros(n)
    d_plain = np.zeros(n)
    for i, tm in enumerate(g["T_mean"]):
        b = np.sqrt(2.0 * O.k_boltz * tm / O.m_H2) / 1e5
        lib.hp_fsh_h2(ctypes.c_long(n), _p(_c(g["N_H2"])), ctypes.c_double(b), _p(out), _p(d),
                      ctypes.c_int(fast))
        np.testing.assert_allclose(out, g[f"fsh_h2_{i}"],
                                   rtol=FAST_TOL["fsh_h2"] if fast else 1e-13, atol=0)
        lib.hp_fsh_h2(ctypes.c_long(n), _p(_c(g["N_H2"])), ctypes.c_double(b), _p(out),
                      _p(d_plain), ctypes.c_int(0))
        np.testing.assert_allclose(d, d_plain, rtol=1e-13, atol=1e-13 * np.abs(d_plain).max())
    lib.hp_fsh_co(ctypes.c_long(n), _p(_c(g["N_CO"])), _p(_c(g["N_H2"])), _p(out), _p(d),
                  ctypes.c_int(fast))
    np.testing.assert_allclose(out, g["fsh_co"], rtol=FAST_TOL["fsh_co"] if fast else 1e-13,
                               atol=0)
    lib.hp_fsh_co(ctypes.c_long(n), _p(_c(g["N_CO"])), _p(_c(g["N_H2"])), _p(out), _p(d_plain),
                  ctypes.c_int(0))
    np.testing.assert_allclose(d, d_plain, rtol=1e-13, atol=1e-13 * np.abs(d_plain).max())
    n = g["N_H"].size
    out = np.zeros(n)
    for z0 in (2e-16, 5e-16):
        lib.hp_cr_rate(ctypes.c_long(n), _p(_c(g["N_H"])), ctypes.c_double(z0), _p(out))
        np.testing.assert_allclose(out, g[f"zeta_{z0:g}"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("fast", [0, 1])
def test_dust_temperature_and_h2_formation(lib, golden, fast):
    from prism3d_gb300.tables import DustTables
    g = golden("elementwise")
    tb = DustTables()
    n = g["G0"].size
    td = np.zeros(n)
    lib.hp_tdust(ctypes.c_long(n), _p(_c(g["G0"])), _p(_c(g["AV"])), _p(_c(g["nH"])),
                 _p(_c(g["Tg"])), _p(td))
    np.testing.assert_allclose(td, g["Td"], rtol=1e-13, atol=0)
    rh2 = np.zeros(n)
    lib.hp_h2_form(ctypes.c_long(n), _p(_c(g["Tg"])), _p(td), _p(_c(g["fn"])),
                   ctypes.c_double(tb.sigma_nano), ctypes.c_double(tb.sigma_largeC),
                   ctypes.c_double(tb.sigma_Sil), _p(rh2), ctypes.c_int(fast))
    np.testing.assert_allclose(rh2, g["RH2"], rtol=FAST_TOL["h2_form"] if fast else 1e-13,
                               atol=0)


def test_pe_heating(lib, golden):
    from prism3d_gb300.tables import DustTables
    g = golden("elementwise")
    tb = DustTables()
    # per (psi, E_g) node: sum over bins of dn/da sigma_abs table, nano bins
    # apart (the bins in order, as the condensing kernel adds them)
    w = tb.bin_dn_da_da * tb.bin_sigma_abs
    nano = tb.bin_is_nano.astype(bool)
    a_nano = np.zeros(tb.pe_table.shape[1:])
    a_rest = np.zeros(tb.pe_table.shape[1:])
    for b in range(tb.n_bins):
        if nano[b]:
            a_nano += w[b] * tb.pe_table[b]
        else:
            a_rest += w[b] * tb.pe_table[b]
    n = g["G0"].size
    out = np.zeros(n)
    lib.hp_pe(ctypes.c_long(n), ctypes.c_double(tb.log_psi_min), ctypes.c_double(tb.log_psi_step),
              ctypes.c_int(tb.n_psi), ctypes.c_double(tb.eg_min), ctypes.c_double(tb.eg_step),
              ctypes.c_int(tb.n_Eg), _p(_c(a_nano)), _p(_c(a_rest)),
              *[_p(_c(g[k])) for k in ("G0", "Tg", "xe", "nH", "fn", "eg")], _p(out))
    np.testing.assert_allclose(out, g["GPE"], rtol=1e-13, atol=0)


def test_interp_idx_weight_known_answers(lib):
    """The reference's Rust unit test (rust/src/pe_table.rs:147-171) on the
    device function: middle of the grid, between nodes, clamped low and
    high."""
    def iw(x):
        i = ctypes.c_int()
        w = ctypes.c_double()
        lib.hp_interp_idx_weight(ctypes.c_double(x), ctypes.c_double(0.0), ctypes.c_double(1.0),
                                 ctypes.c_int(10), ctypes.byref(i), ctypes.byref(w))
        return i.value, w.value
    assert iw(3.0) == (3, 0.0)
    i, w = iw(3.5)
    assert i == 3 and abs(w - 0.5) < 1e-10
    assert iw(-1.0) == (0, 0.0)
    assert iw(100.0) == (8, 1.0)
    assert iw(float("nan"))[0] == 0  # NaN maps to index 0 (Rust's saturating cast)


def test_gas_grain_speed_constants_are_the_rounded_expression():
    """csrc/p3d_phys.cuh keeps sqrt(8 k_B / (pi mu m_H)) for mu = 1, 2 as
    literals; they must be the doubles the per-cell expression rounds to
    (IEEE division and square root are correctly rounded on the host as on
    the device with -prec-div / -prec-sqrt), so the thermal contexts are
    unchanged bit for bit."""
    import math
    import os
    import re
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "prism3d_gb300", "csrc")
    text = open(os.path.join(csrc, "p3d_phys.cuh")).read()
    common = open(os.path.join(csrc, "p3d_common.cuh")).read()

    def const(src, name):
        return re.search(rf"constexpr double {name} = ([^;]+);", src).group(1).strip()

    kb = float(const(common, "kKBoltz"))
    mh = float(const(text, "kMH"))
    pi = float(const(text, "kPi"))
    for mu, name in ((1.0, "kGgSpeedMu1"), (2.0, "kGgSpeedMu2")):
        assert float.fromhex(const(text, name)) == math.sqrt(8.0 * kb / (pi * mu * mh)), name
