"""Diagnostics Gamma and Lambda (_total_heating_vec / _total_cooling_vec,
prism3d/solver_3d.py:898-1050) against golden vectors of the reference
(tests/golden/make_heating.py): the oracle's NumPy restatement, and the
device function heating_cooling64 built for the host (tests/host_root.cpp),
both on the thermal context the oracle's thermal_ctx builds from the same
states.  The GPU entry points are checked in tests/test_gpu_dropin.py.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from hostbuild import ptr as _p
from hostbuild import root_lib

STATE = ("density", "G0", "A_V", "zeta_CR", "x_HI", "x_H2", "x_Cp", "x_C", "x_CO", "x_O", "x_e",
         "T_dust", "Gamma_PE", "R_H2")


@pytest.fixture(scope="module")
def case(golden):
    g = golden("heating")
    ctx = O.thermal_ctx({k: g[k] for k in STATE}, g["f_sh_H2"])
    T = g["T"]
    # Gamma can cancel (heating vs gas-grain cooling): compare on the scale
    # of its two parts
    scale = np.abs(ctx[0]) + np.abs(ctx[1] * np.sqrt(T) * (ctx[2] - T))
    return g, ctx, T, scale


def test_oracle_heating_cooling_matches_reference(case):
    g, ctx, T, scale = case
    G, L = O.total_heating_cooling(ctx, T)
    assert np.max(np.abs(G - g["Gamma"]) / scale) < 1e-12
    np.testing.assert_allclose(L, g["Lambda"], rtol=1e-12, atol=0)
    # Gamma - Lambda is the thermal balance the roots solve
    net = O.net_heating_at(ctx, T)
    assert np.max(np.abs((G - L) - net) / (scale + L)) < 1e-12


def test_host_built_heating_cooling_matches_reference(case, tmp_path):
    g, ctx, T, scale = case
    lib = root_lib(tmp_path)
    c = np.ascontiguousarray(np.stack([np.ravel(a) for a in ctx], axis=1))
    n = c.shape[0]
    G = np.zeros(n)
    L = np.zeros(n)
    lib.hr_heating_cooling(ctypes.c_long(n), _p(c), _p(np.ascontiguousarray(T)), _p(G), _p(L))
    assert np.max(np.abs(G - g["Gamma"]) / scale) < 1e-12
    np.testing.assert_allclose(L, g["Lambda"], rtol=1e-12, atol=0)
