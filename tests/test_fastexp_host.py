"""The table-driven FP64 exponential of the thermal and ray-march kernels
(prism3d_gb300/csrc/p3d_fastexp.cuh, Tang's method), built for the host,
against the C library's exp over the range the kernels use and beyond it
(where it defers to exp).  The device build runs the same operations (FMA,
integer exponent arithmetic); the -m gpu ray-march and thermal tests check
it there through their oracle comparisons."""
import numpy as np
import pytest

from hostbuild import build, ptr


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    return build("host_fastexp.cpp", tmp_path_factory.mktemp("fastexp"))


def _exp(L, x):
    import ctypes
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    L.fe_exp64(ctypes.c_long(x.size), ptr(x), ptr(out))
    return out


def test_exp64_within_one_ulp(lib):
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-700, 700, 400000), rng.uniform(-1, 1, 200000),
                        rng.uniform(-1e-3, 1e-3, 50000),
                        np.arange(-700, 701, dtype=np.float64) * np.log(2.0) / 64.0 * 64,
                        (np.arange(-2000, 2001) + 0.5) * np.log(2.0) / 64.0,
                        [0.0, -0.0, 1e-300, -1e-300, 700.0, -700.0]])
    got = _exp(lib, x)
    ref = np.exp(x)
    rel = np.abs(got - ref) / ref
    ulp = np.abs(got - ref) / np.spacing(ref)
    assert rel.max() < 3.5e-16, rel.max()
    assert ulp.max() <= 2.0, ulp.max()


def test_exp64_outside_range_defers(lib):
    x = np.array([-745.2, -720.0, -708.5, 705.0, 709.7, -np.inf, np.inf, np.nan, 1e5, -1e5])
    got = _exp(lib, x)
    with np.errstate(over="ignore"):
        ref = np.exp(x)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    m = ~np.isnan(ref)
    assert np.array_equal(got[m], ref[m])
