"""Grain-state step: oracle pinned to the reference (CPU), GPU against the
reference's outputs (gpu marker)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

G = np.load(os.path.join(ROOT, "tests", "golden", "dust.npz"))


def test_oracle_dust_step_matches_reference():
    fn, eg = O.evolve_dust_state(G["G0"], G["density"], G["f_nano"], G["E_g"])
    np.testing.assert_array_equal(fn, G["f_nano_out"])
    np.testing.assert_array_equal(eg, G["E_g_out"])


@pytest.mark.gpu
def test_gpu_dust_step_matches_reference():
    from prism3d_gb300.core import evolve_dust_state
    fn, eg = evolve_dust_state(G["G0"], G["density"], G["f_nano"], G["E_g"])
    np.testing.assert_allclose(fn, G["f_nano_out"], rtol=1e-14, atol=0)  # exp rounding
    np.testing.assert_allclose(eg, G["E_g_out"], rtol=1e-14, atol=0)    # log10 rounding
