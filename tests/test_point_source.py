"""Point-source FUV field: oracle pinned to the reference (CPU, bit-exact),
GPU against the reference's own outputs (gpu marker)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

G = np.load(os.path.join(ROOT, "tests", "golden", "point_source.npz"))
KEYS = ("G0", "A_V", "N_H", "N_H2", "N_CO")


def _cases():
    for s in range(len(G["stars"])):
        for w in range(2):
            ab = (G["x_H2"], G["x_CO"]) if w == 0 else (None, None)
            yield s, w, ab


def test_oracle_point_source_matches_reference():
    for s, w, (a, b) in _cases():
        res = O.fuv_point_source(G["density"], G["stars"][s], float(G["L_FUV"]),
                                 float(G["cell_size"]), a, b)
        for k, v in zip(KEYS, res):
            np.testing.assert_array_equal(v, G[f"{k}_{s}_{w}"])


@pytest.mark.gpu
def test_gpu_point_source_matches_reference():
    from prism3d_gb300.core import compute_fuv_field_point_source
    for s, w, (a, b) in _cases():
        res = compute_fuv_field_point_source(G["density"], G["stars"][s], float(G["L_FUV"]),
                                             float(G["cell_size"]), x_H2=a, x_CO=b)
        for k, v in zip(KEYS, res):
            ref = G[f"{k}_{s}_{w}"]
            if k == "G0":  # exp rounding
                np.testing.assert_allclose(v, ref, rtol=1e-14, atol=0)
            else:  # columns: same operations in the same order
                np.testing.assert_array_equal(v, ref)


@pytest.mark.gpu
def test_gpu_point_source_device_tensors_and_size():
    torch = pytest.importorskip("torch")
    from prism3d_gb300.core import compute_fuv_field_point_source
    rng = np.random.default_rng(5)
    shape = (96, 80, 72)
    cell = 1.5428e16
    dens = 10 ** rng.uniform(2, 5, shape)
    xh2 = rng.uniform(0, 0.5, shape)
    pos = np.array([40.3, 17.8, 60.1]) * cell
    res = compute_fuv_field_point_source(torch.from_numpy(dens).cuda(), pos, 1e38, cell,
                                         x_H2=torch.from_numpy(xh2).cuda())
    torch.cuda.synchronize()
    ref = O.fuv_point_source(dens, pos, 1e38, cell, xh2, None)
    for k, v, r in zip(KEYS, res, ref):
        v = v.cpu().numpy()
        if k == "G0":
            np.testing.assert_allclose(v, r, rtol=1e-14, atol=0)
        else:
            np.testing.assert_array_equal(v, r)
