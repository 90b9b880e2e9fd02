"""Selected-ray H2 / CO columns of the steady driver (ss_columns_kernel)
against the oracle's restatement of the reference's per-ray cumulative sums
(prism3d/radiative_transfer/fuv_rt_3d.py:297-392, restricted to each cell's
selected ray).

The grids are non-cubic, with pencil lengths that are not multiples of the
kernel's chunk (8 cells), of the warp width (32) or of the z step (128
cells), so every partial tile, chunk and step is exercised; the abundances
span ten decades so a column that cancelled against a larger sum would show.
The kernel sums in chunks, not strictly left to right, so the columns agree
to rounding (1e-12 relative).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,nside", [((37, 45, 150), 2), ((20, 33, 17), 1),
                                         ((9, 260, 11), 2)])
def test_columns_match_oracle(shape, nside):
    from prism3d_gb300 import fields
    from prism3d_gb300.rays import directional_G0, healpix_directions
    from prism3d_gb300.solver import PDRSolverGPU
    rng = np.random.default_rng(sum(shape))
    dens = 1e3 * fields.lognormal_field(shape, 1.5, seed=3)
    g0 = directional_G0(1e4, [-1.0, 0.3, 0.2], nside)
    cell = fields.CELL_CM
    s = PDRSolverGPU(dens, cell * shape[0], G0_external=g0, nside_rt=nside, T_init=100.0)
    xh2 = 10 ** rng.uniform(-10, np.log10(0.5), shape)
    xco = 10 ** rng.uniform(-14, -4, shape)
    s.set("x_H2", xh2)
    s.set("x_CO", xco)
    nh2, nco = s.columns()
    ray = s.selected_ray()
    dirs, _ = healpix_directions(nside)
    ref_h2, ref_co = O.selected_columns(dens, xh2, xco, ray, dirs, cell)
    s.close()
    assert np.all(ray >= 0)
    for got, ref in ((nh2, ref_h2), (nco, ref_co)):
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)
