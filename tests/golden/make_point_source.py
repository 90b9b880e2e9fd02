"""Golden point-source FUV fields from the reference.

    python tests/golden/make_point_source.py /path/to/prism3d/checkout

Runs compute_fuv_field_point_source (prism3d/radiative_transfer/
fuv_rt_3d.py:74-212) on a seeded non-cubic grid for star positions inside
the grid, on a cell edge, at a corner and outside it, with and without H2/CO
abundances, and writes tests/golden/point_source.npz.  Nothing at test or
run time reads the reference checkout.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.path.insert(0, ref_root)
    from prism3d.radiative_transfer.fuv_rt_3d import compute_fuv_field_point_source
    rng = np.random.default_rng(31)
    shape = (14, 11, 9)
    cell = 1.5428e16
    dens = 10 ** rng.uniform(2, 5, shape)
    xh2 = rng.uniform(0, 0.5, shape)
    xco = 10 ** rng.uniform(-8, -4, shape)
    stars = np.array([[6.3, 4.7, 2.2], [7.0, 0.0, 4.5], [0.0, 0.0, 0.0], [13.99, 10.99, 8.99],
                      [-3.0, 5.5, 20.0]]) * cell
    out = {"density": dens, "x_H2": xh2, "x_CO": xco, "cell_size": np.array(cell),
           "stars": stars, "L_FUV": np.array(3.2e38)}
    for s, pos in enumerate(stars):
        for w, (a, b) in enumerate(((xh2, xco), (None, None))):
            res = compute_fuv_field_point_source(dens, pos, 3.2e38, cell, x_H2=a, x_CO=b)
            for k, v in zip(("G0", "A_V", "N_H", "N_H2", "N_CO"), res):
                out[f"{k}_{s}_{w}"] = v
    np.savez_compressed(os.path.join(HERE, "point_source.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference project checkout>")
    main(sys.argv[1])
