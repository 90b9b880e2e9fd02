"""Golden column-density maps from the reference's observation pipeline.

    python tests/golden/make_maps.py /path/to/prism3d/checkout

Runs column_density_maps and integrate_column
(prism3d/observations/jwst_pipeline.py:109-180, shear :472-520) on seeded
random fields of a non-cubic grid for every LOS axis, edge-on and inclined,
and writes tests/golden/maps.npz.  Nothing at test or run time reads the
reference checkout.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.path.insert(0, ref_root)
    from prism3d.observations.jwst_pipeline import column_density_maps, integrate_column
    rng = np.random.default_rng(21)
    shape = (12, 10, 8)
    s = types.SimpleNamespace()
    s.density = 10 ** rng.uniform(2, 5, shape)
    s.x_H2 = rng.uniform(0, 0.5, shape)
    s.x_CO = 10 ** rng.uniform(-8, -4, shape)
    s.x_Cp = 10 ** rng.uniform(-8, -4, shape)
    s.x_e = 10 ** rng.uniform(-8, -3, shape)
    s.T_gas = rng.uniform(10, 1000, shape)
    s.cell_size = 1.5428e16
    out = {k: getattr(s, k) for k in ("density", "x_H2", "x_CO", "x_Cp", "x_e", "T_gas")}
    out["cell_size"] = np.array(s.cell_size)
    incs = (0.0, 4.0, -7.5)
    out["inclinations"] = np.array(incs)
    for los in range(3):
        out[f"int_T_{los}"] = integrate_column(s, "T_gas", los_axis=los)
        for j, inc in enumerate(incs):
            m = column_density_maps(s, los_axis=los, inclination_deg=inc)
            for k, v in m.items():
                out[f"{k}_{los}_{j}"] = v
    np.savez_compressed(os.path.join(HERE, "maps.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference project checkout>")
    main(sys.argv[1])
