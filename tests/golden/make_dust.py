"""Golden grain-state steps from the reference.

    python tests/golden/make_dust.py /path/to/prism3d/checkout

Calls PDRSolver3D._evolve_dust_state (prism3d/solver_3d.py:465-507) on a
stand-in object carrying seeded G0, density, f_nano and E_g (every branch:
G0 above / below 1 and 10, n_H above / below 1e4, clipping at both ends)
and writes tests/golden/dust.npz.  Nothing at test or run time reads the
reference checkout.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.path.insert(0, ref_root)
    from prism3d.solver_3d import PDRSolver3D
    rng = np.random.default_rng(41)
    n = 4000
    s = types.SimpleNamespace()
    s.G0 = 10 ** rng.uniform(-3, 5, n)
    s.density = 10 ** rng.uniform(-1, 7, n)
    s.f_nano = rng.uniform(0.0, 2.5, n)
    s.E_g = rng.uniform(0.0, 3.0, n)
    s.G0[:4] = [0.5, 0.5, 20.0, 1e-6]
    s.density[:4] = [2e4, 5e3, 1e6, 0.1]
    inp = {k: getattr(s, k).copy() for k in ("G0", "density", "f_nano", "E_g")}
    PDRSolver3D._evolve_dust_state(s)
    np.savez_compressed(os.path.join(HERE, "dust.npz"), **inp, f_nano_out=s.f_nano,
                        E_g_out=s.E_g)
    print("wrote dust.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference project checkout>")
    main(sys.argv[1])
