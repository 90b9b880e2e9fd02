"""Golden total heating and cooling rates from the reference.

    python tests/golden/make_heating.py /path/to/prism3d/checkout

Calls PDRSolver3D._total_heating_vec and _total_cooling_vec
(prism3d/solver_3d.py:898-1050, the diagnostics Gamma and Lambda that
solve() stores and save() writes) on a stand-in object carrying seeded
per-cell states: n_H, G0, A_V, zeta, the seven abundances, T_dust, Gamma_PE,
R_H2 and f_sh_H2, at temperatures spanning 10 K - 1e5 K with every branch
(T_dust above and below T, H2 above and below 0.5, T across 100 K and
3000 K, the CO ladder's break) and writes tests/golden/heating.npz.
Nothing at test or run time reads the reference checkout.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.path.insert(0, ref_root)
    from prism3d.solver_3d import PDRSolver3D
    rng = np.random.default_rng(43)
    n = 2000
    s = types.SimpleNamespace()
    s.density = 10 ** rng.uniform(1, 7, n)
    s.G0 = 10 ** rng.uniform(-2, 5, n)
    s.A_V = rng.uniform(0, 20, n)
    s.zeta_CR = 10 ** rng.uniform(-17, -15, n)
    s.x_H2 = 10 ** rng.uniform(-7, np.log10(0.5), n)
    s.x_HI = 1.0 - 2.0 * s.x_H2
    x_c_total = 1.076e-4
    fco = rng.uniform(0, 1, n)
    fcp = rng.uniform(0, 1, n) * (1 - fco)
    s.x_CO = x_c_total * fco
    s.x_Cp = x_c_total * fcp
    s.x_C = x_c_total - s.x_CO - s.x_Cp
    s.x_O = np.maximum(2.94e-4 - s.x_CO, 1e-30)
    s.x_e = s.x_Cp + 1e-10
    s.T_dust = rng.uniform(5, 200, n)
    s.Gamma_PE = 10 ** rng.uniform(-30, -18, n)
    s._R_H2 = 10 ** rng.uniform(-18, -16, n)
    f_sh = 10 ** rng.uniform(-8, 0, n)
    T = 10 ** rng.uniform(1, 5, n)
    # branch edges: 100 K and 3000 K from both sides, the CO break of J = 4,
    # T_dust = T, x_H2 = 0.5
    T[:8] = [100.0, 100.0 * (1 - 1e-12), 3000.0, 3000.0 * (1 - 1e-12), 11.06, 11.07, 40.0,
             1e5]
    s.T_dust[8] = T[8]
    s.x_H2[9], s.x_HI[9] = 0.5, 0.0
    inp = {k: np.array(getattr(s, k), copy=True) for k in
           ("density", "G0", "A_V", "zeta_CR", "x_HI", "x_H2", "x_Cp", "x_C", "x_CO", "x_O",
            "x_e", "T_dust", "Gamma_PE")}
    inp["R_H2"] = s._R_H2.copy()
    gamma = PDRSolver3D._total_heating_vec(s, T, f_sh)
    lam = PDRSolver3D._total_cooling_vec(s, T)
    np.savez_compressed(os.path.join(HERE, "heating.npz"), **inp, f_sh_H2=f_sh, T=T,
                        Gamma=gamma, Lambda=lam)
    print("wrote heating.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference project checkout>")
    main(sys.argv[1])
