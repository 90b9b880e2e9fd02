"""Export the reference's full PDR network and golden RHS vectors.

    python tests/golden/make_network.py /path/to/prism3d/checkout

Writes
  prism3d_gb300/data/pdr_network.json  the reaction table of
      build_pdr_network() (prism3d/chemistry/network.py:186-896) and the 31
      tracked species of ChemistrySolver (prism3d/chemistry/solver.py:28-36):
      per reaction its type, (alpha, beta, gamma), reactant and product
      names.  It is data -- the network the reference defines -- and the GPU
      kernels read it as such.
  tests/golden/network.npz  ChemistrySolver._rhs (solver.py:69-143) at seeded
      random abundance vectors and physical conditions, and a few
      solve_steady_state() results (BDF, solver.py:145-225).
Nothing at test or run time reads the reference checkout.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main(ref_root):
    sys.path.insert(0, ref_root)
    from prism3d.chemistry.solver import ChemistrySolver
    from prism3d.utils.constants import gas_phase_abundances
    cs = ChemistrySolver()
    rx = []
    for r in cs.network.reactions:
        rx.append({"name": r.name, "type": r.reaction_type, "alpha": r.alpha, "beta": r.beta,
                   "gamma": r.gamma, "reactants": list(r.reactants), "products": list(r.products)})
    net = {"species": list(cs.tracked_species), "reactions": rx,
           "pah_total": 1e-7, "x_floor": 1e-30,
           "gas_phase": {k: gas_phase_abundances[k] for k in ("H", "He", "C", "O", "S", "Si", "Fe")},
           "note": "reaction table of build_pdr_network() in the order ChemistrySolver._rhs "
                   "accumulates it (solver.py:45-60); PAH, PAH+, PAH- are pseudo-species "
                   "set from the PAH charge balance (solver.py:76-88)"}
    with open(os.path.join(ROOT, "prism3d_gb300", "data", "pdr_network.json"), "w") as f:
        json.dump(net, f, indent=1)
    rng = np.random.default_rng(77)
    n = 64
    ns = cs.n_tracked
    Y = 10 ** rng.uniform(-14, -3, (n, ns))
    Y[:, cs.idx["H"]] = rng.uniform(0.01, 1.0, n)
    Y[:, cs.idx["H2"]] = rng.uniform(0.0, 0.5, n)
    Y[:, cs.idx["He"]] = 0.0851
    cond = np.stack([10 ** rng.uniform(1, 6, n), 10 ** rng.uniform(1, 4.7, n),
                     10 ** rng.uniform(-2, 5, n), rng.uniform(0, 20, n),
                     10 ** rng.uniform(-17, -15, n), rng.uniform(0, 1, n), rng.uniform(0, 1, n)],
                    axis=1)
    cond[:4, 1] = [5.0, 10.0, 41000.0, 5e4]  # temperature clamps
    cond[4:6, 2] = [0.0, 1e-9]               # dark cells (PAH charge fallback)
    F = np.stack([cs._rhs(0.0, Y[i], *cond[i]) for i in range(n)])
    out = {"Y": Y, "cond": cond, "F": F}
    # a few BDF steady states of the reference (slow: 4 cells)
    ss_cond = np.array([[1e3, 100.0, 10.0, 0.5, 2e-16, 0.5, 0.9],
                        [1e4, 50.0, 1e3, 3.0, 2e-16, 1e-3, 1e-2],
                        [1e5, 30.0, 1e4, 10.0, 1e-16, 1e-6, 1e-5],
                        [3e3, 300.0, 1e2, 1.0, 2e-16, 0.1, 0.5]])
    X0, XS, CV = [], [], []
    for c in ss_cond:
        x0 = cs._default_initial(c[2], c[3])
        res, conv = cs.solve_steady_state(c[0], c[1], c[2], c[3], c[4], x_init=x0,
                                          f_shield_H2=c[5], f_shield_CO=c[6])
        X0.append(cs._dict_to_array(x0))
        XS.append(cs._dict_to_array(res))
        CV.append(conv)
    out.update(ss_cond=ss_cond, ss_x0=np.array(X0), ss_x=np.array(XS), ss_conv=np.array(CV))
    # the reference's two post-solve corrections on random states; the
    # first half with x(C+) < 1e-6 so that the H+/e- correction applies
    m = 48
    P = 10 ** rng.uniform(-14, -3, (m, ns))
    P[:, cs.idx["H"]] = rng.uniform(0.01, 1.0, m)
    P[:, cs.idx["H2"]] = rng.uniform(0.0, 0.5, m)
    P[: m // 2, cs.idx["C+"]] = 10 ** rng.uniform(-12, -6.5, m // 2)
    pc = np.stack([10 ** rng.uniform(1, 6, m), 10 ** rng.uniform(0.5, 4, m),
                   10 ** rng.uniform(-17, -15, m)], axis=1)
    PC = np.stack([cs._correct_Hp_electron(P[i].copy(), *pc[i]) for i in range(m)])
    PE = np.stack([cs._enforce_conservation(PC[i].copy(), pc[i, 0]) for i in range(m)])
    out.update(post_y=P, post_cond=pc, post_hp=PC, post_out=PE)
    # steady states of the reference RHS with the electron abundance held at
    # charge neutrality (x_e = sum of cations): SciPy BDF on the other 30
    # species, integrated until a further 3x in time changes no species above
    # 1e-20 by more than 1e-7
    from scipy.integrate import solve_ivp
    cat = [cs.idx[s] for s in cs.tracked_species if s.endswith("+")]
    keep = [i for i in range(ns) if i != cs.idx["e-"]]

    def full(z):
        y = np.empty(ns)
        y[keep] = z
        y[cs.idx["e-"]] = max(z[[keep.index(i) for i in cat]].sum(), 1e-30)
        return y

    nss_cond = np.concatenate([ss_cond, [[1e2, 500.0, 1e3, 0.1, 2e-16, 1.0, 1.0],
                                         [1e6, 20.0, 1e5, 15.0, 1e-16, 1e-8, 1e-7]]])
    NX0, NXS, NC = [], [], []
    for c in nss_cond:
        x0 = full(cs._dict_to_array(cs._default_initial(c[2], c[3]))[keep])
        z = x0[keep]
        t0, t1 = 0.0, 1e16
        start = time.time()

        def f(t, z):
            if time.time() - start > 300:
                raise TimeoutError
            return cs._rhs(t, full(z), *c)[keep]
        try:
            while True:
                sol = solve_ivp(f, (t0, t1), z, method="BDF", rtol=1e-9, atol=1e-28)
                assert sol.success
                zn = sol.y[:, -1]
                big = zn > 1e-20
                if t0 > 0 and np.max(np.abs(zn[big] - z[big]) / zn[big]) < 1e-7:
                    break
                assert t1 < 1e18, "no steady state reached"
                z, t0, t1 = zn, t1, 3 * t1
        except TimeoutError:
            print("skipped (integration too slow):", c)
            continue
        NX0.append(x0)
        NXS.append(full(zn))
        NC.append(c)
    out.update(neutral_cond=np.array(NC), neutral_x0=np.array(NX0), neutral_x=np.array(NXS))
    np.savez_compressed(os.path.join(HERE, "network.npz"), **out)
    print("wrote network table and golden vectors;", len(rx), "reactions,", ns, "species")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference project checkout>")
    main(sys.argv[1])
