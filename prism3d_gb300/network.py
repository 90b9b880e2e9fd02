"""Full chemical network on the GB300: the GPU counterpart of
``prism3d.chemistry.solver.ChemistrySolver`` (prism3d/chemistry/solver.py).

The reaction table is data (``prism3d_gb300/data/pdr_network.json``, the 75
reactions of build_pdr_network(), prism3d/chemistry/network.py:186-896, and
the 31 tracked species of solver.py:28-36).  ``ChemistrySolverGPU`` keeps the
reference's method names and arguments:

    _rhs(t, y, n_H, T, G0, A_V, zeta_CR, f_shield_H2, f_shield_CO)
    solve_steady_state(n_H, T, G0, A_V, zeta_CR, x_init=None,
                       f_shield_H2=1.0, f_shield_CO=1.0, ...) -> (dict, converged)
    _default_initial(G0, A_V), _dict_to_array, _abundances_to_dict

and adds the batched forms the device is built for: ``rhs_batch`` and
``solve_steady_state_batch`` over many cells at once (NumPy arrays staged
through host memory, or float64 CUDA tensors used in place).

The steady state is the constrained root of the RHS (element totals of the
initial state, charge neutrality), found by Newton / pseudo-transient
continuation on the device; the reference reaches an approximation of it by
integrating with SciPy BDF to t_max (solver.py:182-215).  Both then apply the
same H+/e- correction and conservation fix-up.
"""
from __future__ import annotations

import ctypes
import json
import os
import re

import numpy as np

from . import _lib as L

NETWORK_JSON = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                            "pdr_network.json")
X_FLOOR = 1e-30
ELEMENTS = ("H", "C", "O", "S", "Si", "Fe", "He")
REFERENCE_SPECIES = (
    "e-", "H", "H2", "H+", "H-", "H2+", "H3+", "C+", "C", "CO", "CH", "CH+", "CH2+", "O", "O+",
    "OH", "OH+", "H2O", "H2O+", "H3O+", "O2", "CO+", "HCO+", "S", "S+", "Si", "Si+", "Fe", "Fe+",
    "He", "He+")
_RX = {"two_body": 0, "recomb": 0, "charge_exchange": 0, "grain_recomb": 0, "photodiss": 1,
       "photoion": 1, "cosmic_ray": 2, "cr_photo": 2, "grain_surface": 3}
_SHIELD = {"H2_photodiss": 1, "CO_photodiss": 2}


def composition(name):
    """(element counts, charge) of a species name: 'H3O+' -> {H: 3, O: 1}, +1."""
    if name == "e-":
        return {}, -1
    counts = {}
    for el, c in re.findall(r"([A-Z][a-z]?)(\d*)", name.rstrip("+-")):
        counts[el] = counts.get(el, 0) + int(c or 1)
    return counts, name.count("+") - name.count("-")


class ChemistrySolverGPU:
    """Device-resident network; one instance holds one compiled table."""

    def __init__(self, path=NETWORK_JSON):
        with open(path) as f:
            d = json.load(f)
        self.tracked_species = list(d["species"])
        self.n_tracked = len(self.tracked_species)
        self.idx = {s: i for i, s in enumerate(self.tracked_species)}
        self.reactions = d["reactions"]
        self.x_pah_total = float(d["pah_total"])
        self.gas_phase = {k: float(v) for k, v in d["gas_phase"].items()}
        self.c_total = self.gas_phase["C"]
        self.o_total = self.gas_phase["O"]
        nr = len(self.reactions)
        rtype = np.array([_RX[r["type"]] for r in self.reactions], np.int32)
        abc = np.array([[r["alpha"], r["beta"], r["gamma"]] for r in self.reactions], float)
        reac = np.full((nr, 2), -1, np.int32)
        prod = np.full((nr, 4), -1, np.int32)
        for j, r in enumerate(self.reactions):
            if len(r["reactants"]) > 2 or len(r["products"]) > 4:
                raise ValueError(f"reaction {r['name']}: too many reactants or products")
            for m, s in enumerate(r["reactants"]):
                reac[j, m] = self.idx.get(s, -2 if s == "PAH-" else -1)
            for m, s in enumerate(r["products"]):
                prod[j, m] = self.idx.get(s, -1)
        shield = np.array([_SHIELD.get(r["name"], 0) for r in self.reactions], np.int32)
        elem = np.zeros((len(ELEMENTS), self.n_tracked))
        charge = np.zeros(self.n_tracked, np.int32)
        for i, s in enumerate(self.tracked_species):
            c, q = composition(s)
            charge[i] = q
            for el, k in c.items():
                elem[ELEMENTS.index(el), i] = k
        self.element_counts = elem
        ref = int(tuple(self.tracked_species) == REFERENCE_SPECIES)
        a, b, g = (np.ascontiguousarray(abc[:, k]) for k in range(3))
        h = ctypes.c_void_p()
        L.call("p3d_network_create", ctypes.byref(h), self.n_tracked, nr, L.iptr(rtype),
               L.dptr(a), L.dptr(b), L.dptr(g), L.iptr(reac.ravel()), L.iptr(prod.ravel()),
               L.iptr(shield), len(ELEMENTS), L.dptr(elem.ravel()), L.iptr(charge),
               self.idx["e-"], self.x_pah_total, ref, self.c_total, self.o_total)
        self._h = h
        self.reference_layout = bool(ref)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            L.lib.p3d_network_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- helpers
    def _abundances_to_dict(self, x_arr):
        """solver.py:62-64."""
        return {self.tracked_species[i]: max(x_arr[i], X_FLOOR) for i in range(self.n_tracked)}

    def _dict_to_array(self, x_dict):
        """solver.py:66-67."""
        return np.array([x_dict.get(s, X_FLOOR) for s in self.tracked_species])

    def _default_initial(self, G0, A_V):
        """Smooth tanh initial abundances (solver.py:297-343)."""
        x = {}
        gp = self.gas_phase
        x_c, x_o, x_he = gp["C"], gp["O"], gp["He"]
        f_h2 = 0.5 * (1.0 + np.tanh((A_V - 1.5) / 0.5))
        f_co = 0.5 * (1.0 + np.tanh((A_V - 3.0) / 0.8))
        x["H"] = max(1.0 - f_h2, 0.003)
        x["H2"] = f_h2 * 0.5
        x["C+"] = x_c * (1.0 - f_co)
        x["CO"] = x_c * f_co * 0.95
        x["C"] = x_c * f_co * 0.05
        x["O"] = max(x_o - x["CO"], 1e-10)
        for ion, neut, tot in (("S+", "S", gp["S"]), ("Si+", "Si", gp["Si"]),
                               ("Fe+", "Fe", gp["Fe"])):
            f = max(0.01, 1.0 - A_V / 3.0) if A_V < 3 else 0.01
            x[ion] = tot * f
            x[neut] = tot * (1 - f)
        x["H+"] = 1e-6 if A_V < 2 else 1e-7
        x["e-"] = max(x.get("C+", 0) + x.get("S+", 0) + x.get("Si+", 0) + x.get("Fe+", 0)
                      + x.get("H+", 0), 1e-7)
        x["H-"] = 1e-14
        x["H2+"] = 1e-13
        x["H3+"] = 5e-10 if A_V > 2 else 1e-12
        x["OH"] = 1e-7 if A_V > 2 else 1e-9
        x["OH+"] = 1e-13
        x["H2O"] = 1e-7 if A_V > 3 else 1e-9
        x["H2O+"] = 1e-14
        x["H3O+"] = 1e-13
        x["O2"] = 1e-8 if A_V > 3 else 1e-12
        x["CH"] = 1e-10
        x["CH+"] = 1e-13
        x["CH2+"] = 1e-14
        x["CO+"] = 1e-15
        x["HCO+"] = 1e-9 if A_V > 2 else 1e-12
        x["O+"] = 1e-13
        x["He"] = x_he
        x["He+"] = 1e-13
        return x

    def default_initial_batch(self, G0, A_V):
        """_default_initial for arrays of G0 and A_V: (n, 31) abundances."""
        G0 = np.asarray(G0, float)
        A_V = np.asarray(A_V, float)
        i = self.idx
        gp = self.gas_phase
        x = np.full((A_V.size, self.n_tracked), X_FLOOR)
        f_h2 = 0.5 * (1.0 + np.tanh((A_V - 1.5) / 0.5))
        f_co = 0.5 * (1.0 + np.tanh((A_V - 3.0) / 0.8))
        x[:, i["H"]] = np.maximum(1.0 - f_h2, 0.003)
        x[:, i["H2"]] = f_h2 * 0.5
        x[:, i["C+"]] = gp["C"] * (1.0 - f_co)
        x[:, i["CO"]] = gp["C"] * f_co * 0.95
        x[:, i["C"]] = gp["C"] * f_co * 0.05
        x[:, i["O"]] = np.maximum(gp["O"] - x[:, i["CO"]], 1e-10)
        f = np.where(A_V < 3, np.maximum(0.01, 1.0 - A_V / 3.0), 0.01)
        for ion, neut in (("S+", "S"), ("Si+", "Si"), ("Fe+", "Fe")):
            x[:, i[ion]] = gp[neut] * f
            x[:, i[neut]] = gp[neut] * (1 - f)
        x[:, i["H+"]] = np.where(A_V < 2, 1e-6, 1e-7)
        x[:, i["e-"]] = np.maximum(x[:, i["C+"]] + x[:, i["S+"]] + x[:, i["Si+"]] +
                                   x[:, i["Fe+"]] + x[:, i["H+"]], 1e-7)
        for s, v in (("H-", 1e-14), ("H2+", 1e-13), ("OH+", 1e-13), ("H2O+", 1e-14),
                     ("H3O+", 1e-13), ("CH", 1e-10), ("CH+", 1e-13), ("CH2+", 1e-14),
                     ("CO+", 1e-15), ("O+", 1e-13), ("He", gp["He"]), ("He+", 1e-13)):
            x[:, i[s]] = v
        x[:, i["H3+"]] = np.where(A_V > 2, 5e-10, 1e-12)
        x[:, i["OH"]] = np.where(A_V > 2, 1e-7, 1e-9)
        x[:, i["H2O"]] = np.where(A_V > 3, 1e-7, 1e-9)
        x[:, i["O2"]] = np.where(A_V > 3, 1e-8, 1e-12)
        x[:, i["HCO+"]] = np.where(A_V > 2, 1e-9, 1e-12)
        return x

    def _check(self, name, a, shape):
        if _is_torch(a):
            import torch
            if a.dtype != torch.float64 or not a.is_cuda or not a.is_contiguous():
                raise TypeError(f"{name}: expected a contiguous float64 CUDA tensor")
        elif not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
            raise TypeError(f"{name}: expected a C-contiguous float64 numpy array")
        if tuple(a.shape) != shape:
            raise ValueError(f"{name}: shape {tuple(a.shape)} != {shape}")

    # ------------------------------------------------------------------- RHS
    def rhs_batch(self, y, cond):
        """dy/dt for n states: y (n, 31), cond (n, 7) = n_H, T, G0, A_V,
        zeta_CR, f_shield_H2, f_shield_CO.  Returns an array like y."""
        n = y.shape[0]
        self._check("y", y, (n, self.n_tracked))
        self._check("cond", cond, (n, 7))
        if _is_torch(y):
            import torch
            out = torch.empty_like(y)
            L.call("p3d_network_rhs_dev", self._h, n, L.dptr(cond), L.dptr(y), L.dptr(out),
                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
            return out
        out = np.empty_like(y)
        L.call("p3d_network_rhs", self._h, n, L.dptr(cond), L.dptr(y), L.dptr(out))
        return out

    def _rhs(self, t, y, n_H, T, G0, A_V, zeta_CR, f_shield_H2, f_shield_CO):
        """solver.py:69-143 for one state (t unused, as in the reference)."""
        cond = np.array([[n_H, T, G0, A_V, zeta_CR, f_shield_H2, f_shield_CO]], float)
        return self.rhs_batch(np.ascontiguousarray(np.asarray(y, float)[None, :]), cond)[0]

    # ---------------------------------------------------------- steady state
    def solve_steady_state_batch(self, cond, x, mixed=True, post=True, rtol=1e-8,
                                 max_iter=300, return_iters=False):
        """Steady state of n cells.  x (n, 31) holds the initial abundances and
        receives the result (in place); cond (n, 7) as in rhs_batch.  Returns
        the per-cell status (0 = converged) [and Newton iterations]."""
        n = x.shape[0]
        self._check("x", x, (n, self.n_tracked))
        self._check("cond", cond, (n, 7))
        if _is_torch(x):
            import torch
            st = torch.empty(n, dtype=torch.int32, device=x.device)
            it = torch.empty(n, dtype=torch.int32, device=x.device)
            L.call("p3d_network_steady_dev", self._h, n, L.dptr(cond), L.dptr(x), int(mixed),
                   int(post), int(max_iter), float(rtol), L.iptr(st), L.iptr(it),
                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        else:
            st = np.empty(n, np.int32)
            it = np.empty(n, np.int32)
            rc = L.lib.p3d_network_steady(self._h, n, L.dptr(cond), L.dptr(x), int(mixed),
                                          int(post), int(max_iter), float(rtol), L.iptr(st),
                                          L.iptr(it))
            if rc not in (0, -5):  # P3D_ECONVERGE: status says which cells
                L.check("p3d_network_steady", rc)
        return (st, it) if return_iters else st

    def solve_steady_state(self, n_H, T, G0, A_V, zeta_CR, x_init=None, f_shield_H2=1.0,
                           f_shield_CO=1.0, t_max=None, rtol=1e-3, atol=1e-20, fast=False):
        """One cell, the reference's signature (solver.py:145-147); t_max, rtol,
        atol and fast belong to its time integrator and are accepted for
        compatibility.  Returns (abundance dict, converged)."""
        if x_init is None:
            x_init = self._default_initial(G0, A_V)
        x = self._dict_to_array(x_init)[None, :].copy()
        cond = np.array([[n_H, T, G0, A_V, zeta_CR, f_shield_H2, f_shield_CO]], float)
        st = self.solve_steady_state_batch(cond, x, mixed=False, post=True)
        return self._abundances_to_dict(x[0]), bool(st[0] == 0)


def _is_torch(a):
    return hasattr(a, "is_cuda") and hasattr(a, "data_ptr")



def _main():
    """python -m prism3d_gb300.network [--cells N] [--fp64]: solve a seeded
    batch (prism3d_gb300/fields.py:network_cells) on the current GPU and
    print cells/s, Newton iterations and the unconverged fraction."""
    import argparse
    import time

    from . import fields
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=1 << 16)
    ap.add_argument("--fp64", action="store_true", help="FP64 factorisation throughout")
    ap.add_argument("--seed", type=int, default=11)
    a = ap.parse_args()
    net = ChemistrySolverGPU()
    cond = fields.network_cells(a.cells, seed=a.seed)
    x = net.default_initial_batch(cond[:, 2], cond[:, 3])
    t0 = time.perf_counter()
    st, it = net.solve_steady_state_batch(cond, x, mixed=not a.fp64, post=True, return_iters=True)
    t = time.perf_counter() - t0
    print(f"{a.cells} cells  {a.cells / t:.4g} cells/s (host buffers)  Newton iterations "
          f"mean {it.mean():.1f}  unconverged {(st != 0).mean():.4f}")
    net.close()


if __name__ == "__main__":
    _main()
