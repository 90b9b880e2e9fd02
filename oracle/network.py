"""CPU oracle for the full 31-species network (test infrastructure only).

Restates, in NumPy and in FP64:

* ``rhs``      ChemistrySolver._rhs (prism3d/chemistry/solver.py:69-143):
               rate coefficients per reaction type, the PAH charge pseudo-
               species, the 1e-30 floor, reactant/product accumulation in the
               order of build_pdr_network() (prism3d/chemistry/network.py:186-896).
* ``jacobian`` the analytic Jacobian of that RHS (not in the reference; the
               reference's BDF estimates it by finite differences).
* ``steady_state``  the steady state the GPU kernel computes: pseudo-transient
               continuation / Newton in relative variables on F(y) = 0 with the
               seven element totals of the initial state (H, C, O, S, Si, Fe,
               He) and charge neutrality as constraint rows.  The reference
               integrates the same RHS with BDF windows instead
               (solver.py:145-225); see ``tests/test_network.py`` for how the
               two are compared.
* ``correct_hp_electron``  solver.py:227-281.
* ``enforce_conservation`` solver.py:345-388.

Only tests, the smoke check and the CPU baseline of the benchmark use this
module.  It is pinned against ``tests/golden/network.npz`` (RHS of the
reference at 64 random states, including the temperature clamps and the dark
PAH branch).
"""
from __future__ import annotations

import json
import os
import re

import numpy as np

X_FLOOR = 1e-30
Y_TEST = 1e-25  # abundances at or below this are not tested for convergence
_HERE = os.path.dirname(os.path.abspath(__file__))
NETWORK_JSON = os.path.join(os.path.dirname(_HERE), "prism3d_gb300", "data", "pdr_network.json")

# reaction-type codes (also used by the GPU table)
TWO_BODY, PHOTO, CR, GRAIN_SURFACE = 0, 1, 2, 3
_TYPE = {"two_body": TWO_BODY, "recomb": TWO_BODY, "charge_exchange": TWO_BODY,
         "grain_recomb": TWO_BODY, "photodiss": PHOTO, "photoion": PHOTO,
         "cosmic_ray": CR, "cr_photo": CR, "grain_surface": GRAIN_SURFACE}
ELEMENTS = ("H", "C", "O", "S", "Si", "Fe", "He")


def _composition(name):
    """(element counts, charge) parsed from a species name ('H3O+' -> H3 O1, +1)."""
    if name == "e-":
        return {}, -1
    base = name.rstrip("+-")
    counts = {}
    for el, c in re.findall(r"([A-Z][a-z]?)(\d*)", base):
        counts[el] = counts.get(el, 0) + int(c or 1)
    return counts, name.count("+") - name.count("-")


def load(path=NETWORK_JSON):
    """Network table as arrays.  Species index -1 = untracked (its abundance
    is 0 in the reference's RHS), -2 = the PAH- pseudo-species."""
    with open(path) as f:
        d = json.load(f)
    sp = d["species"]
    idx = {s: i for i, s in enumerate(sp)}
    nr = len(d["reactions"])
    rtype = np.zeros(nr, np.int32)
    abc = np.zeros((nr, 3))
    reac = np.full((nr, 2), -1, np.int32)
    prod = np.full((nr, 4), -1, np.int32)
    shield = np.zeros(nr, np.int32)
    for j, r in enumerate(d["reactions"]):
        rtype[j] = _TYPE[r["type"]]
        abc[j] = (r["alpha"], r["beta"], r["gamma"])
        for m, s in enumerate(r["reactants"]):
            reac[j, m] = idx.get(s, -2 if s == "PAH-" else -1)
        for m, s in enumerate(r["products"]):
            prod[j, m] = idx.get(s, -1)
        shield[j] = {"H2_photodiss": 1, "CO_photodiss": 2}.get(r["name"], 0)
    elem = np.zeros((len(ELEMENTS), len(sp)))
    charge = np.zeros(len(sp))
    for i, s in enumerate(sp):
        c, q = _composition(s)
        charge[i] = q
        for el, k in c.items():
            elem[ELEMENTS.index(el), i] = k
    return {"species": sp, "idx": idx, "rtype": rtype, "abc": abc, "reac": reac,
            "prod": prod, "shield": shield, "elem": elem, "charge": charge,
            "pah_total": d["pah_total"], "C_total": d["gas_phase"]["C"],
            "O_total": d["gas_phase"]["O"], "gas_phase": d["gas_phase"],
            "names": [r["name"] for r in d["reactions"]]}


def _cond(cond):
    cond = np.atleast_2d(np.asarray(cond, float))
    return [cond[:, k] for k in range(7)]  # n_H, T, G0, A_V, zeta, fH2, fCO


def rate_coefficients(net, cond):
    """k[cell, reaction] as the reference computes it (solver.py:101-127).
    Bilinear rates are k x_A x_B n_H, the grain-surface rate k x_H n_H / 2;
    those factors are not folded in here."""
    n_h, t, g0, a_v, zeta, fh2, fco = _cond(cond)
    a, b, g = net["abc"].T
    tc = np.clip(t, 10.0, 41000.0)[:, None]
    k = np.zeros((len(t), len(a)))
    m = net["rtype"] == TWO_BODY
    k[:, m] = a[m] * (tc / 300.0) ** b[m] * np.exp(-g[m] / tc)
    m = net["rtype"] == PHOTO
    k[:, m] = a[m] * g0[:, None] * np.exp(-g[m] * a_v[:, None])
    k[:, net["shield"] == 1] *= fh2[:, None]
    k[:, net["shield"] == 2] *= fco[:, None]
    m = net["rtype"] == CR
    k[:, m] = a[m] * zeta[:, None]
    m = net["rtype"] == GRAIN_SURFACE
    k[:, m] = a[m] * (t[:, None] / 300.0) ** b[m]
    return k


def pah_minus(net, y_e, n_h, t, g0):
    """x(PAH-) and d x(PAH-) / d y_e (solver.py:76-88)."""
    n_e = np.maximum(y_e, 1e-10) * n_h
    lit = g0 > 0
    psi = np.where(lit, g0 * np.sqrt(t) / np.where(lit, n_e, 1.0), 0.0)
    fm = np.where(lit, np.maximum(500.0 / (psi + 500.0) * 0.5, 0.0), 0.4)
    dfm = np.where(lit & (y_e > 1e-10), 0.5 * 500.0 * psi / (psi + 500.0) ** 2
                   / np.maximum(y_e, 1e-10), 0.0)
    return net["pah_total"] * fm, net["pah_total"] * dfm


def _rates(net, k, yf, n_h, pahm):
    """Per-reaction rates with the floored abundances yf (cells x species)."""
    nr = len(net["rtype"])
    r = np.zeros((yf.shape[0], nr))
    for j in range(nr):
        t = net["rtype"][j]
        i0, i1 = net["reac"][j]
        if t == TWO_BODY:
            xa = yf[:, i0] if i0 >= 0 else (pahm if i0 == -2 else 0.0)
            xb = yf[:, i1] if i1 >= 0 else (pahm if i1 == -2 else 0.0)
            r[:, j] = k[:, j] * xa * xb * n_h
        elif t in (PHOTO, CR):
            r[:, j] = k[:, j] * (yf[:, i0] if i0 >= 0 else 0.0)
        else:
            r[:, j] = k[:, j] * yf[:, net["idx"]["H"]] * n_h * 0.5
    return r


def rhs(net, y, cond):
    """dy/dt of the reference's _rhs, for each row of y (cells x 31)."""
    y = np.atleast_2d(np.asarray(y, float))
    n_h, t, g0 = _cond(cond)[:3]
    yf = np.maximum(y, X_FLOOR)
    pahm, _ = pah_minus(net, yf[:, 0], n_h, t, g0)
    r = _rates(net, rate_coefficients(net, cond), yf, n_h, pahm)
    f = np.zeros_like(yf)
    for j in range(r.shape[1]):
        for i in net["reac"][j]:
            if i >= 0:
                f[:, i] -= r[:, j]
        for i in net["prod"][j]:
            if i >= 0:
                f[:, i] += r[:, j]
    return f


def rhs_scale(net, y, cond):
    """Sum over reactions of |stoichiometry x rate| per species (the size of
    its production plus destruction); the residual tolerance is relative to it."""
    y = np.atleast_2d(np.asarray(y, float))
    n_h, t, g0 = _cond(cond)[:3]
    yf = np.maximum(y, X_FLOOR)
    pahm, _ = pah_minus(net, yf[:, 0], n_h, t, g0)
    r = _rates(net, rate_coefficients(net, cond), yf, n_h, pahm)
    s = np.zeros_like(yf)
    for j in range(r.shape[1]):
        for i in list(net["reac"][j]) + list(net["prod"][j]):
            if i >= 0:
                s[:, i] += r[:, j]
    return s


def jacobian(net, y, cond, k=None):
    """d rhs / d y (cells x 31 x 31), taking d max(y, floor)/dy = 1."""
    y = np.atleast_2d(np.asarray(y, float))
    n_h, t, g0 = _cond(cond)[:3]
    if k is None:
        k = rate_coefficients(net, cond)
    yf = np.maximum(y, X_FLOOR)
    pahm, dpahm = pah_minus(net, yf[:, 0], n_h, t, g0)
    nc, ns = yf.shape
    J = np.zeros((nc, ns, ns))
    h = net["idx"]["H"]
    for j in range(k.shape[1]):
        tp = net["rtype"][j]
        i0, i1 = net["reac"][j]
        parts = []  # (column, d rate / d y_column)
        if tp == TWO_BODY:
            def val(i):
                return yf[:, i] if i >= 0 else (pahm if i == -2 else np.zeros(nc))
            if i0 >= 0:
                parts.append((i0, k[:, j] * val(i1) * n_h))
            if i1 >= 0:
                parts.append((i1, k[:, j] * val(i0) * n_h))
            if -2 in (i0, i1):
                other = i1 if i0 == -2 else i0
                parts.append((0, k[:, j] * val(other) * dpahm * n_h))
        elif tp in (PHOTO, CR):
            if i0 >= 0:
                parts.append((i0, k[:, j]))
        else:
            parts.append((h, k[:, j] * n_h * 0.5))
        for c, d in parts:
            for i in net["reac"][j]:
                if i >= 0:
                    J[:, i, c] -= d
            for i in net["prod"][j]:
                if i >= 0:
                    J[:, i, c] += d
    return J


# ---------------------------------------------------------------------------
# steady state
# ---------------------------------------------------------------------------
# constraint rows: the equation of one species of each element (a species
# made of that element alone, the most abundant one) is replaced by the
# element total; the electron equation by charge neutrality.
_PIVOTS = {"H": ("H", "H2", "H+", "H-", "H2+", "H3+"), "C": ("C+", "C"), "O": ("O", "O+"),
           "S": ("S", "S+"), "Si": ("Si", "Si+"), "Fe": ("Fe", "Fe+"), "He": ("He", "He+")}


def cation_mask(net):
    return net["charge"] > 0


def _system(net, y, cond, k, tot, inv_dt):
    """Relative-variable Newton/PTC system A w = d for every cell.

    ODE rows r: (inv_dt - J) scaled by y; element rows: sum_i c_i y_i w_i =
    total - sum_i c_i y_i; electron row: sum_cations y w - y_e w_e =
    y_e - sum_cations.  Rows are equilibrated by their largest entry."""
    nc, ns = y.shape
    f = rhs(net, y, cond)
    sc = rhs_scale(net, y, cond)
    J = jacobian(net, y, cond, k)
    A = -J.copy()
    A[:, np.arange(ns), np.arange(ns)] += inv_dt if np.ndim(inv_dt) == 2 else inv_dt[:, None]
    d = f.copy()
    ode = np.ones((nc, ns), bool)
    for e, el in enumerate(ELEMENTS):
        piv = [net["idx"][s] for s in _PIVOTS[el]]
        p = np.array(piv)[np.argmax(y[:, piv] * net["elem"][e, piv], axis=1)]
        rows = np.arange(nc)
        A[rows, p, :] = net["elem"][e][None, :]
        d[rows, p] = tot[:, e] - y @ net["elem"][e]
        ode[rows, p] = False
    cat = cation_mask(net).astype(float)
    A[:, 0, :] = cat[None, :]
    A[:, 0, 0] = -1.0
    d[:, 0] = y[:, 0] - y @ cat
    ode[:, 0] = False
    A = A * y[:, None, :]
    s = np.max(np.abs(A), axis=2)
    s[s == 0] = 1.0
    return A / s[:, :, None], d / s, f, sc, ode


def _solve(A, d):
    """Batched solve; a singular or non-finite system gives a NaN solution."""
    try:
        return np.linalg.solve(A, d[:, :, None])[:, :, 0]
    except np.linalg.LinAlgError:
        w = np.full(d.shape, np.nan)
        for c in range(d.shape[0]):
            try:
                w[c] = np.linalg.solve(A[c], d[c])
            except np.linalg.LinAlgError:
                pass
        return w


def element_totals(net, y):
    return np.maximum(np.atleast_2d(y), X_FLOOR) @ net["elem"].T


def steady_state(net, y0, cond, rtol=1e-8, max_iter=300, growth=2.0):
    """Constrained steady state of the RHS for each cell.

    Pseudo-transient continuation: the first step is pure Newton; a step
    that would make an abundance above 1e-25 non-positive is rejected (one
    at or below it goes to the floor instead) and repeated with
    1/dt = max|J_ii| / 10, which then shrinks by ``growth`` per accepted step
    (x4 on each rejection).  Abundances are floored at 1e-30 after a step.
    Converged when, for every species above 1e-25, the relative change is
    <= rtol and (ODE rows) the residual is <= rtol of that species'
    production plus destruction.
    Returns (y, status: 0 converged / 1 not, iterations)."""
    y = np.maximum(np.atleast_2d(np.asarray(y0, float)).copy(), X_FLOOR)
    cond = np.atleast_2d(np.asarray(cond, float))
    nc = y.shape[0]
    k = rate_coefficients(net, cond)
    tot = element_totals(net, y)
    inv_dt = np.zeros(nc)
    done = np.zeros(nc, bool)
    iters = np.zeros(nc, np.int64)
    for _ in range(max_iter):
        act = ~done
        if not act.any():
            break
        ia = np.nonzero(act)[0]
        A, d, f, sc, ode = _system(net, y[ia], cond[ia], k[ia], tot[ia], inv_dt[ia])
        w = _solve(A, d)
        # a step that would make an abundance above Y_TEST non-positive is
        # rejected; smaller ones go to the floor
        yy = y[ia]
        ok = np.all(np.isfinite(w), axis=1) & np.all((w > -1.0) | (yy <= Y_TEST), axis=1)
        # convergence of the state before the step
        res_ok = np.all(~ode | (np.abs(f) <= rtol * sc) | (yy <= Y_TEST), axis=1)
        step_ok = np.all((np.abs(w) <= rtol) | (yy <= Y_TEST), axis=1)
        iters[ia] += 1
        # rejected steps: grow the pseudo time-step weight
        jd = np.abs(np.diagonal(jacobian(net, yy, cond[ia], k[ia]), axis1=1, axis2=2))
        lam = np.max(jd, axis=1)
        bad = ~ok
        inv_dt[ia[bad]] = np.where(inv_dt[ia[bad]] == 0.0, lam[bad] / 10.0 + 1e-30,
                                   inv_dt[ia[bad]] * 4.0)
        good = ia[ok]
        y[good] = np.maximum(yy[ok] * (1.0 + np.maximum(w[ok], -1.0)), X_FLOOR)
        conv = ok & res_ok & step_ok
        done[ia[conv]] = True
        inv_dt[good] /= growth
    status = np.where(done, 0, 1).astype(np.int32)
    return y, status, iters


# ---------------------------------------------------------------------------
# post-processing of solve_steady_state (solver.py:220-225)
# ---------------------------------------------------------------------------
def correct_hp_electron(net, y, n_h, t, zeta):
    """solver.py:227-281, per cell."""
    i = net["idx"]
    y = np.array(y, float, copy=True)
    for c in range(y.shape[0]):
        x_h, x_cp = y[c, i["H"]], y[c, i["C+"]]
        r_form = zeta[c] * 0.46 * x_h
        tc = max(t[c], 10.0)
        alpha = 2.753e-14 * (tc / 300.0) ** (-0.745) + 1.0e-14 * np.sqrt(tc / 100.0)
        a = alpha * n_h[c]
        b = alpha * n_h[c] * x_cp
        cc = -r_form
        if a > 0:
            disc = b ** 2 - 4 * a * cc
            if disc >= 0:
                xhp = max((-b + np.sqrt(disc)) / (2 * a), X_FLOOR)
                if x_cp < 1e-6:
                    y[c, i["H+"]] = xhp
                    n_pos = 0.0
                    for s in ["H+", "C+", "H3+", "HCO+", "S+", "Si+", "Fe+", "O+", "H2+",
                              "OH+", "H2O+", "H3O+", "CH+", "CH2+", "CO+", "He+"]:
                        n_pos += y[c, i[s]]
                    y[c, i["e-"]] = max(n_pos, X_FLOOR)
    return y


def enforce_conservation(net, y):
    """solver.py:345-388, per cell."""
    i = net["idx"]
    y = np.array(y, float, copy=True)
    for c in range(y.shape[0]):
        v = y[c]
        h_major = v[i["H"]] + 2 * v[i["H2"]]
        h_minor = 0.0
        for s, m in [("H+", 1), ("H-", 1), ("H2+", 2), ("H3+", 3), ("OH", 1), ("OH+", 1),
                     ("H2O", 2), ("H2O+", 2), ("H3O+", 3), ("CH", 1), ("CH+", 1), ("HCO+", 1)]:
            h_minor += v[i[s]] * m
        if h_major > 0:
            sc = np.clip(max(1.0 - h_minor, 0.9) / h_major, 0.8, 1.2)
            v[i["H"]] *= sc
            v[i["H2"]] *= sc
        c_tot = net["C_total"]
        c_major = v[i["C+"]] + v[i["C"]] + v[i["CO"]]
        c_minor = 0.0
        for s in ["CH", "CH+", "CH2+", "CO+", "HCO+"]:
            c_minor += v[i[s]]
        if c_major > 0:
            sc = np.clip(max(c_tot - c_minor, c_tot * 0.9) / c_major, 0.8, 1.2)
            v[i["C+"]] *= sc
            v[i["C"]] *= sc
            v[i["CO"]] *= sc
        o_mol = (v[i["CO"]] + v[i["OH"]] + v[i["H2O"]] + v[i["O+"]] + v[i["OH+"]]
                 + v[i["H2O+"]] + v[i["H3O+"]] + v[i["CO+"]] + v[i["HCO+"]])
        o_mol += 2 * v[i["O2"]]
        v[i["O"]] = max(net["O_total"] - o_mol, X_FLOOR)
        n_pos = 0.0
        for s in ["H+", "C+", "S+", "Si+", "Fe+", "O+", "H2+", "H3+", "OH+", "H2O+", "H3O+",
                  "CH+", "CH2+", "CO+", "HCO+", "He+"]:
            n_pos += v[i[s]]
        v[i["e-"]] = max(n_pos, X_FLOOR)
        y[c] = np.maximum(v, X_FLOOR)
    return y


def solve_steady_state(net, y0, cond, rtol=1e-8, max_iter=300, post=True):
    """Steady state followed by the reference's two corrections."""
    cond = np.atleast_2d(np.asarray(cond, float))
    y, st, it = steady_state(net, y0, cond, rtol, max_iter)
    if post:
        y = correct_hp_electron(net, y, cond[:, 0], cond[:, 1], cond[:, 4])
        y = enforce_conservation(net, y)
    return y, st, it
