"""The steady driver's mixed thermal root, built for the host, against its
plain FP64 root on the oracle's thermal contexts (no GPU).

tests/host_root.cpp compiles prism3d_gb300/csrc/p3d_thermal_fast.cuh with
g++; the contexts are those of the oracle's steady method on a 24^3 cut of
the Orion-Bar-like slab (oracle.map_residual of its states after 5 and 6
outer iterations).  Checked: the mixed root's bracket decisions and polish
land on the plain root (cold start); a warm start with replayed decisions
returns a sign change of the net heating (or a root pinned at 10 K / 1e5 K,
which then costs one FP64 evaluation); the warm and cold roots agree; and
the oracle's whole steady method, run with the mixed root in place of its
plain one, reaches the plain fixed point to 1e-6 in every cell.  The device
build of the same source runs these paths in the -m gpu tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from hostbuild import ptr as _p
from hostbuild import root_lib

TOL = 1e-10  # the mixed path's settled root tolerance


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    return root_lib(tmp_path_factory.mktemp("hostroot"))


@pytest.fixture(scope="module")
def contexts():
    from prism3d_gb300 import fields
    from prism3d_gb300.core import directional_G0
    dens = fields.orion_bar_slab(24, seed=1)
    g0 = directional_G0(2.6e4, [-1.0, 0.0, 0.0], 2)
    keep = {}
    keys = ("x_HI", "x_H2", "x_Cp", "x_C", "x_CO", "x_O", "x_e", "T_gas")

    def cb(it, st):
        if it in (5, 6):
            keep[it] = {k: st[k].copy() for k in keys}
    O.steady_run(dens, g0, fields.CELL_CM, nside=2, zeta0=2e-16, T_init=100.0, max_outer=7,
                 tol=1e-300, w_chem=0.1, callback=cb)
    out = []
    for it in (5, 6):
        _, _, _, ctx = O.map_residual(keep[it], dens, g0, fields.CELL_CM, 2, 2e-16)
        out.append(np.ascontiguousarray(np.stack([np.ravel(c) for c in ctx], axis=1)))
    return out


def _mixed(L, ctx, t_warm, delta, node, margin, tol=TOL):
    n = ctx.shape[0]
    t = np.zeros(n)
    ev = np.zeros(n, np.int32)
    st = np.zeros(n, np.int32)
    L.hr_root_mixed(ctypes.c_long(n), _p(ctx), _p(np.ascontiguousarray(t_warm, dtype=np.float64)),
                    _p(np.ascontiguousarray(delta, dtype=np.float64)), _p(node), _p(margin),
                    ctypes.c_double(tol), _p(t), _p(ev), _p(st))
    return t, ev, st


def _plain(L, ctx):
    n = ctx.shape[0]
    t = np.zeros(n)
    ev = np.zeros(n, np.int32)
    st = np.zeros(n, np.int32)
    L.hr_root_plain(ctypes.c_long(n), _p(ctx), ctypes.c_double(1e-12), _p(t), _p(ev), _p(st))
    return t, ev, st


def _net(L, ctx, t):
    out = np.zeros(ctx.shape[0])
    L.hr_net64(ctypes.c_long(ctx.shape[0]), _p(ctx), _p(np.ascontiguousarray(t)), _p(out))
    return out


def test_cold_mixed_root_matches_plain(lib, contexts):
    ctx = contexts[1]
    n = ctx.shape[0]
    tp, _, sp = _plain(lib, ctx)
    node, margin = np.zeros(n, np.int32), np.zeros(n, np.float32)
    tm, ev, sm = _mixed(lib, ctx, np.zeros(n), np.full(n, np.inf), node, margin)
    assert sp.sum() == 0 and sm.sum() == 0
    rel = np.abs(tm - tp) / tp
    assert np.mean(rel <= 1e-6) >= 0.999, np.sort(rel)[-10:]
    # every full bisection left a node of the tree's last level
    assert np.all((node >= 1024) & (node < 2048))
    # FP64 work: a root within tol of a bracket end (pinned at 10 K, or on
    # the 100 K discontinuity, a node of the tree) costs two evaluations --
    # the Newton step that leaves the bracket and the end check -- instead
    # of a bisection creeping towards the end (~25)
    pinned = tm <= 10.0 * (1.0 + TOL)
    on_100 = np.abs(tm - 100.0) <= 100.0 * TOL
    assert pinned.any() and on_100.any()
    assert np.all(ev[pinned] <= 2), np.bincount(ev[pinned])
    assert np.mean(ev[on_100] <= 2) >= 0.99, np.bincount(ev[on_100])
    assert ev.mean() < 2.5, ev.mean()


def test_warm_root_is_a_sign_change_and_pinned_roots_cost_one_evaluation(lib, contexts):
    c5, c6 = contexts
    n = c5.shape[0]
    node, margin = np.zeros(n, np.int32), np.zeros(n, np.float32)
    t5, _, _ = _mixed(lib, c5, np.zeros(n), np.full(n, np.inf), node, margin)
    delta = np.max(np.abs(c6 - c5) / np.maximum(np.abs(c6), 1e-300), axis=1)
    tw, ev, st = _mixed(lib, c6, t5, delta, node, margin)
    assert st.sum() == 0
    lo_pin = tw <= 10.0 * (1.0 + 2 * TOL)
    hi_pin = tw >= 1e5 * (1.0 - 2 * TOL)
    inner = ~(lo_pin | hi_pin)
    assert lo_pin.any(), "the slab cut should hold cells at the 10 K floor"
    # pinned: the net heating keeps its sign at the root; one FP64 evaluation
    assert np.all(_net(lib, c6[lo_pin], tw[lo_pin]) <= 0.0)
    assert np.all(_net(lib, c6[hi_pin], tw[hi_pin]) > 0.0)
    warm_pinned = lo_pin & (t5 <= 10.0 * (1.0 + TOL))
    assert warm_pinned.any() and np.all(ev[warm_pinned] == 1), np.bincount(ev[warm_pinned])
    # elsewhere the root brackets a sign change within 1e-7 T
    fa = _net(lib, c6[inner], tw[inner] * (1.0 - 1e-7))
    fb = _net(lib, c6[inner], tw[inner] * (1.0 + 1e-7))
    assert np.all((fa > 0.0) & (fb <= 0.0))
    # warm and cold starts agree (a bracket holding two sign changes may let
    # them pick different ones: allowed for a handful of cells)
    nc, mc = np.zeros(n, np.int32), np.zeros(n, np.float32)
    tc, evc, _ = _mixed(lib, c6, np.zeros(n), np.full(n, np.inf), nc, mc)
    rel = np.abs(tw - tc) / tc
    assert np.mean(rel <= 1e-6) >= 0.99, np.sort(rel)[-10:]
    assert ev.mean() < 2.5 and ev.max() <= 32, (ev.mean(), ev.max())


def test_root_at_a_bracket_end_costs_one_end_check(lib, contexts):
    """A balance the outer iteration has pushed onto a node of the bisection
    tree: the root sits within tol above the node, the bracket's lower end
    (1000 K is the first decision).  Cells of this kind alternate between
    branches from one outer iteration to the next and make the slow tail of
    a solve; their Newton step from the bracket's middle lands just past the
    end.  Built here from the oracle's contexts whose plain root lies in
    [300, 3000] K by moving Gamma_fixed so that the root is 1000 (1 + 3e-11)
    K: the mixed root lands within tol of it with at most three FP64
    evaluations (the FP64 sign at the 1000 K node, the Newton step, the end
    check) where the bisection towards the end took ~20, cold and warm from
    the other branch (100 K) alike."""
    ctx = contexts[1]
    tp, _, _ = _plain(lib, ctx)
    sel = np.where((tp > 300.0) & (tp < 3000.0))[0][:256]
    assert sel.size >= 64
    c = ctx[sel].copy()
    t_root = 1000.0 * (1.0 + 3e-11)
    c[:, 0] -= _net(lib, c, np.full(sel.size, t_root))
    f_below = _net(lib, c, np.full(sel.size, 1000.0))
    f_above = _net(lib, c, np.full(sel.size, 1000.0 * (1.0 + 1e-10)))
    ok = (f_below > 0.0) & (f_above <= 0.0)  # the net heating falls through the root
    assert ok.mean() > 0.9
    c = np.ascontiguousarray(c[ok])
    n = c.shape[0]
    for t_warm in (np.zeros(n), np.full(n, 100.0)):
        node, margin = np.zeros(n, np.int32), np.zeros(n, np.float32)
        tm, ev, st = _mixed(lib, c, t_warm, np.full(n, np.inf), node, margin)
        assert st.sum() == 0
        assert np.all(np.abs(tm - t_root) <= TOL * t_root), np.abs(tm - t_root).max()
        assert ev.max() <= 3, np.bincount(ev)


def test_cooperative_net_heating_and_root(lib, contexts):
    """The thermal kernel's warp-cooperative FP64 net heating
    (net_heating_coop64: the 5 fine-structure lines and 40 CO levels as one
    table of two-level lines, coop_line) and the mixed root's lane-wise form
    (net_heating_mixed64_body: power laws as products of T^0.01)
    against the plain form (net_heating_fast64_body) on the oracle's contexts at 12 temperatures
    over 10 K - 1e5 K: equal to 1e-13 of the heating + cooling scale (the
    table's folded constants and the summation order differ); and the mixed
    root with it lands on the lane-wise root to 1e-9 (both to tol 1e-10)."""
    ctx = contexts[1]
    n = ctx.shape[0]
    rng = np.random.default_rng(7)
    for t0 in np.geomspace(10.0, 1e5, 12):
        t = np.ascontiguousarray(t0 * np.exp(rng.uniform(-0.05, 0.05, n)))
        a = _net(lib, ctx, t)
        b = np.zeros(n)
        lib.hr_net64_coop(ctypes.c_long(n), _p(ctx), _p(t), _p(b))
        m = np.zeros(n)
        lib.hr_net64_mixed(ctypes.c_long(n), _p(ctx), _p(t), _p(m))
        g, l = np.zeros(n), np.zeros(n)
        lib.hr_heating_cooling(ctypes.c_long(n), _p(ctx), _p(t), _p(g), _p(l))
        scale = np.abs(g) + np.abs(l)
        for other in (b, m):  # cooperative form; mixed form (power laws as products)
            assert np.all(np.abs(a - other) <= 1e-13 * scale), (t0, np.max(
                np.abs(a - other) / scale))
    tm, _, sm = _mixed(lib, ctx, np.zeros(n), np.full(n, np.inf), np.zeros(n, np.int32),
                       np.zeros(n, np.float32))
    tc = np.zeros(n)
    ev = np.zeros(n, np.int32)
    st = np.zeros(n, np.int32)
    lib.hr_root_mixed_coop(ctypes.c_long(n), _p(ctx), _p(np.zeros(n)), _p(np.full(n, np.inf)),
                           _p(np.zeros(n, np.int32)), _p(np.zeros(n, np.float32)),
                           ctypes.c_double(TOL), _p(tc), _p(ev), _p(st))
    assert sm.sum() == 0 and st.sum() == 0
    rel = np.abs(tc - tm) / tm
    assert np.mean(rel <= 1e-9) >= 0.999, np.sort(rel)[-5:]


@pytest.mark.parametrize("coop", [False, True])
def test_mixed_root_in_the_outer_loop_reaches_the_plain_fixed_point(lib, monkeypatch, coop):
    """The oracle's steady method on the 24^3 slab cut, once with its plain
    FP64 roots and once with the host-built mixed root in their place (warm
    starts, replayed decisions and the one-evaluation pinned roots across
    outer iterations, tol 1e-10; coop: every FP64 evaluation in the
    cooperative form the thermal kernel uses for short worklists): same
    iteration count, and every cell's T and abundances within 1e-6 of the
    plain fixed point.  (The root before its Newton slope was confined to
    T's continuous piece left 20 cells of this grid 1e-6 to 9e-3 away.)"""
    from prism3d_gb300 import fields
    from prism3d_gb300.core import directional_G0
    dens = fields.orion_bar_slab(24, seed=1)
    g0 = directional_G0(2.6e4, [-1.0, 0.0, 0.0], 2)
    keys = ("T_gas", "x_HI", "x_H2", "x_Cp", "x_C", "x_CO")

    def solve():
        st, hist = O.steady_run(dens, g0, fields.CELL_CM, nside=2, zeta0=2e-16, T_init=100.0,
                                max_outer=600, tol=1e-8, w_chem=0.1)
        return {k: st[k].ravel().copy() for k in keys}, len(hist), hist[-1]["dmax"]

    plain, it_p, d_p = solve()
    state = {}

    def mixed_root(ctx10, *args, **kw):
        c = np.ascontiguousarray(np.stack([np.ravel(np.asarray(x, dtype=np.float64))
                                           for x in ctx10], axis=1))
        n = c.shape[0]
        if not state:
            state.update(t=np.zeros(n), node=np.zeros(n, np.int32),
                         margin=np.zeros(n, np.float32), ctx=None)
        delta = (np.full(n, np.inf) if state["ctx"] is None else
                 np.max(np.abs(c - state["ctx"]) / np.maximum(np.abs(c), 1e-300), axis=1))
        if coop:
            t = np.zeros(n)
            ev = np.zeros(n, np.int32)
            st = np.zeros(n, np.int32)
            lib.hr_root_mixed_coop(ctypes.c_long(n), _p(c), _p(state["t"]), _p(delta),
                                   _p(state["node"]), _p(state["margin"]), ctypes.c_double(TOL),
                                   _p(t), _p(ev), _p(st))
        else:
            t, ev, st = _mixed(lib, c, state["t"], delta, state["node"], state["margin"])
        state["t"], state["ctx"] = t, c
        return t, ev.astype(np.int64), st

    monkeypatch.setattr(O, "thermal_root", mixed_root)
    mixed, it_m, d_m = solve()
    assert d_p < 1e-8 and d_m < 1e-8
    assert it_m == it_p
    for k in keys:
        m = np.abs(plain[k]) > 1e-20
        rel = np.abs(mixed[k] - plain[k])[m] / np.abs(plain[k])[m]
        assert rel.max() <= 1e-6, (k, rel.max(), int((rel > 1e-6).sum()))
