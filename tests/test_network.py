"""Full 31-species network: oracle pins (CPU) and GPU parity (gpu marker).

The oracle (oracle/network.py) is pinned to the reference's own RHS
(ChemistrySolver._rhs, prism3d/chemistry/solver.py:69-143), to its two
post-solve corrections (solver.py:227-281, :345-388) and to steady states of
the reference RHS integrated with SciPy BDF at charge neutrality
(tests/golden/make_network.py).  The GPU kernels are then checked against the
oracle on the same seeded inputs.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import network as N  # noqa: E402

GOLD = np.load(os.path.join(ROOT, "tests", "golden", "network.npz"))
NET = N.load()


def _cells(n, seed):
    """Seeded physical conditions and the reference's initial abundances."""
    rng = np.random.default_rng(seed)
    cond = np.stack([10 ** rng.uniform(1, 6.5, n), 10 ** rng.uniform(1, 4, n),
                     10 ** rng.uniform(-1, 5, n), rng.uniform(0, 20, n),
                     10 ** rng.uniform(-17, -15, n), 10 ** rng.uniform(-8, 0, n),
                     10 ** rng.uniform(-6, 0, n)], axis=1)
    x0 = np.stack([_default_initial(c[2], c[3]) for c in cond])
    return np.ascontiguousarray(cond), np.ascontiguousarray(x0)


def _default_initial(g0, a_v):
    """solver.py:297-343 as an array in the tracked-species order."""
    gp = NET["gas_phase"]
    i = NET["idx"]
    x = np.full(len(NET["species"]), N.X_FLOOR)
    f_h2 = 0.5 * (1.0 + np.tanh((a_v - 1.5) / 0.5))
    f_co = 0.5 * (1.0 + np.tanh((a_v - 3.0) / 0.8))
    x[i["H"]] = max(1.0 - f_h2, 0.003)
    x[i["H2"]] = f_h2 * 0.5
    x[i["C+"]] = gp["C"] * (1.0 - f_co)
    x[i["CO"]] = gp["C"] * f_co * 0.95
    x[i["C"]] = gp["C"] * f_co * 0.05
    x[i["O"]] = max(gp["O"] - x[i["CO"]], 1e-10)
    for ion, neut in (("S+", "S"), ("Si+", "Si"), ("Fe+", "Fe")):
        f = max(0.01, 1.0 - a_v / 3.0) if a_v < 3 else 0.01
        x[i[ion]] = gp[neut] * f
        x[i[neut]] = gp[neut] * (1 - f)
    x[i["H+"]] = 1e-6 if a_v < 2 else 1e-7
    x[i["e-"]] = max(x[i["C+"]] + x[i["S+"]] + x[i["Si+"]] + x[i["Fe+"]] + x[i["H+"]], 1e-7)
    for s, v in (("H-", 1e-14), ("H2+", 1e-13), ("OH+", 1e-13), ("H2O+", 1e-14),
                 ("H3O+", 1e-13), ("CH", 1e-10), ("CH+", 1e-13), ("CH2+", 1e-14),
                 ("CO+", 1e-15), ("O+", 1e-13), ("He", gp["He"]), ("He+", 1e-13)):
        x[i[s]] = v
    x[i["H3+"]] = 5e-10 if a_v > 2 else 1e-12
    x[i["OH"]] = 1e-7 if a_v > 2 else 1e-9
    x[i["H2O"]] = 1e-7 if a_v > 3 else 1e-9
    x[i["O2"]] = 1e-8 if a_v > 3 else 1e-12
    x[i["HCO+"]] = 1e-9 if a_v > 2 else 1e-12
    return x


def _rel(a, b, floor=1e-20):
    big = np.maximum(np.abs(a), np.abs(b)) > floor
    return np.max(np.abs(a - b)[big] / np.abs(b)[big])


# --------------------------------------------------------------------- CPU
def test_network_table():
    assert tuple(NET["species"]) == tuple(GOLD_SPECIES)
    names = NET["names"]
    assert len(names) == 75 and len(set(names)) == 75
    counts = np.bincount(NET["rtype"], minlength=4)
    # 28 two-body + 18 recombination + 7 grain recombination + 2 charge exchange,
    # 7 photodissociation + 4 photoionisation, 3 cosmic-ray + 5 CR-photon, 1 grain surface
    assert counts.tolist() == [55, 11, 8, 1]
    # the tracked species conserve H, C, O, S, Si, Fe, He in every reaction
    S = np.zeros((31, 75))
    for j in range(75):
        for i in NET["reac"][j]:
            if i >= 0:
                S[i, j] -= 1
        for i in NET["prod"][j]:
            if i >= 0:
                S[i, j] += 1
    assert np.all(NET["elem"] @ S == 0)


GOLD_SPECIES = ("e-", "H", "H2", "H+", "H-", "H2+", "H3+", "C+", "C", "CO", "CH", "CH+", "CH2+",
                "O", "O+", "OH", "OH+", "H2O", "H2O+", "H3O+", "O2", "CO+", "HCO+", "S", "S+",
                "Si", "Si+", "Fe", "Fe+", "He", "He+")


def test_oracle_rhs_matches_reference():
    f = N.rhs(NET, GOLD["Y"], GOLD["cond"])
    sc = N.rhs_scale(NET, GOLD["Y"], GOLD["cond"])
    assert np.max(np.abs(f - GOLD["F"]) / sc) < 1e-14


def test_oracle_jacobian_matches_differences():
    y, c = GOLD["Y"], GOLD["cond"]
    J = N.jacobian(NET, y, c)
    sc = N.rhs_scale(NET, y, c)
    Jfd = np.zeros_like(J)
    for k in range(31):
        h = 1e-6 * y[:, k]
        yp, ym = y.copy(), y.copy()
        yp[:, k] += h
        ym[:, k] -= h
        Jfd[:, :, k] = (N.rhs(NET, yp, c) - N.rhs(NET, ym, c)) / (2 * h[:, None])
    assert np.max(np.abs(J - Jfd) * y[:, None, :] / sc[:, :, None]) < 1e-8


def test_oracle_post_processing_matches_reference():
    y, pc = GOLD["post_y"], GOLD["post_cond"]
    hp = N.correct_hp_electron(NET, y, pc[:, 0], pc[:, 1], pc[:, 2])
    np.testing.assert_array_equal(hp, GOLD["post_hp"])
    out = N.enforce_conservation(NET, hp)
    np.testing.assert_array_equal(out, GOLD["post_out"])


def test_oracle_steady_state_matches_reference_rhs_bdf():
    """Newton steady state = long SciPy BDF integration of the reference RHS
    (electrons at charge neutrality)."""
    cond, x0, xs = GOLD["neutral_cond"], GOLD["neutral_x0"], GOLD["neutral_x"]
    assert len(cond) >= 4
    y, st, _ = N.steady_state(NET, x0, cond)
    assert np.all(st == 0)
    assert _rel(y, xs, 1e-20) < 1e-5


def test_oracle_steady_state_is_a_root():
    cond, x0 = _cells(64, 3)
    y, st, it = N.steady_state(NET, x0, cond)
    assert (st == 0).mean() >= 0.95
    ok = st == 0
    f = N.rhs(NET, y[ok], cond[ok])
    sc = N.rhs_scale(NET, y[ok], cond[ok])
    live = y[ok] > N.Y_TEST
    live[:, 0] = False  # the electron row is charge neutrality
    assert np.max(np.where(live, np.abs(f) / sc, 0.0)) < 1e-7
    tot0 = N.element_totals(NET, x0[ok])
    np.testing.assert_allclose(N.element_totals(NET, y[ok]), tot0, rtol=1e-10)
    cat = N.cation_mask(NET)
    np.testing.assert_allclose(y[ok][:, 0], y[ok][:, cat].sum(axis=1), rtol=1e-10)


def test_oracle_reference_bdf_differs_only_through_electrons():
    """The reference's own solve_steady_state results (BDF to t_max, then the
    corrections) are not steady states: the PAH- recombinations remove charge
    from the tracked species, so its electrons exceed the cations until the
    final conservation step resets them.  Documented here with numbers: the
    ions and neutrals that do not recombine with electrons agree with the
    Newton steady state to a few per cent, the electron-coupled ones to a
    factor of a few."""
    cond, x0, ref = GOLD["ss_cond"], GOLD["ss_x0"], GOLD["ss_x"]
    y, st, _ = N.solve_steady_state(NET, x0, cond)
    assert np.all(st == 0)
    i = NET["idx"]
    for s in ("H", "H2", "C+", "O"):
        rel = np.abs(y[:, i[s]] - ref[:, i[s]]) / ref[:, i[s]]
        assert np.all(rel[ref[:, i[s]] > 1e-6] < 0.2), s


def test_network_api_without_gpu_raises():
    pytest.importorskip("ctypes")
    from prism3d_gb300 import _lib as L
    if L.lib.p3d_device_count() > 0:
        pytest.skip("GPU present")
    from prism3d_gb300.network import ChemistrySolverGPU
    with pytest.raises(L.P3DError):
        ChemistrySolverGPU()


# --------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def gpu_net():
    from prism3d_gb300.network import ChemistrySolverGPU
    s = ChemistrySolverGPU()
    yield s
    s.close()


@pytest.mark.gpu
def test_gpu_rhs_matches_reference(gpu_net):
    f = gpu_net.rhs_batch(np.ascontiguousarray(GOLD["Y"]), np.ascontiguousarray(GOLD["cond"]))
    sc = N.rhs_scale(NET, GOLD["Y"], GOLD["cond"])
    assert np.max(np.abs(f - GOLD["F"]) / sc) < 1e-13


@pytest.mark.gpu
def test_gpu_rhs_single_state_signature(gpu_net):
    y = GOLD["Y"][5]
    c = GOLD["cond"][5]
    f = gpu_net._rhs(0.0, y, *c)
    sc = N.rhs_scale(NET, y[None], c[None])[0]
    assert np.max(np.abs(f - GOLD["F"][5]) / sc) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_steady_matches_oracle(gpu_net, mixed):
    cond, x0 = _cells(256, 11)
    ref, st_ref, _ = N.steady_state(NET, x0, cond)
    x = x0.copy()
    st, it = gpu_net.solve_steady_state_batch(cond, x, mixed=mixed, post=False,
                                             return_iters=True)
    both = (st == 0) & (st_ref == 0)
    assert (st == 0).mean() >= 0.97
    assert both.mean() >= 0.95
    assert _rel(x[both], ref[both], 1e-20) < 1e-6
    assert np.all(it >= 1) and np.all(it <= 300)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_steady_matches_reference_rhs_bdf(gpu_net, mixed):
    cond = np.ascontiguousarray(GOLD["neutral_cond"])
    x = np.ascontiguousarray(GOLD["neutral_x0"]).copy()
    st = gpu_net.solve_steady_state_batch(cond, x, mixed=mixed, post=False)
    assert np.all(st == 0)
    assert _rel(x, GOLD["neutral_x"], 1e-20) < 1e-5


@pytest.mark.gpu
def test_gpu_post_processing_is_the_reference_step(gpu_net):
    cond, x0 = _cells(128, 12)
    raw = x0.copy()
    gpu_net.solve_steady_state_batch(cond, raw, mixed=False, post=False)
    post = x0.copy()
    gpu_net.solve_steady_state_batch(cond, post, mixed=False, post=True)
    exp = N.enforce_conservation(NET, N.correct_hp_electron(NET, raw, cond[:, 0], cond[:, 1],
                                                            cond[:, 4]))
    # same Newton iterates on the device, then the reference's arithmetic
    np.testing.assert_allclose(post, exp, rtol=1e-13, atol=0)


@pytest.mark.gpu
def test_gpu_solve_steady_state_signature(gpu_net):
    c = GOLD["ss_cond"][2]
    res, conv = gpu_net.solve_steady_state(*c[:5], f_shield_H2=c[5], f_shield_CO=c[6])
    assert conv and set(res) == set(GOLD_SPECIES)
    y, st, _ = N.solve_steady_state(NET, GOLD["ss_x0"][2:3], GOLD["ss_cond"][2:3])
    arr = np.array([res[s] for s in GOLD_SPECIES])
    assert _rel(arr, y[0], 1e-20) < 1e-6


@pytest.mark.gpu
def test_gpu_edge_cases(gpu_net):
    # empty batch
    e = np.zeros((0, 31))
    assert gpu_net.solve_steady_state_batch(np.zeros((0, 7)), e).shape == (0,)
    # dark cell (PAH fallback branch), temperature clamps, refine-pass input
    # with only ten species set (the rest at the 1e-30 floor)
    cond = np.array([[1e4, 20.0, 0.0, 20.0, 1e-16, 1e-9, 1e-9],
                     [1e3, 5.0, 1e2, 1.0, 2e-16, 0.1, 0.5],
                     [1e3, 5e4, 1e3, 0.5, 2e-16, 1.0, 1.0],
                     [1e4, 60.0, 1e3, 4.0, 2e-16, 1e-3, 1e-2]])
    x0 = np.stack([_default_initial(c[2], c[3]) for c in cond])
    keep = [NET["idx"][s] for s in ("H", "H2", "C+", "C", "CO", "O", "e-", "OH", "H2O", "HCO+")]
    sparse = np.full(31, N.X_FLOOR)
    sparse[keep] = x0[3, keep]
    x0[3] = sparse
    ref, st_ref, _ = N.steady_state(NET, x0, cond)
    x = x0.copy()
    st = gpu_net.solve_steady_state_batch(cond, x, mixed=False, post=False)
    assert np.all(st == 0) and np.all(st_ref == 0)
    assert _rel(x, ref, 1e-20) < 1e-6
    f = gpu_net.rhs_batch(x0, cond)
    np.testing.assert_allclose(f, N.rhs(NET, x0, cond), rtol=1e-12,
                               atol=1e-14 * np.max(N.rhs_scale(NET, x0, cond)))


@pytest.mark.gpu
def test_gpu_argument_errors(gpu_net):
    from prism3d_gb300 import _lib as L
    cond, x0 = _cells(4, 1)
    with pytest.raises(ValueError):
        gpu_net.solve_steady_state_batch(cond[:3], x0.copy())
    with pytest.raises(TypeError):
        gpu_net.solve_steady_state_batch(cond, x0.astype(np.float32))
    with pytest.raises(L.P3DError):
        gpu_net.solve_steady_state_batch(cond, x0.copy(), max_iter=0)
    with pytest.raises(L.P3DError):
        gpu_net.solve_steady_state_batch(cond, x0.copy(), rtol=0.0)


@pytest.mark.gpu
def test_gpu_large_batch_properties(gpu_net):
    """At 2^17 cells: element totals and neutrality hold to rounding, the
    residual test holds where the status says converged, and the result
    does not depend on the batch position (a cell solved alone gives the
    same numbers)."""
    torch = pytest.importorskip("torch")
    n = 1 << 17
    cond, x0 = _cells(n, 21)
    dc = torch.from_numpy(cond).cuda()
    dx = torch.from_numpy(x0).cuda()
    st = gpu_net.solve_steady_state_batch(dc, dx, mixed=True, post=False)
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    x = dx.cpu().numpy()
    assert (st == 0).mean() >= 0.97
    ok = st == 0
    np.testing.assert_allclose(N.element_totals(NET, x[ok]), N.element_totals(NET, x0[ok]),
                               rtol=1e-9)
    cat = N.cation_mask(NET)
    np.testing.assert_allclose(x[ok][:, 0], x[ok][:, cat].sum(axis=1), rtol=1e-9)
    sub = np.nonzero(ok)[0][:: n // 64]
    f = N.rhs(NET, x[sub], cond[sub])
    sc = N.rhs_scale(NET, x[sub], cond[sub])
    live = x[sub] > N.Y_TEST
    live[:, 0] = False
    assert np.max(np.where(live, np.abs(f) / sc, 0.0)) < 1e-6
    one = x0[sub[:8]].copy()
    gpu_net.solve_steady_state_batch(np.ascontiguousarray(cond[sub[:8]]), one, mixed=True,
                                     post=False)
    np.testing.assert_array_equal(one, x[sub[:8]])
