"""GPU steady-state driver against the FP64 CPU restatement of the method.

The outer map is compared step by step (the first iterations from the
initial state, before rounding can steer the few bistable cells), and the
converged GPU state is checked to be a fixed point of the oracle's map:
recomputing the chemistry steady state and the thermal root from it changes
the abundances by <= 1e-6 relative (species above 1e-20 of n_H) and T by
<= 1e-4 relative -- or T sits on a sign change of the thermal balance at one
of its discontinuities.  The model's steady state is not unique (cells with
thermal bistability can settle on either branch, and the grid-mean T couples
every cell to that choice), so two converged runs are compared through this
fixed-point property, not cell by cell.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
SPECIES = ("x_HI", "x_H2", "x_Cp", "x_C", "x_CO")


def _solver(name, seed=1):
    from prism3d_gb300 import fields
    from prism3d_gb300.solver import PDRSolverGPU
    dens, g0, nside, zeta, cell = fields.workload(name, seed)
    s = PDRSolverGPU(dens, cell * dens.shape[0], G0_external=g0, zeta_CR_0=zeta, nside_rt=nside,
                     T_init=100.0)
    return s, (dens, g0, nside, zeta, cell)


@pytest.mark.parametrize("mixed,k", [(False, 3), (True, 1)])
def test_first_iterations_match_oracle(mixed, k):
    """Plain: three outer iterations.  Mixed: the first one (from the second
    on, the mixed path warm-starts each thermal root from the previous one and
    may follow a different but equally valid path through bistable cells)."""
    s, (dens, g0, nside, zeta, cell) = _solver("cube16")
    s.run(max_iterations=k, convergence_tol=1e-300, mixed=mixed, n_allow=0)
    assert s.iterations == k
    ref, hist = O.steady_run(dens, g0, cell, nside=nside, zeta0=zeta, max_outer=k, tol=0.0)
    assert np.array_equal(s.selected_ray(), ref["ray"])
    np.testing.assert_array_equal(s.get("A_V"), ref["A_V"])
    np.testing.assert_array_equal(s.get("N_H"), ref["N_H"])
    np.testing.assert_allclose(s.get("G0"), ref["G0"], rtol=1e-12)
    # plain: FP64 end to end; mixed: FP32 factorisation and bisection (signs
    # certified), compaction from iteration 3 on
    tol, frac = (1e-8, 0.999) if not mixed else (1e-6, 0.99)
    for key in SPECIES + ("T_gas",):
        a, b = s.get(key), ref[key]
        m = np.abs(b) > 1e-20
        rel = np.abs(a - b)[m] / np.abs(b)[m]
        assert np.mean(rel <= tol) >= frac, (key, np.mean(rel <= tol), rel.max())


@pytest.mark.parametrize("mixed", [False, True])
def test_converged_state_is_fixed_point(mixed):
    s, (dens, g0, nside, zeta, cell) = _solver("cube16")
    ok = s.run(max_iterations=3000, convergence_tol=1e-9, mixed=mixed, n_allow=0)
    assert ok, s.last_change
    st = {k: s.get(k) for k in SPECIES + ("x_O", "x_e", "T_gas")}
    np.testing.assert_allclose(st["x_HI"] + 2 * st["x_H2"], 1.0, atol=1e-12)
    np.testing.assert_allclose(st["x_Cp"] + st["x_C"] + st["x_CO"], O.X_C, rtol=1e-12)
    x_star, G, _, ctx = O.map_residual(st, dens, g0, cell, nside, zeta)
    for k in SPECIES:
        m = st[k] > 1e-20
        rel = np.abs(x_star[k] - st[k])[m] / st[k][m]
        assert rel.max() <= 1e-6, (k, rel.max())
    T = st["T_gas"]
    off = np.abs(G - T) / T > 1e-4
    assert np.mean(off) < 0.01, int(off.sum())
    if np.any(off):
        # allowed only where the outer map jumps across T: G(T) - T changes
        # sign between T (1 - 1e-7) and T (1 + 1e-7)
        r = {}
        for f in (1 - 1e-7, 1 + 1e-7):
            s2 = dict(st)
            s2["T_gas"] = T * f
            _, G2, _, _ = O.map_residual(s2, dens, g0, cell, nside, zeta)
            r[f] = (G2 - T * f)[off]
        jump = (r[1 - 1e-7] > 0) & (r[1 + 1e-7] < 0)
        assert np.sum(~jump) <= max(2, int(1e-3 * T.size)), (int(off.sum()), int(np.sum(~jump)))


def test_autotune_keeps_results():
    """The launch shape changes no per-cell arithmetic: a solve after
    autotuning reproduces the untuned one exactly."""
    s, _ = _solver("cube16")
    s.run(max_iterations=12, convergence_tol=1e-300, mixed=True, n_allow=0)
    ref = {k: s.get(k) for k in SPECIES + ("T_gas",)}
    threads, per_sm, ms = s.autotune(warm_iterations=5)
    assert threads in (128, 256) and per_sm in (2, 4, 8, 16, 32, 64) and ms > 0
    s.run(max_iterations=12, convergence_tol=1e-300, mixed=True, n_allow=0)
    for k, v in ref.items():
        np.testing.assert_array_equal(s.get(k), v)
    s.close()


def test_cooperative_thermal_root_reaches_the_plain_state():
    """The mixed thermal kernel solves short worklists one cell per warp with
    the warp-cooperative FP64 net heating (net_heating_coop64: same terms,
    another summation order).  Forced on every mixed solve (and off), the
    converged 16^3 state matches the plain FP64 one in every settled cell
    (1e-6 species above 1e-20 of n_H, 1e-4 T)."""
    tol = 1e-8
    plain, _ = _solver("cube16")
    n_allow = 8
    assert plain.run(max_iterations=3000, convergence_tol=tol, mixed=False, n_allow=n_allow,
                     w_chem=0.1)
    ref = {k: plain.get(k) for k in SPECIES + ("T_gas", "change")}
    plain.close()
    for coop in (1 << 30, 0):
        s, _ = _solver("cube16")
        s.set_coop_max(coop)
        assert s.run(max_iterations=3000, convergence_tol=tol, mixed=True, n_allow=n_allow,
                     w_chem=0.1)
        moving = (s.get("change") > tol) | (ref["change"] > tol)
        for k in SPECIES + ("T_gas",):
            a, b = s.get(k), ref[k]
            m = (np.abs(b) > 1e-20) & ~moving
            rel = np.abs(a - b)[m] / np.abs(b)[m]
            assert rel.max() <= (1e-4 if k == "T_gas" else 1e-6), (coop, k, rel.max())
        s.close()


def test_max_iterations_is_a_cap():
    """The mixed path runs graphs of eight iterations; a max_iterations that
    is not a multiple of eight still stops there (the remainder one by one),
    and graph and single launches give the same state."""
    s, _ = _solver("cube16")
    s.run(max_iterations=13, convergence_tol=1e-300, mixed=True, n_allow=0)
    assert s.iterations == 13 and s.convergence_history().shape[0] == 13
    ref = {k: s.get(k) for k in SPECIES + ("T_gas",)}
    s.reset()
    for _ in range(13):
        s.run(max_iterations=1, convergence_tol=1e-300, mixed=True, n_allow=0)
    assert s.iterations == 13
    for k, v in ref.items():
        np.testing.assert_array_equal(s.get(k), v)
    s.close()


def test_column_tiles_left_out_match_full_passes():
    """From its second iteration a mixed run recomputes only the column
    tiles (32 pencils along x or y, one pencil along z) holding cells the
    last chemistry rewrote; every run() starts with a full pass.  A full
    mixed solve of the 96^3 slab in one run and as many one-iteration runs
    (a full column pass each time) give the same state bit for bit, the tail
    of the solve included (a few thousand cells listed, in the H/H2
    transition front, most tiles left out)."""
    s, (dens, *_) = _solver("slab96")
    n_allow = max(8, int(1e-5 * dens.size))
    assert s.run(max_iterations=4000, convergence_tol=1e-8, mixed=True, n_allow=n_allow,
                 w_chem=0.1)
    k_it = s.iterations
    ref = {k: s.get(k) for k in SPECIES + ("T_gas", "N_H2", "N_CO")}
    listed = s.convergence_history()[:, 8]
    assert listed[-1] < 0.01 * dens.size, listed[-5:]
    s.reset()
    for _ in range(k_it):
        s.run(max_iterations=1, convergence_tol=1e-8, mixed=True, n_allow=n_allow, w_chem=0.1)
    assert s.iterations == k_it
    for k, v in ref.items():
        np.testing.assert_array_equal(s.get(k), v)
    s.close()


def test_heating_cooling_diagnostics_and_saved_state(tmp_path):
    """Gamma and Lambda of the converged state (the reference stores them
    after each thermal solve, solver_3d.py:891-892) against the oracle's
    restatement of _total_heating_vec / _total_cooling_vec on the same state,
    and save() writing the keys of PDRSolver3D.save() (solver_3d.py:1152-1166)
    that PDRSolver3D.load() reads back (:1184-1187)."""
    s, (dens, g0, nside, zeta, cell) = _solver("cube16")
    assert s.run(max_iterations=3000, convergence_tol=1e-9, mixed=True, n_allow=0)
    st = {k: s.get(k) for k in SPECIES + ("x_O", "x_e", "T_gas", "T_dust", "Gamma_PE", "G0",
                                          "A_V", "zeta_CR", "f_sh_H2", "Gamma", "Lambda")}
    tb = s.tables
    st["density"] = dens
    st["R_H2"] = O.h2_formation_rate(st["T_gas"], st["T_dust"], 1.0, tb.sigma_nano,
                                     tb.sigma_largeC, tb.sigma_Sil)
    ctx = O.thermal_ctx(st, st["f_sh_H2"])
    T = st["T_gas"].ravel()
    G, L = O.total_heating_cooling(ctx, T)
    scale = np.abs(np.ravel(ctx[0])) + np.abs(np.ravel(ctx[1]) * np.sqrt(T) *
                                              (np.ravel(ctx[2]) - T))
    # the kernels' context holds Gamma_PE and R_H2 of each cell's last
    # chemistry solve, at the T before its last update (<= 1e-9 away)
    assert np.max(np.abs(st["Gamma"].ravel() - G) / scale) < 1e-6
    np.testing.assert_allclose(st["Lambda"].ravel(), L, rtol=1e-6)
    path = tmp_path / "state.npz"
    s.save(str(path))
    data = np.load(path)
    ref_keys = {"density", "T_gas", "T_dust", "G0", "A_V", "N_H", "N_H2", "N_CO", "zeta_CR",
                "x_HI", "x_H2", "x_Cp", "x_C", "x_CO", "x_O", "x_e", "x_OH", "x_H2O", "x_HCOp",
                "Gamma", "Lambda", "Gamma_PE", "f_nano", "E_g", "box_size", "G0_external",
                "zeta_CR_0"}
    assert ref_keys <= set(data.files), ref_keys - set(data.files)
    for k in ("T_gas", "Gamma", "Lambda", "x_CO"):
        np.testing.assert_array_equal(data[k], st[k])
    s.close()
