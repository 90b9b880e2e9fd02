"""GPU steady-state solver with the constructor and state of the reference's
PDRSolver3D (prism3d/solver_3d.py:34-149).

    s = PDRSolverGPU(density, box_size, G0_external=directional_G0(...),
                     zeta_CR_0=2e-16, nside_rt=2, T_init=100.0)
    converged = s.run(convergence_tol=1e-10, mixed=True)
    s.T_gas, s.x_H2, ...          # (nx, ny, nz) NumPy arrays
    s.save("state.npz")            # the reference's save() keys

The whole outer iteration runs on the device (libprism3d_gb300.so,
p3d_steady_*): the FUV ray march once (G0, A_V, N_H and the selected ray
depend on density only), then per iteration the selected-ray H2/CO columns,
shielding, cosmic rays, dust coupling, steady-state chemistry and the
thermal root.  ``mixed=False`` is the plain FP64 path, ``mixed=True`` the
batched mixed-precision path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from . import constants as C
from .rays import directional_G0, healpix_directions  # noqa: F401
from .tables import DustTables, line_params

FIELDS = {"T_gas": 0, "x_HI": 1, "x_H2": 2, "x_Cp": 3, "x_C": 4, "x_CO": 5, "x_O": 6, "x_e": 7,
          "G0": 8, "A_V": 9, "N_H": 10, "N_H2": 11, "N_CO": 12, "T_dust": 13, "Gamma_PE": 14,
          "zeta_CR": 15, "f_sh_H2": 16, "Gamma": 17, "Lambda": 18, "change": 19, "f_nano": 20,
          "E_g": 21}


class NotConvergedError(RuntimeError):
    pass


class PDRSolverGPU:
    """Device-resident PRISM-3D steady state on one GB300."""

    def __init__(self, density, box_size, G0_external=1.0, zeta_CR_0=2e-16, nside_rt=1,
                 T_init=50.0, tables=None, star=None):
        self.density = np.ascontiguousarray(density, dtype=np.float64)
        if self.density.ndim != 3:
            raise ValueError("density must be (nx, ny, nz)")
        self.nx, self.ny, self.nz = self.density.shape
        self.n_cells = self.density.size
        self.box_size = float(box_size)
        self.cell_size = self.box_size / self.nx
        self.G0_external = G0_external
        self.zeta_CR_0 = float(zeta_CR_0)
        self.nside_rt = int(nside_rt)
        self.T_init = float(T_init)
        self.tables = tables if tables is not None else DustTables()
        self.history = []
        self.iterations = 0
        self._h = ctypes.c_void_p()
        tb = self.tables
        dirs, w = healpix_directions(self.nside_rt)
        g = np.atleast_1d(np.asarray(G0_external, dtype=np.float64)).ravel()
        sig = np.array([tb.sigma_nano, tb.sigma_largeC, tb.sigma_Sil])
        lines = line_params()
        self._keep = (dirs, w, g, sig, lines)
        p = L.dptr
        L.call("p3d_steady_create", ctypes.byref(self._h), self.nx, self.ny, self.nz,
               p(self.density), p(g), g.size, self.cell_size, p(dirs), p(w), len(dirs),
               self.zeta_CR_0, C.x_C_total, C.x_O_total, self.T_init,
               p(np.ascontiguousarray(tb.pe_table)), tb.n_bins, tb.log_psi_min,
               tb.log_psi_step, tb.n_psi, tb.eg_min, tb.eg_step, tb.n_Eg,
               p(tb.bin_sigma_abs), p(tb.bin_dn_da_da), p(tb.bin_is_nano.astype(np.float64)),
               p(sig), *[p(a) for a in lines])
        # point source: dict with 'position' [cm] and 'L_FUV' [erg/s], as the
        # reference's PDRSolver3D(star=...) (solver_3d.py:70-71, 270-276)
        self.star = star
        if star is not None:
            self._star_pos = np.ascontiguousarray(star["position"], dtype=np.float64).reshape(3)
            L.call("p3d_steady_set_point_source", self._h, p(self._star_pos),
                   float(star["L_FUV"]))
        self.reset()

    def reset(self):
        """Ray march, per-cell constants and analytic initial abundances."""
        L.call("p3d_steady_reset", self._h)
        self.iterations = 0

    def run(self, max_iterations=2000, convergence_tol=1e-8, mixed=True, w_chem=0.5, w_T=0.5,
            n_allow=None, raise_on_failure=False, dust_steps=1):
        """Outer iterations until at most n_allow cells (default
        max(8, 1e-5 n_cells)) change by more than convergence_tol (relative,
        T_gas and species above 1e-20).  With dust_steps > 1 the reference's
        two-level loop (solver_3d.py:239-249): before every inner
        convergence but the first, one THEMIS grain step (_evolve_dust_state)
        on every cell; max_iterations bounds each inner loop.  Returns True
        when the (last) inner loop converged."""
        if dust_steps < 1:
            raise ValueError("dust_steps must be >= 1")
        ok = True
        for step in range(int(dust_steps)):
            if step > 0:
                L.call("p3d_steady_dust_step", self._h)
            ok = self._inner(max_iterations, convergence_tol, mixed, w_chem, w_T, n_allow,
                             raise_on_failure)
        return ok

    def _inner(self, max_iterations, convergence_tol, mixed, w_chem, w_T, n_allow,
               raise_on_failure):
        if n_allow is None:
            n_allow = max(8, int(1e-5 * self.n_cells))
        it = L._i64(0)
        dm = L._f64(0.0)
        rc = L.lib.p3d_steady_run(self._h, int(bool(mixed)), int(max_iterations),
                                  float(convergence_tol), int(n_allow), float(w_chem), float(w_T),
                                  ctypes.byref(it), ctypes.byref(dm))
        self.iterations = int(it.value)
        self.last_change = float(dm.value)
        if rc == -5:
            if raise_on_failure:
                raise NotConvergedError(L.lib.p3d_last_error().decode())
            return False
        L.check("p3d_steady_run", rc)
        return True

    def autotune(self, warm_iterations=13):
        """Time the per-cell kernels' launch shapes on a representative state
        and keep the fastest (threads per block, blocks per SM); resets the
        solver.  Returns (threads, blocks_per_sm, ms)."""
        cfg = np.zeros(2, np.int32)
        ms = L._f64(0.0)
        L.call("p3d_steady_autotune", self._h, int(warm_iterations), L.iptr(cfg),
               ctypes.byref(ms))
        self.iterations = 0
        return int(cfg[0]), int(cfg[1]), float(ms.value)

    def set_launch(self, threads, blocks_per_sm):
        """Set the per-cell kernels' launch shape directly (threads 128 or
        256, 1-64 blocks per SM), e.g. one autotune() chose before for the
        same grid; the state is kept."""
        L.call("p3d_steady_set_launch", self._h, int(threads), int(blocks_per_sm))

    def set_coop_max(self, max_cells):
        """Worklists of at most max_cells cells are solved one cell per warp
        by the mixed thermal kernel (its FP64 net heating evaluated by the
        whole warp; default 4096, 0 never)."""
        L.call("p3d_steady_set_coop_max", self._h, int(max_cells))

    RATE_NAMES = ("H2_formation", "H2_photodiss", "H2_cr_destruction", "C_photoion",
                  "Cp_recombination", "CO_photodiss", "CO_cr_dissociation", "C_OH_to_CO")

    def set_rate_scale(self, scale):
        """Multipliers of the reduced network's eight rate coefficients
        (RATE_NAMES order; 1 = the reference's), used from the next run()."""
        sc = np.ascontiguousarray(scale, dtype=np.float64)
        if sc.shape != (8,):
            raise ValueError("rate scale needs 8 values")
        L.call("p3d_steady_set_rate_scale", self._h, L.dptr(sc))

    def refine(self, network=None, mixed=True, rtol=1e-8, max_iter=300, return_species=False,
               return_conditions=False):
        """Refinement pass with the full 31-species network (the reference's
        BDF refine(), solver_3d.py:1056-1089): every cell's network steady
        state from the current conditions and abundances, written back, then
        T_gas re-solved.  Returns the per-cell network status (0 =
        converged), then with return_species the (nx, ny, nz, 31) abundances
        and with return_conditions the (n_cells, 7) conditions used."""
        from .network import ChemistrySolverGPU
        own = network is None
        net = ChemistrySolverGPU() if own else network
        x = np.empty((self.n_cells, 31)) if return_species else None
        cond = np.empty((self.n_cells, 7)) if return_conditions else None
        st = np.empty(self.n_cells, np.int32)
        try:
            rc = L.lib.p3d_steady_refine(self._h, net._h, int(bool(mixed)), int(max_iter),
                                         float(rtol), L.dptr(cond), L.dptr(x), L.iptr(st))
            if rc != -5:  # P3D_ECONVERGE: results kept, status says which cells
                L.check("p3d_steady_refine", rc)
        finally:
            if own:
                net.close()
        out = [st.reshape(self.nx, self.ny, self.nz)]
        if return_species:
            out.append(x.reshape(self.nx, self.ny, self.nz, 31))
        if return_conditions:
            out.append(cond)
        return out[0] if len(out) == 1 else tuple(out)

    def set_fixed_temperature(self, fixed=True):
        """Hold T_gas at its current values in later run() calls (chemistry
        and shielding only) or solve the thermal balance again."""
        L.call("p3d_steady_set_fixed_temperature", self._h, int(bool(fixed)))

    def adjoint(self, w_columns=(0.0, 0.0, 1.0, 1.0, 1.0), w_T=1.0, max_sweeps=20000, tol=1e-10,
                omega=0.5, density_gradient=False):
        """Gradient of L = sum_cells n_H dx sum_s w_columns[s] x_s + w_T mean(T_gas)
        (s = x_HI, x_H2, x_C+, x_C, x_CO: weighted column sums over the grid)
        at the converged state with respect to the log rate multipliers
        (RATE_NAMES) and log G0.  Returns a dict with 'grad' (9,), 'loss_col',
        'loss_T', 'sweeps', 'n_jump', 'converged' (sweeps reached tol) and
        'message'."""
        w = np.zeros(6)
        w[:5] = np.asarray(w_columns, float)
        w[5] = float(w_T)
        g = np.zeros(9)
        loss = np.zeros(2)
        sw = L._i64(0)
        nj = L._i64(0)
        gn = np.zeros(self.n_cells) if density_gradient else None
        rc = L.lib.p3d_steady_adjoint(self._h, L.dptr(w), self.cell_size, int(max_sweeps),
                                      float(tol), float(omega), L.dptr(g), L.dptr(gn),
                                      L.dptr(loss), ctypes.byref(sw), ctypes.byref(nj))
        if rc != -5:  # P3D_ECONVERGE: tol not reached, results kept
            L.check("p3d_steady_adjoint", rc)
        out = {"grad": g, "loss_col": float(loss[0]), "loss_T": float(loss[1]),
               "sweeps": int(sw.value), "n_jump": int(nj.value), "converged": rc == 0,
               "message": "" if rc == 0 else L.lib.p3d_last_error().decode()}
        if density_gradient:
            out["grad_ln_nH"] = gn.reshape(self.nx, self.ny, self.nz)
        return out

    def set(self, name, values):
        """Overwrite T_gas or one of x_HI, x_H2, x_Cp, x_C, x_CO on the device."""
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if v.size != self.n_cells:
            raise ValueError(f"{name}: {v.size} values for {self.n_cells} cells")
        if name not in ("T_gas", "x_HI", "x_H2", "x_Cp", "x_C", "x_CO"):
            raise KeyError(name)
        L.call("p3d_steady_set", self._h, FIELDS[name], L.dptr(v))

    def get(self, name):
        out = np.empty(self.n_cells)
        L.call("p3d_steady_get", self._h, FIELDS[name], L.dptr(out))
        return out.reshape(self.density.shape)

    def columns(self):
        """(N_H2, N_CO) along each cell's selected ray for the current
        abundances: the columns the next outer iteration's shielding sees."""
        nh2 = np.empty(self.n_cells)
        nco = np.empty(self.n_cells)
        L.call("p3d_steady_columns", self._h, L.dptr(nh2), L.dptr(nco))
        return nh2.reshape(self.density.shape), nco.reshape(self.density.shape)

    def elapsed_ms(self):
        """Device time of the last reset + run (CUDA events, library stream)."""
        ms = L._f64(0.0)
        L.call("p3d_steady_elapsed_ms", self._h, ctypes.byref(ms))
        return float(ms.value)

    def launch_count(self):
        """Kernels launched on the device since the last reset."""
        c = L._i64(0)
        L.call("p3d_steady_launch_count", self._h, ctypes.byref(c))
        return int(c.value)

    def selected_ray(self):
        out = np.empty(self.n_cells, dtype=np.int32)
        L.call("p3d_steady_get_ray", self._h, L.iptr(out))
        return out.reshape(self.density.shape)

    HISTORY_COLUMNS = ("max_rel_change", "chem_fail", "therm_fail", "n_gt_100tol", "n_gt_tol",
                       "n_gt_tol/100", "fp64_net_heating_evals", "t_mean", "n_active")

    def convergence_history(self):
        """(iterations, 9) array, columns HISTORY_COLUMNS."""
        h = np.empty((max(self.iterations, 1), len(self.HISTORY_COLUMNS)))
        n = L._i64(0)
        L.call("p3d_steady_history", self._h, L.dptr(h), h.shape[0], ctypes.byref(n))
        return h[: n.value]

    def __getattr__(self, name):
        if name in FIELDS:
            return self.get(name)
        raise AttributeError(name)

    def state(self):
        return {k: self.get(k) for k in FIELDS}

    def save(self, filepath):
        """np.savez_compressed with the keys of PDRSolver3D.save()
        (solver_3d.py:1150-1170), so the reference's load() reads it.  The
        reference stores one scalar G0_external; the per-ray field and the
        ray count of this solve are added as G0_rays and nside_rt (keys
        load() ignores)."""
        st = self.state()
        shp = self.density.shape
        np.savez_compressed(
            filepath, density=self.density, T_gas=st["T_gas"], T_dust=st["T_dust"],
            G0=st["G0"], A_V=st["A_V"], N_H=st["N_H"], N_H2=st["N_H2"], N_CO=st["N_CO"],
            zeta_CR=st["zeta_CR"], x_HI=st["x_HI"], x_H2=st["x_H2"], x_Cp=st["x_Cp"],
            x_C=st["x_C"], x_CO=st["x_CO"], x_O=st["x_O"], x_e=st["x_e"],
            x_OH=1e-9 + 9e-8 * np.clip(10.0 * st["x_H2"], 0, 1), x_H2O=np.full(shp, 1e-8),
            x_HCOp=np.full(shp, 1e-10), Gamma=st["Gamma"], Lambda=st["Lambda"],
            Gamma_PE=st["Gamma_PE"], f_nano=st["f_nano"], E_g=st["E_g"], box_size=self.box_size,
            G0_external=np.max(np.atleast_1d(self.G0_external)), zeta_CR_0=self.zeta_CR_0,
            G0_rays=np.atleast_1d(np.asarray(self.G0_external, dtype=np.float64)),
            nside_rt=self.nside_rt)

    def close(self):
        if self._h:
            L.lib.p3d_steady_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
