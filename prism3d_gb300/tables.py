"""One-time host tables for the hot path.

* THEMIS grain bins and the photoelectric-heating table PE(bin, log psi, E_g)
  that ``pe_heating_vec`` interpolates (grains/themis.py:81-289 for the grain
  populations, grains/themis_tables.py:57-151 for the table, :255-276 for the
  H2-formation area sums of buchbend/prism3d).
* Line-parameter vectors in the layout ``solve_thermal_vec`` takes
  (solver_3d.py:778-781).
* The CO rotational ladder constants (rust/src/thermal.rs:21-41).

These are built once on the host with NumPy (about 0.2 s) and uploaded to the
device; nothing here runs per iteration.
"""
from __future__ import annotations

import numpy as np

from . import constants as C


class GrainPopulation:
    """Size-binned grain population (grains/themis.py:109-171)."""

    def __init__(self, name, a_min, a_max, n_bins, rho, E_g=0.1, slope=-3.5,
                 mass_fraction=0.1):
        self.name = name
        self.n_bins = n_bins
        edges = np.logspace(np.log10(a_min), np.log10(a_max), n_bins + 1)
        self.a = np.sqrt(edges[:-1] * edges[1:])
        self.da = edges[1:] - edges[:-1]
        raw = self.a ** slope
        mass = np.sum((4.0 / 3.0) * np.pi * self.a ** 3 * rho * raw * self.da)
        target = mass_fraction * C.DUST_TO_GAS * C.m_H
        self.dn_da = raw * (target / mass) if mass > 0 else raw * 0
        x = 2 * np.pi * self.a / 0.1e-4  # FUV size parameter at 1000 A
        if "aC" in name:
            q = np.where(x > 1, 1.0, x)
            q = q * np.clip(1.0 + 0.5 * (0.1 - min(E_g, 0.5)), 0.5, 1.5)
        else:
            q = np.where(x > 1, 0.7, 0.7 * x)
        self.Q_abs_FUV = q

    def total_number(self):
        return np.sum(self.dn_da * self.da)


def themis_populations(f_nano=1.0, E_g=0.1):
    """The three THEMIS populations (grains/themis.py:249-289)."""
    nano = GrainPopulation("aC_nano", 4e-8, 2e-7, 12, 1.6, E_g=E_g,
                           mass_fraction=0.005 * f_nano)
    n_cur = nano.total_number()
    if n_cur > 0:
        nano.dn_da = nano.dn_da * (1e-7 * f_nano / n_cur)
    large = GrainPopulation("aC_large", 2e-7, 2e-5, 10, 1.6, E_g=0.1,
                            mass_fraction=0.30)
    sil = GrainPopulation("aSil", 2e-7, 3e-5, 10, 3.5, mass_fraction=0.695)
    return [nano, large, sil]


class DustTables:
    """PE table + grain bin vectors + H2 formation area sums.

    Attribute names follow grains/themis_tables.py so a caller of the
    reference's ``THEMISTables`` finds the same fields.
    """

    def __init__(self, n_psi=200, n_Eg=20, f_nano=1.0, E_g=0.1):
        self.n_psi = n_psi
        self.n_Eg = n_Eg
        self.log_psi_grid = np.linspace(-1, 7, n_psi)
        self.Eg_grid = np.linspace(0.01, 2.5, n_Eg)
        pops = themis_populations(f_nano, E_g)
        self._build_pe(pops)
        self._build_h2(pops)

    @property
    def log_psi_min(self):
        return float(self.log_psi_grid[0])

    @property
    def log_psi_step(self):
        return float(self.log_psi_grid[1] - self.log_psi_grid[0])

    @property
    def eg_min(self):
        return float(self.Eg_grid[0])

    @property
    def eg_step(self):
        return float(self.Eg_grid[1] - self.Eg_grid[0])

    def _build_pe(self, pops):
        # per-bin records in population order (themis_tables.py:68-89)
        a_l, sig_l, ndd_l, carb_l, nano_l = [], [], [], [], []
        for pop in pops:
            for i in range(pop.n_bins):
                a_l.append(pop.a[i])
                sig_l.append(np.pi * pop.a[i] ** 2 * pop.Q_abs_FUV[i])
                ndd_l.append(pop.dn_da[i] * pop.da[i])
                carb_l.append("aC" in pop.name)
                nano_l.append(pop.name == "aC_nano")
        self.n_bins = len(a_l)
        self.bin_a = np.array(a_l)
        self.bin_sigma_abs = np.array(sig_l)
        self.bin_dn_da_da = np.array(ndd_l)
        self.bin_is_carbon = np.array(carb_l)
        self.bin_is_nano = np.array(nano_l)

        table = np.zeros((self.n_bins, self.n_psi, self.n_Eg))
        psi = 10.0 ** self.log_psi_grid[:, None]
        eg = self.Eg_grid[None, :]
        e2 = C.e_charge ** 2
        for ib in range(self.n_bins):
            a = self.bin_a[ib]
            carbon = bool(self.bin_is_carbon[ib])
            y0 = 0.14 if carbon else 0.05
            W = 4.0 + eg if carbon else np.full((1, 1), 8.0)
            zmax = np.maximum((10.0 - W) * a * C.eV_to_erg / e2, 0.5)
            z = np.arange(-1, int(np.max(zmax)) + 2)[None, None, :]
            zmean = np.minimum(psi * a / 5e-7, zmax)
            sz = np.maximum(1.0, np.sqrt(zmean + 1))
            pz = np.exp(-0.5 * ((z - zmean[:, :, None]) / sz[:, :, None]) ** 2)
            pz /= np.sum(pz, axis=2, keepdims=True)
            zpos = np.maximum(z, 0)
            yz = y0 * np.maximum(1.0 - zpos / (zmax[:, :, None] + 1), 0.01)
            if a < 1e-7:
                yz = yz * min(3.0, 1e-7 / a)
            ip = W[:, :, None] * C.eV_to_erg + zpos * e2 / max(a, 1e-8)
            epe = np.maximum(C.E_FUV_MEAN - ip, 0.0)
            table[ib] = np.sum(pz * yz * epe, axis=2)
            if not carbon:
                table[ib, :, :] = table[ib, :, 0:1]
        self.pe_table = table

    def _build_h2(self, pops):
        area = {p.name: np.sum(np.pi * p.a ** 2 * p.dn_da * p.da) for p in pops}
        self.sigma_nano = float(area.get("aC_nano", 0.0))
        self.sigma_largeC = float(area.get("aC_large", 0.0))
        self.sigma_Sil = float(area.get("aSil", 0.0))


def line_params():
    """(cii[5], oi63[5], oi145[5], ci[10]) in the solve_thermal_vec layout."""
    f64 = np.float64
    return (np.array(C.CII_158, dtype=f64), np.array(C.OI_63, dtype=f64),
            np.array(C.OI_145, dtype=f64),
            np.array(C.CI_609 + C.CI_370, dtype=f64))


def co_ladder():
    """(40, 5) array of (T_u, A, g_u/g_l, 1 + 0.1 J, A h nu) for J_u = 1..40."""
    out = np.zeros((40, 5))
    for ju in range(1, 41):
        j = float(ju)
        freq = 2.0 * C.CO_B_rot * j
        t_u = C.h_planck * C.CO_B_rot * j * (j + 1.0) / C.k_boltz
        a_co = (64.0 * np.pi ** 4 * freq ** 3 * C.CO_dipole ** 2 * j) / \
               (3.0 * C.h_planck * C.c_light ** 3 * (2.0 * j + 1.0))
        out[ju - 1] = (t_u, a_co, (2.0 * j + 1.0) / (2.0 * (j - 1.0) + 1.0),
                       1.0 + 0.1 * j, a_co * C.h_planck * freq)
    return out
