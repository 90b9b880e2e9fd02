"""CGS constants and line data used on the hot path.

Values follow prism3d/utils/constants.py:8-114 and rust/src/constants.rs of
buchbend/prism3d; they are physical constants and tabulated line data, so they
are the same numbers by necessity.
"""

c_light = 2.99792458e10  # cm/s
h_planck = 6.62607015e-27  # erg s
k_boltz = 1.380649e-16  # erg/K
m_H = 1.6735575e-24  # g
m_H2 = 2.0 * m_H
e_charge = 4.80320451e-10  # esu
eV_to_erg = 1.602176634e-12
pc_cm = 3.0856776e18

G0_to_flux = 1.6e-3  # Habing flux, erg cm^-2 s^-1
AV_per_NH = 5.34e-22  # mag cm^2
tau_FUV_per_AV = 1.8

# gas-phase abundances: solar x depletion (utils/constants.py:90-99)
x_C_total = 2.69e-4 * 0.4
x_O_total = 4.90e-4 * 0.6

# Fine-structure lines: (freq_Hz, A_ul, E_u/k, g_u, g_l)
# (utils/constants.py:103-109, without the wavelength column)
CII_158 = (1.9005e12, 2.321e-6, 91.21, 4.0, 2.0)
OI_63 = (4.7448e12, 8.910e-5, 227.71, 3.0, 5.0)
OI_145 = (2.0604e12, 1.750e-5, 326.58, 1.0, 3.0)
CI_609 = (4.9231e11, 7.880e-8, 23.62, 3.0, 1.0)
CI_370 = (8.0929e11, 2.650e-7, 62.46, 5.0, 3.0)

CO_B_rot = 57.635968e9  # Hz
CO_dipole = 0.1098e-18  # esu cm

# THEMIS grain constants (grains/themis.py:53-69)
F_HABING = 1.6e-3
E_FUV_MEAN = 10.0 * eV_to_erg
DUST_TO_GAS = 0.01
m_C = 12.0 * m_H
