// p3d_phys.cuh -- per-cell physics used by the steady-state driver (FP64).
#pragma once

#include "p3d_common.cuh"
#include "p3d_fastexp.cuh"

namespace p3d {

constexpr double kMH = 1.6735575e-24;
constexpr double kPi = 3.14159265358979323846;
// sqrt(8 k_B / (pi mu m_H)) for mu = 1 and mu = 2, the gas-grain coupling's
// speed factor (thermal.rs's gg_coeff): the correctly rounded double of the
// same expression, so the per-cell contexts keep their values while leaving
// out a division and a square root per cell (checked in
// tests/test_phys_host.py)
constexpr double kGgSpeedMu1 = 0x1.c4f0d56852f3cp+13;
constexpr double kGgSpeedMu2 = 0x1.404708f2a8ebep+13;

// f_shield_H2, Draine & Bertoldi 1996 (radiative_transfer/shielding.py:17-59)
// with b the Doppler parameter in km/s; *dfdn = d f / d N_H2 (0 where the
// clip to [0, 1] is active).
// FAST (the mixed path): the two fractions over one denominator and exp64
// (one FP64 division instead of four; relative difference ~1e-16).
template <bool FAST = false>
__device__ __forceinline__ double fsh_h2(double n, double b, double* dfdn) {
  double x = n / 5.0e14;
  double q = 1.0 + x / b;
  double sq = sqrt(1.0 + x);
  double e = FAST ? exp64(-8.5e-4 * sq) : exp(-8.5e-4 * sq);
  double f = FAST ? (0.965 * sq + 0.035 * e * (q * q)) / ((q * q) * sq)
                  : 0.965 / (q * q) + 0.035 / sq * e;
  double d = -2.0 * 0.965 / (q * q * q) / b +
             0.035 * e * (-0.5 / ((1.0 + x) * sq) - 0.5 * 8.5e-4 / (1.0 + x));
  *dfdn = (f > 0.0 && f < 1.0) ? d / 5.0e14 : 0.0;
  return fmin(fmax(f, 0.0), 1.0);
}

// |d ln f_H2 / d ln b| at column n given f = fsh_h2(n, b): only the
// 0.965 / q^2 term (q = 1 + x / b) depends on b, and f is never clipped
// (0 < f < 0.99997), so d ln f / d ln b = 2 (0.965 / q^2) (x / b) / (q f).
__device__ __forceinline__ double fsh_h2_dlnb(double n, double b, double f) {
  const double xb = n / 5.0e14 / b;
  const double q = 1.0 + xb;
  return 2.0 * 0.965 * xb / (q * q * q * fmax(f, 1e-300));
}

// f_shield_CO (shielding.py:136-171) and its N_H2 derivative.  FAST (the
// mixed-precision path): the four power laws come from two logarithms (x^a =
// exp(a ln x)) and the exponentials from exp64, with exp(-A) exp(-B) =
// exp(-(A + B)) -- on GB300 the FP64 operations of four pow() calls are a
// large part of the chemistry kernel, which evaluates this once per cell and
// outer iteration; relative difference from the pow() form <= ~1e-13 (the
// error of ln x times a ln x <= ~25 for the columns met).  The plain FP64
// path keeps the pow() form.
template <bool FAST = false>
__device__ __forceinline__ double fsh_co(double nco_in, double nh2_in, double* d_h2) {
  double nco = fmax(nco_in, 1.0), nh2 = fmax(nh2_in, 1.0);
  double A, B, Cc, P4, E, f;
  if (FAST) {
    const double lco = log(nco), lh2 = log(nh2);
    A = 6.428e-8 * exp64(0.53 * lco);
    B = 3.0e-12 * exp64(0.495 * lh2);
    Cc = 1e-5 * exp64(0.6 * lco);
    P4 = exp64(0.48 * lh2);
    E = exp64(-8e-12 * P4);
    f = exp64(-(A + B)) * (1.0 / (1.0 + Cc * E));
  } else {
    A = 6.428e-8 * pow(nco, 0.53);
    B = 3.0e-12 * pow(nh2, 0.495);
    Cc = 1e-5 * pow(nco, 0.6);
    P4 = pow(nh2, 0.48);
    E = exp(-8e-12 * P4);
    f = exp(-A) * exp(-B) * (1.0 / (1.0 + Cc * E));
  }
  bool live = (f > 1e-10 && f < 1.0);
  *d_h2 = (live && nh2_in > 1.0)
              ? f * (-0.495 * B / nh2 + Cc * E * 8e-12 * 0.48 * P4 / (nh2 * (1.0 + Cc * E)))
              : 0.0;
  return fmin(fmax(f, 1e-10), 1.0);
}

// Padovani et al. model 'M' (cosmic_rays/attenuation.py:18-113).
__device__ __forceinline__ double padovani(double nh, double a0, double a1, double a2,
                                           double b0, double b1, double deep) {
  double x = log10(fmax(nh, 1e18) / 1e20);
  double lz = x < -1.0 ? a0 : (x < 2.0 ? a0 - a1 * x - a2 * x * x
                                      : (x < 5.0 ? b0 - b1 * (x - 2.0) : deep));
  return pow(10.0, lz);
}

__device__ __forceinline__ double cr_rate(double nh, double zeta0) {
  double zl = padovani(nh, -15.7, 0.4, 0.1, -16.3, 0.8, -18.7);
  double zh = padovani(nh, -15.0, 0.35, 0.08, -15.6, 0.7, -17.7);
  return fmax(sqrt(zl * zh) * (zeta0 / 2e-16), 1e-22);
}

// Radiative part of the THEMIS dust temperature (themis_tables.py:333-342).
__device__ __forceinline__ double tdust_rad(double g0, double av) {
  double F = kFHabing * g0 * exp(-1.8 * av);
  F = F + kFHabing * 0.5 * exp(-av);
  F = fmax(F, 1e-30);
  return fmin(fmax(16.4 * pow(F / kFHabing, 0.167), 5.0), 200.0);
}

// Gas-grain coupling at high density (themis_tables.py:344-352).
__device__ __forceinline__ double tdust(double td_rad, double nh, double tg) {
  double fc = fmin(fmax(nh / 1e7, 0.0), 1.0);
  return nh > 1e5 ? td_rad * (1.0 - fc) + tg * fc : td_rad;
}

// H2 formation rate coefficient (themis_tables.py:278-319).  FAST (the mixed
// path): 8 k_B / (pi m_H) folded into one constant and the two exponentials
// from exp64 with their divisions as multiplies (two FP64 divisions and two
// library exponentials less per cell; ~1e-16 relative).
constexpr double kH2SpeedSq = 0x1.90b1aa149d378p+27;  // 8 k_B / (pi m_H)
template <bool FAST = false>
__device__ __forceinline__ double h2_form(double tg, double td, double fnano, double s_nano,
                                          double s_lc, double s_sil) {
  double v = FAST ? sqrt(kH2SpeedSq * tg) : sqrt(8.0 * kKBoltz * tg / (kPi * kMH));
  double s = 1.0 / (1.0 + 0.04 * sqrt(tg + td) + 0.002 * tg + 8e-6 * tg * tg);
  double e_sil = td < 14.0 ? 1.0
                 : (td < 25.0 ? (FAST ? exp64((14.0 - td) * 0.2) : exp(-(td - 14.0) / 5.0))
                              : 0.01);
  double e_c = td < 50.0 ? 0.8
               : (td < 400.0 ? 0.8 * (FAST ? exp64((50.0 - td) * 0.005) : exp(-(td - 50.0) / 200.0))
                             : 0.01);
  e_c = fmax(e_c, 0.005);
  return 0.5 * v * s * (e_c * s_nano * fnano + e_c * s_lc + e_sil * s_sil);
}

}  // namespace p3d
