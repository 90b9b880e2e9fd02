// p3d_thermal.cuh -- device net-heating function and the reference root.
#pragma once

#include "p3d_common.cuh"

namespace p3d {

// Upper level population of a two-level line: R_lu / (R_lu + R_ul)
// (rust/src/thermal.rs:84-128).
__device__ __forceinline__ double two_level(double q, double a_ul, double boltz,
                                            double g_ratio) {
  double r_lu = g_ratio * q * boltz;
  double r_ul = a_ul + q;
  return r_lu / (r_lu + r_ul);
}

// Gamma - Lambda at temperature t (rust/src/thermal.rs:50-184), FP64.
__device__ __forceinline__ double net_heating64(double t, const ThermalCtx& c,
                                                const LineParams& lp,
                                                const CoLevel* __restrict__ co) {
  const double sqrt_t = sqrt(t);
  const double inv_t = 1.0 / t;
  const double t_01 = t * 0.01;
  double net = c.gamma_fixed + c.gg_coeff * sqrt_t * (c.t_dust - t);
  {  // [CII] 158 um
    const double* l = lp.cii;
    double b = exp(-l[2] * inv_t);
    double gamma_e = 8.63e-6 / (l[4] * sqrt_t) * 2.15 * b;
    double gamma_h = 8.0e-10 * pow(t_01, 0.07);
    double gamma_h2 = 4.9e-10 * pow(t_01, 0.12);
    double q = gamma_e * c.n_e + gamma_h * c.n_hi + gamma_h2 * c.n_h2;
    net -= c.n_cp_nh * two_level(q, l[1], b, l[3] / l[4]) * l[1] * kHPlanck * l[0];
  }
  {  // [OI] 63 um
    const double* l = lp.oi63;
    double q = 9.2e-12 * pow(t, 0.67) * c.n_hi + 4.5e-12 * pow(t, 0.64) * c.n_h2 +
               1.4e-8 * pow(t_01, 0.39) * c.n_e;
    net -= c.n_o_nh * two_level(q, l[1], exp(-l[2] * inv_t), l[3] / l[4]) * l[1] * kHPlanck *
           l[0];
  }
  {  // [OI] 145 um
    const double* l = lp.oi145;
    double q = 4.0e-12 * pow(t, 0.60) * c.n_hi + 2.0e-12 * pow(t, 0.58) * c.n_h2 +
               5.0e-9 * pow(t_01, 0.39) * c.n_e;
    net -= c.n_o_nh * two_level(q, l[1], exp(-l[2] * inv_t), l[3] / l[4]) * l[1] * kHPlanck *
           l[0];
  }
  {  // [CI] 609 + 370 um
    double t03 = pow(t_01, 0.3);
    double tm05 = pow(t_01, -0.5);
    double q = 1.0e-10 * t03 * c.n_hi + 5.0e-11 * t03 * c.n_h2 + 2.0e-7 * tm05 * c.n_e;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const double* l = lp.ci + 5 * k;
      net -= c.n_c_nh * two_level(q, l[1], exp(-l[2] * inv_t), l[3] / l[4]) * l[1] *
             kHPlanck * l[0];
    }
  }
  {  // CO rotational ladder, early break at T_u >= 5 T
    const double g0 = 3.3e-11 * sqrt(t_01);
    const double t5 = 5.0 * t;
    for (int k = 0; k < 40; ++k) {
      const double t_u = co[k].t_u;
      if (t_u >= t5) break;
      double gam = g0 * co[k].j_factor;
      double r_lu = co[k].g_ratio * gam * c.n_h2 * exp(-t_u * inv_t);
      double r_ul = co[k].a_co + gam * c.n_h2;
      net -= c.n_co * r_lu / (r_lu + r_ul) * co[k].ahv;
    }
  }
  if (t >= 100.0) {  // H2 ro-vibrational
    double x = fmin(fmax(log10(fmax(t, 100.0)), 2.0), 4.5);
    double x2 = x * x, x3 = x2 * x, x4 = x3 * x, x5 = x4 * x, x6 = x5 * x;
    double llh = -24.311 + 3.5692 * x - 11.332 * x2 + 15.738 * x3 - 10.581 * x4 +
                 3.5803 * x5 - 0.48365 * x6;
    double llh2 = -24.311 + 4.6585 * x - 14.272 * x2 + 19.779 * x3 - 13.255 * x4 +
                  4.4840 * x5 - 0.60504 * x6;
    double l0 = pow(10.0, llh) * c.n_hi + pow(10.0, llh2) * c.n_h2;
    double lte = pow(10.0, -19.703 + 0.5 * x);
    net -= c.n_h2 * l0 * lte / fmax(l0 + lte, 1e-50);
  }
  if (t >= 3000.0) {  // Lyman alpha
    double q_lu = 2.41e-6 / sqrt_t * 0.486 * exp(-1.18e5 * inv_t);
    net -= c.n_hi * c.n_e * q_lu * 10.2 * kEVtoErg;
  }
  {
    double gg_cool = c.gg_coeff * sqrt_t * (t - c.t_dust);
    if (gg_cool > 0.0) net -= gg_cool;
  }
  net -= c.n_cp_nh * c.n_e * (4.67e-12 * pow(t / 300.0, -0.6)) * kKBoltz * t;
  return net;
}

// Diagnostics Gamma and Lambda at t (_total_heating_vec / _total_cooling_vec,
// solver_3d.py:898-1050): the heating is the context's fixed part plus the
// signed gas-grain exchange, the cooling the sum of the terms net_heating64
// subtracts, accumulated in the reference's order.  Gamma - Lambda is the
// net heating up to rounding.
__device__ __forceinline__ void heating_cooling64(double t, const ThermalCtx& c,
                                                  const LineParams& lp,
                                                  const CoLevel* __restrict__ co,
                                                  double* gamma, double* lambda) {
  const double sqrt_t = sqrt(t);
  const double inv_t = 1.0 / t;
  const double t_01 = t * 0.01;
  *gamma = c.gamma_fixed + c.gg_coeff * sqrt_t * (c.t_dust - t);
  double lam = 0.0;
  {  // [CII] 158 um
    const double* l = lp.cii;
    double b = exp(-l[2] * inv_t);
    double q = 8.63e-6 / (l[4] * sqrt_t) * 2.15 * b * c.n_e +
               8.0e-10 * pow(t_01, 0.07) * c.n_hi + 4.9e-10 * pow(t_01, 0.12) * c.n_h2;
    lam += c.n_cp_nh * two_level(q, l[1], b, l[3] / l[4]) * l[1] * kHPlanck * l[0];
  }
  {  // [OI] 63 um
    const double* l = lp.oi63;
    double q = 9.2e-12 * pow(t, 0.67) * c.n_hi + 4.5e-12 * pow(t, 0.64) * c.n_h2 +
               1.4e-8 * pow(t_01, 0.39) * c.n_e;
    lam += c.n_o_nh * two_level(q, l[1], exp(-l[2] * inv_t), l[3] / l[4]) * l[1] * kHPlanck *
           l[0];
  }
  {  // [OI] 145 um
    const double* l = lp.oi145;
    double q = 4.0e-12 * pow(t, 0.60) * c.n_hi + 2.0e-12 * pow(t, 0.58) * c.n_h2 +
               5.0e-9 * pow(t_01, 0.39) * c.n_e;
    lam += c.n_o_nh * two_level(q, l[1], exp(-l[2] * inv_t), l[3] / l[4]) * l[1] * kHPlanck *
           l[0];
  }
  {  // [CI] 609 + 370 um
    double t03 = pow(t_01, 0.3);
    double q = 1.0e-10 * t03 * c.n_hi + 5.0e-11 * t03 * c.n_h2 +
               2.0e-7 * pow(t_01, -0.5) * c.n_e;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const double* l = lp.ci + 5 * k;
      lam += c.n_c_nh * two_level(q, l[1], exp(-l[2] * inv_t), l[3] / l[4]) * l[1] *
             kHPlanck * l[0];
    }
  }
  {  // CO rotational ladder: levels with T_u < 5 T
    const double g0 = 3.3e-11 * sqrt(t_01);
    const double t5 = 5.0 * t;
    for (int k = 0; k < 40; ++k) {
      const double t_u = co[k].t_u;
      if (t_u >= t5) break;
      double gam = g0 * co[k].j_factor;
      double r_lu = co[k].g_ratio * gam * c.n_h2 * exp(-t_u * inv_t);
      double r_ul = co[k].a_co + gam * c.n_h2;
      lam += c.n_co * r_lu / (r_lu + r_ul) * co[k].ahv;
    }
  }
  if (t >= 100.0) {  // H2 ro-vibrational
    double x = fmin(fmax(log10(fmax(t, 100.0)), 2.0), 4.5);
    double x2 = x * x, x3 = x2 * x, x4 = x3 * x, x5 = x4 * x, x6 = x5 * x;
    double llh = -24.311 + 3.5692 * x - 11.332 * x2 + 15.738 * x3 - 10.581 * x4 +
                 3.5803 * x5 - 0.48365 * x6;
    double llh2 = -24.311 + 4.6585 * x - 14.272 * x2 + 19.779 * x3 - 13.255 * x4 +
                  4.4840 * x5 - 0.60504 * x6;
    double l0 = pow(10.0, llh) * c.n_hi + pow(10.0, llh2) * c.n_h2;
    double lte = pow(10.0, -19.703 + 0.5 * x);
    lam += c.n_h2 * l0 * lte / fmax(l0 + lte, 1e-50);
  }
  if (t >= 3000.0) {  // Lyman alpha
    double q_lu = 2.41e-6 / sqrt_t * 0.486 * exp(-1.18e5 * inv_t);
    lam += c.n_hi * c.n_e * q_lu * 10.2 * kEVtoErg;
  }
  lam += fmax(c.gg_coeff * sqrt_t * (t - c.t_dust), 0.0);  // gas-grain
  lam += c.n_cp_nh * c.n_e * (4.67e-12 * pow(t / 300.0, -0.6)) * kKBoltz * t;
  *lambda = lam;
}

// The reference's hybrid root (rust/src/thermal.rs:189-270).
__device__ __forceinline__ double thermal13_cell(const ThermalCtx& c, const LineParams& lp,
                                                 const CoLevel* __restrict__ co, int n_bisect,
                                                 int n_newton) {
  double t_lo = 10.0, t_hi = 1e5;
  for (int k = 0; k < n_bisect; ++k) {
    double t_mid = sqrt(t_lo * t_hi);
    if (net_heating64(t_mid, c, lp, co) > 0.0) t_lo = t_mid; else t_hi = t_mid;
  }
  double t = sqrt(t_lo * t_hi);
  for (int k = 0; k < n_newton; ++k) {
    double f = net_heating64(t, c, lp, co);
    if (f > 0.0) t_lo = fmax(t_lo, t); else t_hi = fmin(t_hi, t);
    double eps = t * 0.01;
    double fp = net_heating64(t + eps, c, lp, co);
    double dfdt = (fp - f) / eps;
    double dt = (fabs(dfdt) > 1e-50) ? -f / dfdt : -f / (-1e-50);
    dt = fmin(fmax(dt, -(t - t_lo)), t_hi - t);
    dt = fmin(fmax(dt, -0.5 * t), 0.5 * t);
    t += dt;
  }
  return t;
}

cudaError_t upload_co_levels(const CoLevel* host40, cudaStream_t s);
cudaError_t launch_thermal13(int64_t n, const double* const* ctx, const LineParams& lp,
                             int n_bisect, int n_newton, double* t_out, int sms,
                             cudaStream_t s);
cudaError_t launch_heating_cooling(int64_t n, const double* const* ctx, const LineParams& lp,
                                   const double* t, double* gamma, double* lambda, int sms,
                                   cudaStream_t s);

}  // namespace p3d

namespace p3d {

// Bisection of [10, 1e5] K (rust/src/thermal.rs:231-243) followed by a
// safeguarded Newton iteration (Newton with a forward-difference slope,
// bisection whenever the step leaves the bracket or does not halve the
// previous step) until |dT| <= tol T or the bracket is narrower than tol T.
// A sign change at one of the discontinuities of the net heating (the CO
// ladder break, T = 100 K, T = 3000 K) converges to the jump.
// Returns the root; *status 0 converged, 1 iteration limit.
__device__ __forceinline__ double thermal_root64(const ThermalCtx& c, const LineParams& lp,
                                                 const CoLevel* __restrict__ co, int n_bisect,
                                                 int max_newton, double tol, int* status,
                                                 int* iters) {
  double t_lo = 10.0, t_hi = 1e5;
  for (int k = 0; k < n_bisect; ++k) {
    double t_mid = sqrt(t_lo * t_hi);
    if (net_heating64(t_mid, c, lp, co) > 0.0) t_lo = t_mid; else t_hi = t_mid;
  }
  double t = sqrt(t_lo * t_hi);
  double dx_old = t_hi - t_lo, dx = dx_old;
  *status = 1;
  int k;
  for (k = 0; k < max_newton; ++k) {
    double f = net_heating64(t, c, lp, co);
    double eps = t * 1e-7;
    double df = (net_heating64(t + eps, c, lp, co) - f) / eps;
    if (f > 0.0) t_lo = t; else t_hi = t;
    if (f == 0.0) { *status = 0; ++k; break; }
    double tn = t - f / df;
    if (!(df != 0.0) || !(tn > t_lo && tn < t_hi) || fabs(2.0 * f) > fabs(dx_old * df)) {
      dx_old = dx;
      tn = 0.5 * (t_lo + t_hi);
    } else {
      dx_old = dx;
    }
    dx = tn - t;
    t = tn;
    if (fabs(dx) <= tol * t || t_hi - t_lo <= tol * t) { *status = 0; ++k; break; }
  }
  *iters = k;
  return t;
}

}  // namespace p3d
