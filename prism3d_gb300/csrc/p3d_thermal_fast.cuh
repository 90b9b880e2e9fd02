// p3d_thermal_fast.cuh -- net heating for the steady-state driver.
//
// Same terms as rust/src/thermal.rs:50-184, rearranged for the GB300's
// FP64/FP32 balance:
//  * every power law T^a is exp(a ln T) from one shared logarithm (one log +
//    one exp instead of a pow);
//  * the CO ladder's Boltzmann factors exp(-T_u(J)/T) use
//    T_u(J) - T_u(J-1) = 2 theta J:  b_J = b_{J-1} q_J,  q_J = q_{J-1} q_1
//    (two multiplies per level instead of an exp; relative drift <= J^2 eps);
//  * an FP32 twin evaluates the same terms on per-cell coefficients
//    pre-scaled by 1 / Gamma_fixed and returns the sum of |terms| S, so a
//    sign is certified when |net| > kCertify S (each term's FP32 error is
//    < 1e-5 of itself); otherwise the FP64 value decides.
#pragma once

#include "p3d_common.cuh"
#include "p3d_thermal.cuh"

namespace p3d {

constexpr double kLn100 = 4.605170185988091368;  // ln 100
constexpr double kLn300 = 5.703782474656201152;  // ln 300
constexpr double kLn10 = 2.302585092994045684;
constexpr float kCertify = 1e-4f;

// Two-level fraction and line energy for one line.
__device__ __forceinline__ double line64(double q, const double* l, double inv_t) {
  double r_lu = (l[3] / l[4]) * q * exp(-l[2] * inv_t);
  double r_ul = l[1] + q;
  return r_lu / (r_lu + r_ul) * l[1] * kHPlanck * l[0];
}

__device__ __forceinline__ double net_heating_fast64_body(double t, const ThermalCtx& c,
                                                     const LineParams& lp,
                                                     const CoLevel* __restrict__ co,
                                                     double theta2) {
  const double lt = log(t);
  const double l01 = lt - kLn100;
  const double sqrt_t = sqrt(t);
  const double inv_t = 1.0 / t;
  double net = c.gamma_fixed + c.gg_coeff * sqrt_t * (c.t_dust - t);
  {  // [CII] 158
    const double* l = lp.cii;
    double b = exp(-l[2] * inv_t);
    double q = 8.63e-6 / (l[4] * sqrt_t) * 2.15 * b * c.n_e + 8.0e-10 * exp(0.07 * l01) * c.n_hi +
               4.9e-10 * exp(0.12 * l01) * c.n_h2;
    double r_lu = (l[3] / l[4]) * q * b;
    net -= c.n_cp_nh * (r_lu / (r_lu + l[1] + q)) * l[1] * kHPlanck * l[0];
  }
  const double e039 = exp(0.39 * l01);
  net -= c.n_o_nh * line64(9.2e-12 * exp(0.67 * lt) * c.n_hi + 4.5e-12 * exp(0.64 * lt) * c.n_h2 +
                               1.4e-8 * e039 * c.n_e, lp.oi63, inv_t);
  net -= c.n_o_nh * line64(4.0e-12 * exp(0.60 * lt) * c.n_hi + 2.0e-12 * exp(0.58 * lt) * c.n_h2 +
                               5.0e-9 * e039 * c.n_e, lp.oi145, inv_t);
  {
    double t03 = exp(0.3 * l01);
    double q = 1.0e-10 * t03 * c.n_hi + 5.0e-11 * t03 * c.n_h2 + 2.0e-7 * (10.0 / sqrt_t) * c.n_e;
    net -= c.n_c_nh * (line64(q, lp.ci, inv_t) + line64(q, lp.ci + 5, inv_t));
  }
  {  // CO ladder
    const double g0 = 3.3e-11 * (0.1 * sqrt_t);
    const double t5 = 5.0 * t;
    const double q1 = exp(-theta2 * inv_t);
    double qj = q1, bj = 1.0, sum = 0.0;
    for (int k = 0; k < 40; ++k) {
      if (co[k].t_u >= t5) break;
      bj *= qj;  // exp(-T_u(J) / T), J = k + 1
      qj *= q1;
      double gam = g0 * co[k].j_factor * c.n_h2;
      double r_lu = co[k].g_ratio * gam * bj;
      sum += r_lu / (r_lu + co[k].a_co + gam) * co[k].ahv;
    }
    net -= c.n_co * sum;
  }
  if (t >= 100.0) {
    double x = fmin(fmax(lt / kLn10, 2.0), 4.5);
    double llh = -24.311 + x * (3.5692 + x * (-11.332 + x * (15.738 + x * (-10.581 +
                 x * (3.5803 + x * -0.48365)))));
    double llh2 = -24.311 + x * (4.6585 + x * (-14.272 + x * (19.779 + x * (-13.255 +
                  x * (4.4840 + x * -0.60504)))));
    double l0 = exp(llh * kLn10) * c.n_hi + exp(llh2 * kLn10) * c.n_h2;
    double lte = exp((-19.703 + 0.5 * x) * kLn10);
    net -= c.n_h2 * l0 * lte / fmax(l0 + lte, 1e-50);
  }
  if (t >= 3000.0) net -= c.n_hi * c.n_e * (2.41e-6 / sqrt_t * 0.486 * exp(-1.18e5 * inv_t)) *
                          10.2 * kEVtoErg;
  {
    double gg_cool = c.gg_coeff * sqrt_t * (t - c.t_dust);
    if (gg_cool > 0.0) net -= gg_cool;
  }
  net -= c.n_cp_nh * c.n_e * (4.67e-12 * exp(-0.6 * (lt - kLn300))) * kKBoltz * t;
  return net;
}

// Out of line for the mixed root, which calls it from several places: one
// copy keeps the mixed thermal kernel within the instruction cache.  The
// plain root inlines the body.
__device__ __noinline__ double net_heating_fast64(double t, const ThermalCtx& c,
                                                  const LineParams& lp,
                                                  const CoLevel* __restrict__ co,
                                                  double theta2) {
  return net_heating_fast64_body(t, c, lp, co, theta2);
}

// Per-cell FP32 coefficients, scaled by 1 / Gamma_fixed.
struct ThermalCtx32 {
  float gg, td, ne, nhi, nh2, cii, o63, o145, ci609, ci370, co, h2, lya, rec;
  double nhi64, nh264;  // H2 cooling weights stay FP64 (the fit cancels)
};

__device__ __forceinline__ ThermalCtx32 make_ctx32(const ThermalCtx& c, const LineParams& lp,
                                                   const CoLevel* co, double* scale) {
  double K = 1.0 / fmax(c.gamma_fixed, 1e-300);
  *scale = K;
  ThermalCtx32 f;
  f.gg = (float)(c.gg_coeff * K);
  f.td = (float)c.t_dust;
  f.ne = (float)c.n_e;
  f.nhi = (float)c.n_hi;
  f.nh2 = (float)c.n_h2;
  f.cii = (float)(c.n_cp_nh * lp.cii[1] * kHPlanck * lp.cii[0] * K);
  f.o63 = (float)(c.n_o_nh * lp.oi63[1] * kHPlanck * lp.oi63[0] * K);
  f.o145 = (float)(c.n_o_nh * lp.oi145[1] * kHPlanck * lp.oi145[0] * K);
  f.ci609 = (float)(c.n_c_nh * lp.ci[1] * kHPlanck * lp.ci[0] * K);
  f.ci370 = (float)(c.n_c_nh * lp.ci[6] * kHPlanck * lp.ci[5] * K);
  f.co = (float)(c.n_co * co[0].ahv * K);
  f.h2 = (float)(c.n_h2 * K);
  f.lya = (float)(c.n_hi * c.n_e * 10.2 * kEVtoErg * K);
  f.rec = (float)(c.n_cp_nh * c.n_e * kKBoltz * K);
  f.nhi64 = c.n_hi;
  f.nh264 = c.n_h2;
  return f;
}

__device__ __forceinline__ float line32(float q, float a_ul, float t_ul, float g_ratio,
                                        float inv_t) {
  float r_lu = g_ratio * q * expf(-t_ul * inv_t);
  return r_lu / (r_lu + a_ul + q);
}

// FP32 net heating / Gamma_fixed and the sum of |terms|.
// Branch points (the CO ladder break, T >= 100 K, T >= 3000 K) are decided
// on the FP64 temperature t64 so the FP32 and FP64 functions switch terms at
// the same temperatures.
__device__ __noinline__ float net_heating32(double t64, const ThermalCtx32& f,
                                               const float* __restrict__ lines32,
                                               const float* __restrict__ co32,
                                               const CoLevel* __restrict__ co, float* S) {
  const float t = (float)t64;
  // lines32: 4 floats per line (A, T_ul, g_u / g_l, g_l) for CII, OI 63,
  // OI 145, CI 609, CI 370; co32: 5 floats per CO level (T_u, A, g_u / g_l,
  // 1 + 0.1 J, A h nu / (A h nu)_{J=1}).
  const float lt = logf(t);
  const float l01 = lt - 4.6051702f;
  const float sqrt_t = sqrtf(t);
  const float inv_t = 1.0f / t;
  float heat = 1.0f + f.gg * sqrt_t * (f.td - t);
  float s = fabsf(1.0f) + fabsf(f.gg * sqrt_t * (f.td - t));
  float cool = 0.0f;
  {
    float b = expf(-lines32[1] * inv_t);
    float q = 8.63e-6f / (lines32[3] * sqrt_t) * 2.15f * b * f.ne +
              8.0e-10f * expf(0.07f * l01) * f.nhi + 4.9e-10f * expf(0.12f * l01) * f.nh2;
    float r_lu = lines32[2] * q * b;
    cool += f.cii * (r_lu / (r_lu + lines32[0] + q));
  }
  const float e039 = expf(0.39f * l01);
  cool += f.o63 * line32(9.2e-12f * expf(0.67f * lt) * f.nhi + 4.5e-12f * expf(0.64f * lt) * f.nh2 +
                             1.4e-8f * e039 * f.ne, lines32[4], lines32[5], lines32[6], inv_t);
  cool += f.o145 * line32(4.0e-12f * expf(0.60f * lt) * f.nhi + 2.0e-12f * expf(0.58f * lt) * f.nh2 +
                              5.0e-9f * e039 * f.ne, lines32[8], lines32[9], lines32[10], inv_t);
  {
    float t03 = expf(0.3f * l01);
    float q = 1.0e-10f * t03 * f.nhi + 5.0e-11f * t03 * f.nh2 + 2.0e-7f * (10.0f / sqrt_t) * f.ne;
    cool += f.ci609 * line32(q, lines32[12], lines32[13], lines32[14], inv_t);
    cool += f.ci370 * line32(q, lines32[16], lines32[17], lines32[18], inv_t);
  }
  {
    const float g0 = 3.3e-11f * (0.1f * sqrt_t);
    const double t5 = 5.0 * t64;
    float sum = 0.0f;
    for (int k = 0; k < 40; ++k) {
      const float* L = co32 + 5 * k;  // T_u, A, g_ratio, j_factor, ahv / ahv_1
      if (co[k].t_u >= t5) break;
      float gam = g0 * L[3] * f.nh2;
      float r_lu = L[2] * gam * expf(-L[0] * inv_t);
      sum += r_lu / (r_lu + L[1] + gam) * L[4];
    }
    cool += f.co * sum;
  }
  if (t64 >= 100.0) {
    double x = fmin(fmax((double)lt / kLn10, 2.0), 4.5);
    double llh = -24.311 + x * (3.5692 + x * (-11.332 + x * (15.738 + x * (-10.581 +
                 x * (3.5803 + x * -0.48365)))));
    double llh2 = -24.311 + x * (4.6585 + x * (-14.272 + x * (19.779 + x * (-13.255 +
                  x * (4.4840 + x * -0.60504)))));
    float lte = exp2f((float)((-19.703 + 0.5 * x) * 3.321928094887362));
    float lh = exp2f((float)(llh * 3.321928094887362));
    float lh2 = exp2f((float)(llh2 * 3.321928094887362));
    float l0 = lh * (float)f.nhi64 + lh2 * (float)f.nh264;
    cool += f.h2 * (l0 * (lte / fmaxf(l0 + lte, 1e-37f)));
  }
  if (t64 >= 3000.0) cool += f.lya * (2.41e-6f / sqrt_t * 0.486f * expf(-1.18e5f * inv_t));
  {
    float gg_cool = f.gg * sqrt_t * (t - f.td);
    if (gg_cool > 0.0f) cool += gg_cool;
  }
  cool += f.rec * (4.67e-12f * expf(-0.6f * (lt - 5.7037825f))) * t;
  *S = s + cool;
  return heat - cool;
}


// Plain FP64 root: 10 geometric bisections of [10, 1e5] K (thermal.rs:231-243)
// then a safeguarded Newton iteration with a forward-difference slope
// (bisection whenever the step leaves the bracket or does not halve the
// previous one) to |dT| <= tol T or a bracket narrower than tol T.  A sign
// change at a discontinuity of the net heating (the CO ladder break,
// T = 100 K, 3000 K) converges to the jump.
__device__ __forceinline__ double root_plain(const ThermalCtx& c, const LineParams& lp,
                                             const CoLevel* __restrict__ co, double theta2,
                                             double tol, int max_it, int* status, int* n64) {
  double t_lo = 10.0, t_hi = 1e5;
  for (int k = 0; k < 10; ++k) {
    double t_mid = sqrt(t_lo * t_hi);
    if (net_heating_fast64_body(t_mid, c, lp, co, theta2) > 0.0) t_lo = t_mid; else t_hi = t_mid;
  }
  int evals = 10;
  double t = sqrt(t_lo * t_hi);
  double dx_old = t_hi - t_lo, dx = dx_old;
  *status = 1;
  for (int k = 0; k < max_it; ++k) {
    double f = net_heating_fast64_body(t, c, lp, co, theta2);
    double eps = t * 1e-7;
    double df = (net_heating_fast64_body(t + eps, c, lp, co, theta2) - f) / eps;
    evals += 2;
    if (f > 0.0) t_lo = t; else t_hi = t;
    if (f == 0.0) { *status = 0; break; }
    double tn = t - f / df;
    if (!(df != 0.0) || !(tn > t_lo && tn < t_hi) || fabs(2.0 * f) > fabs(dx_old * df)) {
      dx_old = dx;
      tn = 0.5 * (t_lo + t_hi);
    } else {
      dx_old = dx;
    }
    dx = tn - t;
    t = tn;
    if (fabs(dx) <= tol * t || t_hi - t_lo <= tol * t) { *status = 0; break; }
  }
  *n64 = evals;
  return t;
}

// Mixed root: the same 10 bisection decisions as root_plain (the midpoints
// come from `mid_tab`, the FP64 bisection tree: node k has children 2k, 2k+1;
// a sign is taken from the FP32 evaluation when certified, else from FP64),
// so the bracket equals the plain path's.  Start: the previous root when it
// lies in the bracket (warm start; a root pinned at 10 K or 1e5 K is then
// confirmed by one FP64 evaluation), else a few FP32 Newton steps.  A
// discontinuity of the net heating within 1e-3 T is tested for a sign change
// across it (two FP64 evaluations; the root is then the discontinuity).
// Finish: up to three FP64 Newton steps with the FP32 slope of T's
// continuous piece (slope32; relative error ~1e-3), done once a step stays
// in the bracket and moves T by at most 1e-8 T (the slope error then bounds
// the remaining error by ~1e-11 T); else a two-point FP64 check for a jump
// of the net heating at T, else the safeguarded FP64 iteration of
// root_plain to tol.
// A warm cell replays the last full bisection's decisions when its inputs
// moved by less than margin / kReuseFactor (relative): the net heating's terms
// then change by far less than the smallest certified |net| of those
// decisions.
constexpr double kReuseFactor = 300.0;

// Discontinuities of the net heating nearest to t from below (<= t; 0 when
// none) and above (> t; infinity when none): H2 cooling from 100 K,
// Ly-alpha from 3000 K, CO level J from T_u(J) / 5 (the ladder's break
// T_u >= 5 T).  T_u(J) = (T_u(1) / 2) J (J + 1): the breaks next to t are
// those of the J around the real solution of J (J + 1) = 10 t / T_u(1).
__device__ __forceinline__ void jumps_around(double t, const CoLevel* __restrict__ co,
                                             double theta2, double* below, double* above) {
  double lo = 0.0, hi = INFINITY;
  if (100.0 <= t) lo = 100.0; else hi = 100.0;
  if (3000.0 <= t) lo = 3000.0; else hi = fmin(hi, 3000.0);
  const double j = 0.5 * (sqrt(1.0 + 40.0 * t / theta2) - 1.0);
  const int k0 = (int)fmin(fmax(j, 0.0), 40.0);  // co[k] is J = k + 1
#pragma unroll
  for (int dk = -2; dk <= 1; ++dk) {
    const int k = k0 + dk;
    if (k >= 0 && k < 40) {
      const double d = 0.2 * co[k].t_u;
      if (d <= t) lo = fmax(lo, d); else hi = fmin(hi, d);
    }
  }
  *below = lo;
  *above = hi;
}

// Slope of the FP32 twin (net / Gamma_fixed) at t by a difference inside
// t's continuous piece: a difference across a jump returns the jump's size
// over the step, and Newton then stalls short of a root next to the jump.
// Central with half-step 1e-3 t, cut to half the room to the nearest
// discontinuity; one-sided into the wider side (step <= 1e-3 t) when t sits
// within 4e-4 t of one.
__device__ __forceinline__ double slope32(double t, const ThermalCtx32& f32,
                                          const float* __restrict__ lines32,
                                          const float* __restrict__ co32,
                                          const CoLevel* __restrict__ co, double theta2) {
  double d_lo, d_hi;
  jumps_around(t, co, theta2, &d_lo, &d_hi);
  const double r_lo = t - d_lo, r_hi = d_hi - t;
  float S1, S2;
  const double room = fmin(r_lo, r_hi);
  if (room >= 4e-4 * t) {
    const double h = fmin(1e-3 * t, 0.5 * room);
    return (double)(net_heating32(t + h, f32, lines32, co32, co, &S1) -
                    net_heating32(t - h, f32, lines32, co32, co, &S2)) / (2.0 * h);
  }
  const double h = fmin(1e-3 * t, 0.5 * fmax(r_lo, r_hi));
  const float f0 = net_heating32(t, f32, lines32, co32, co, &S1);
  if (r_hi >= r_lo) return (double)(net_heating32(t + h, f32, lines32, co32, co, &S2) - f0) / h;
  return (double)(f0 - net_heating32(t - h, f32, lines32, co32, co, &S2)) / h;
}

__device__ __forceinline__ double root_mixed(const ThermalCtx& c, const LineParams& lp,
                                             const CoLevel* __restrict__ co, double theta2,
                                             const float* __restrict__ lines32,
                                             const float* __restrict__ co32,
                                             const double* __restrict__ mid_tab, double tol,
                                             int max_it, double t_warm, double delta,
                                             int* node_io, float* margin_io, int* status,
                                             int* n64) {
  double K;
  const ThermalCtx32 f32 = make_ctx32(c, lp, co, &K);
  double t_lo = 10.0, t_hi = 1e5;
  int evals = 0;
  if (*node_io >= 1024 && *node_io < 2048 && delta * kReuseFactor < (double)*margin_io) {
    // the inputs moved too little to flip any of the last solve's decisions
    // (each was certified with |net| >= margin sum|terms|): replay them
    const int path = *node_io - 1024;
    int node = 1;
    for (int k = 0; k < 10; ++k) {
      const double t_mid = __ldg(mid_tab + node);
      if ((path >> (9 - k)) & 1) { t_lo = t_mid; node = 2 * node + 1; } else { t_hi = t_mid; node = 2 * node; }
    }
  } else {
    int node = 1;
    float margin = INFINITY;
    for (int k = 0; k < 10; ++k) {
      double t_mid = __ldg(mid_tab + node);
      float S;
      float v = net_heating32(t_mid, f32, lines32, co32, co, &S);
      bool pos;
      if (fabsf(v) > kCertify * S) {
        pos = v > 0.0f;
        margin = fminf(margin, fabsf(v) / S);
      } else {
        const double f = net_heating_fast64(t_mid, c, lp, co, theta2);
        pos = f > 0.0;
        ++evals;
        margin = fminf(margin, S > 0.0f ? (float)(fabs(f) / (double)S) : 0.0f);
      }
      if (pos) { t_lo = t_mid; node = 2 * node + 1; } else { t_hi = t_mid; node = 2 * node; }
    }
    *node_io = node;
    *margin_io = margin == margin ? margin : 0.0f;
  }
  double t;
  // (closed: a root returned on a discontinuity can be a bracket end, e.g.
  // 100 K, a node of the bisection tree)
  if (t_warm >= t_lo && t_warm <= t_hi) {
    t = t_warm;
    // a root pinned at an end of [10, 1e5] K (the net heating keeps one
    // sign over the whole range, every decision went that way): a warm start
    // within tol of that end that keeps the sign leaves the root between the
    // end and t -- one FP64 evaluation instead of the polish below
    const bool at_lo = t_lo == 10.0 && t <= 10.0 * (1.0 + tol);
    const bool at_hi = t_hi == 1e5 && t >= 1e5 * (1.0 - tol);
    if (at_lo || at_hi) {
      const double f = net_heating_fast64(t, c, lp, co, theta2);
      ++evals;
      if (at_lo ? !(f > 0.0) : (f > 0.0)) {
        *status = 0;
        *n64 = evals;
        return t;
      }
      if (f > 0.0) t_lo = t; else t_hi = t;
      t = sqrt(t_lo * t_hi);
    }
  } else {
    t = sqrt(t_lo * t_hi);
    for (int k = 0; k < 4; ++k) {  // FP32 Newton inside the bracket
      float S;
      const float v = net_heating32(t, f32, lines32, co32, co, &S);
      const double d = slope32(t, f32, lines32, co32, co, theta2);
      double tn = t - (double)v / d;
      if (!(tn > t_lo && tn < t_hi)) break;
      bool small = fabs(tn - t) <= 1e-6 * t;
      t = tn;
      if (small) break;
    }
  }
  {  // a root on a discontinuity next to t: sign change across it
    double d_lo, d_hi;
    jumps_around(t, co, theta2, &d_lo, &d_hi);
    const double d = (t - d_lo <= d_hi - t) ? d_lo : d_hi;
    if (fabs(t - d) <= 1e-3 * t && d >= t_lo && d <= t_hi) {
      const double a = d * (1.0 - 0.5 * tol), b = d * (1.0 + 0.5 * tol);
      const double fa = net_heating_fast64(a, c, lp, co, theta2);
      const double fb = net_heating_fast64(b, c, lp, co, theta2);
      evals += 2;
      if (fa > 0.0 && !(fb > 0.0)) {
        *status = 0;
        *n64 = evals;
        return d;
      }
      double lo2 = t_lo, hi2 = t_hi;
      if (fa > 0.0) lo2 = fmax(lo2, a); else hi2 = fmin(hi2, a);
      if (fb > 0.0) lo2 = fmax(lo2, b); else hi2 = fmin(hi2, b);
      if (lo2 < hi2) { t_lo = lo2; t_hi = hi2; }
    }
  }
  if (!(t > t_lo && t < t_hi)) t = sqrt(t_lo * t_hi);
  const double slope = slope32(t, f32, lines32, co32, co, theta2) / K;
  *status = 1;
  for (int k = 0; k < 3; ++k) {  // up to three FP64 Newton steps
    double f = net_heating_fast64(t, c, lp, co, theta2);
    ++evals;
    if (f > 0.0) t_lo = fmax(t_lo, t); else t_hi = fmin(t_hi, t);
    if (f == 0.0) {
      *status = 0;
      *n64 = evals;
      return t;
    }
    double tn = t - f / slope;
    if (!(slope < 0.0 && tn > t_lo && tn < t_hi)) break;
    bool small = fabs(tn - t) <= fmax(1e-8, tol) * t;
    t = tn;
    if (small) {
      *status = 0;
      *n64 = evals;
      return t;
    }
  }
  {  // jump of the net heating at t: sign change across t (1 +- tol / 2)
    double a = t * (1.0 - 0.5 * tol), b = t * (1.0 + 0.5 * tol);
    double fa = net_heating_fast64(a, c, lp, co, theta2);
    double fb = net_heating_fast64(b, c, lp, co, theta2);
    evals += 2;
    if (fa > 0.0 && !(fb > 0.0)) {
      *status = 0;
      *n64 = evals;
      return t;
    }
    double lo2 = t_lo, hi2 = t_hi;
    if (fa > 0.0) lo2 = fmax(lo2, a); else hi2 = fmin(hi2, a);
    if (fb > 0.0) lo2 = fmax(lo2, b); else hi2 = fmin(hi2, b);
    if (lo2 < hi2) { t_lo = lo2; t_hi = hi2; }
    if (!(t > t_lo && t < t_hi)) t = sqrt(t_lo * t_hi);
  }
  double dx_old = t_hi - t_lo, dx = dx_old;
  for (int k = 0; k < max_it; ++k) {
    double f = net_heating_fast64(t, c, lp, co, theta2);
    ++evals;
    if (f > 0.0) t_lo = t; else t_hi = t;
    if (f == 0.0) { *status = 0; break; }
    double tn = t - f / slope;
    if (!(slope < 0.0) || !(tn > t_lo && tn < t_hi) || fabs(2.0 * f) > fabs(dx_old * slope)) {
      dx_old = dx;
      tn = 0.5 * (t_lo + t_hi);
    } else {
      dx_old = dx;
    }
    dx = tn - t;
    t = tn;
    if (fabs(dx) <= tol * t || t_hi - t_lo <= tol * t) { *status = 0; break; }
  }
  *n64 = evals;
  return t;
}

}  // namespace p3d
