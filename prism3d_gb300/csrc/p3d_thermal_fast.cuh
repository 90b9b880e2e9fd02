// p3d_thermal_fast.cuh -- net heating for the steady-state driver.
//
// Same terms as rust/src/thermal.rs:50-184, rearranged for the GB300's
// FP64/FP32 balance:
//  * every power law T^a is exp(a ln T) from one shared logarithm (one log +
//    one exp instead of a pow), and the exponentials are the table-driven
//    exp64 (p3d_fastexp.cuh: ten FP64 operations);
//  * the CO ladder's Boltzmann factors exp(-T_u(J)/T) use
//    T_u(J) - T_u(J-1) = 2 theta J:  b_J = b_{J-1} q_J,  q_J = q_{J-1} q_1
//    (two multiplies per level instead of an exp; relative drift <= J^2 eps);
//  * the ladder's break (T_u >= 5 T) is located once per evaluation (an FP32
//    estimate of J, settled by one or two FP64 compares with the level
//    table) instead of one FP64 compare per level;
//  * an FP32 twin evaluates the same terms on per-cell coefficients
//    pre-scaled by 1 / Gamma_fixed and returns the sum of |terms| S, so a
//    sign is certified when |net| > kCertify S (each term's FP32 error is
//    < 1e-5 of itself); otherwise the FP64 value decides.
#pragma once

#include "p3d_common.cuh"
#include "p3d_fastexp.cuh"
#include "p3d_thermal.cuh"

namespace p3d {

constexpr double kLn100 = 4.605170185988091368;  // ln 100
constexpr double kLn300 = 5.703782474656201152;  // ln 300
constexpr double kLn10 = 2.302585092994045684;
constexpr float kCertify = 1e-4f;

// Number of CO levels below the ladder's break: the k with co[k].t_u < t5
// (T_u increases with J, so they are the first ones).  T_u(J) = (T_u(1) / 2)
// J (J + 1), so J(J + 1) = 2 t5 / T_u(1) locates the break; the FP32 estimate
// is settled by the same FP64 compares the per-level test would make.
__device__ __forceinline__ int co_levels_below(double t5, const CoLevel* __restrict__ co) {
  const float r = (float)t5 / (float)co[0].t_u;
  int k = (int)fminf(fmaxf(0.5f * (sqrtf(1.0f + 8.0f * r) - 1.0f), 0.0f), 40.0f);
  while (k < 40 && co[k].t_u < t5) ++k;
  while (k > 0 && !(co[k - 1].t_u < t5)) --k;
  return k;
}

// Two-level fraction times the line's A h nu.
__device__ __forceinline__ double line64(double q, const LineFast& lf, int k, double inv_t) {
  const double r_lu = lf.g_ratio[k] * q * exp64(-lf.t_ul[k] * inv_t);
  return r_lu / (r_lu + lf.a[k] + q) * lf.e[k];
}

__device__ __forceinline__ double net_heating_fast64_body(double t, const ThermalCtx& c,
                                                     const LineFast& lf,
                                                     const CoLevel* __restrict__ co,
                                                     double theta2) {
  const double lt = log(t);
  const double l01 = lt - kLn100;
  const double sqrt_t = sqrt(t);
  const double inv_t = 1.0 / t;
  const double inv_sqrt_t = sqrt_t * inv_t;
  double net = c.gamma_fixed + c.gg_coeff * sqrt_t * (c.t_dust - t);
  {  // [CII] 158
    const double b = exp64(-lf.t_ul[0] * inv_t);
    const double q = lf.cii_ce * inv_sqrt_t * b * c.n_e + 8.0e-10 * exp64(0.07 * l01) * c.n_hi +
                     4.9e-10 * exp64(0.12 * l01) * c.n_h2;
    const double r_lu = lf.g_ratio[0] * q * b;
    net -= c.n_cp_nh * (r_lu / (r_lu + lf.a[0] + q)) * lf.e[0];
  }
  const double e039 = exp64(0.39 * l01);
  net -= c.n_o_nh * line64(9.2e-12 * exp64(0.67 * lt) * c.n_hi + 4.5e-12 * exp64(0.64 * lt) * c.n_h2 +
                               1.4e-8 * e039 * c.n_e, lf, 1, inv_t);
  net -= c.n_o_nh * line64(4.0e-12 * exp64(0.60 * lt) * c.n_hi + 2.0e-12 * exp64(0.58 * lt) * c.n_h2 +
                               5.0e-9 * e039 * c.n_e, lf, 2, inv_t);
  {
    const double t03 = exp64(0.3 * l01);
    const double q = 1.0e-10 * t03 * c.n_hi + 5.0e-11 * t03 * c.n_h2 + 2.0e-6 * inv_sqrt_t * c.n_e;
    net -= c.n_c_nh * (line64(q, lf, 3, inv_t) + line64(q, lf, 4, inv_t));
  }
  {  // CO ladder: sum_J A h nu r_lu / (r_lu + A + gamma), the fractions of
     // up to 8 levels combined over a common denominator (one division per
     // group instead of one per level)
    const double gn = 3.3e-11 * (0.1 * sqrt_t) * c.n_h2;
    const int nlev = co_levels_below(5.0 * t, co);
    const double q1 = exp64(-theta2 * inv_t);
    double qj = q1, bj = 1.0, sum = 0.0;
    for (int k0 = 0; k0 < nlev; k0 += 8) {
      const int k1 = k0 + 8 < nlev ? k0 + 8 : nlev;
      double num = 0.0, den = 1.0;
      for (int k = k0; k < k1; ++k) {
        bj *= qj;  // exp(-T_u(J) / T), J = k + 1
        qj *= q1;
        const double gam = gn * co[k].j_factor;
        const double r_lu = co[k].g_ratio * gam * bj;
        const double d = r_lu + co[k].a_co + gam;
        num = fma(num, d, r_lu * co[k].ahv * den);
        den *= d;
      }
      sum += num / den;
    }
    net -= c.n_co * sum;
  }
  if (t >= 100.0) {
    double x = fmin(fmax(lt / kLn10, 2.0), 4.5);
    double llh = -24.311 + x * (3.5692 + x * (-11.332 + x * (15.738 + x * (-10.581 +
                 x * (3.5803 + x * -0.48365)))));
    double llh2 = -24.311 + x * (4.6585 + x * (-14.272 + x * (19.779 + x * (-13.255 +
                  x * (4.4840 + x * -0.60504)))));
    double l0 = exp64(llh * kLn10) * c.n_hi + exp64(llh2 * kLn10) * c.n_h2;
    double lte = exp64((-19.703 + 0.5 * x) * kLn10);
    net -= c.n_h2 * l0 * lte / fmax(l0 + lte, 1e-50);
  }
  if (t >= 3000.0) net -= c.n_hi * c.n_e * (2.41e-6 * inv_sqrt_t * 0.486 * exp64(-1.18e5 * inv_t)) *
                          10.2 * kEVtoErg;
  {
    double gg_cool = c.gg_coeff * sqrt_t * (t - c.t_dust);
    if (gg_cool > 0.0) net -= gg_cool;
  }
  net -= c.n_cp_nh * c.n_e * (4.67e-12 * exp64(-0.6 * (lt - kLn300))) * kKBoltz * t;
  return net;
}

// The mixed root's form of the same net heating: the eight power laws of T
// in the line collision rates as products of u = T^0.01 (one exp64 and 22
// multiplies instead of eight exp64; each power a few ulp from the direct
// form, the (T / 100)^a factors as constants 100^-a times T^a).  The plain
// path keeps net_heating_fast64_body as it is (its FP64 solves are the
// reference's method; a change of its rounding moves which few cells
// chatter on a bisection node at tight tolerances).
constexpr double k100m007 = 0x1.72e94529230b1p-1;  // 100^-0.07
constexpr double k100m012 = 0x1.26a0103f59cb3p-1;  // 100^-0.12
constexpr double k100m039 = 0x1.53e22669d9ed8p-3;  // 100^-0.39
constexpr double k100m030 = 0x1.0137987dd704cp-2;  // 100^-0.30

struct TPowers {
  double p007, p012, p039, p067, p064, p060, p058, p030;  // (T/100)^0.07 ... T^0.67 ...
};

__device__ __forceinline__ TPowers t_powers_mixed(double lt) {
  TPowers w;
  const double u = exp64(0.01 * lt);
  const double u2 = u * u, u4 = u2 * u2, u8 = u4 * u4, u16 = u8 * u8, u32 = u16 * u16;
  const double u3 = u2 * u, u12 = u8 * u4, u6 = u4 * u2;
  w.p007 = k100m007 * (u4 * u3);
  w.p012 = k100m012 * u12;
  w.p039 = k100m039 * (u32 * (u4 * u3));
  w.p067 = (u32 * u32) * u3;
  w.p064 = u32 * u32;
  w.p060 = (u32 * u16) * u12;
  w.p058 = (u32 * u16) * (u8 * u2);
  w.p030 = k100m030 * ((u16 * u8) * u6);
  return w;
}

__device__ __forceinline__ double net_heating_mixed64_body(double t, const ThermalCtx& c,
                                                     const LineFast& lf,
                                                     const CoLevel* __restrict__ co,
                                                     double theta2) {
  const double lt = log(t);
  const double l01 = lt - kLn100;
  const double sqrt_t = sqrt(t);
  const double inv_t = 1.0 / t;
  const double inv_sqrt_t = sqrt_t * inv_t;
  const TPowers w = t_powers_mixed(lt);
  double net = c.gamma_fixed + c.gg_coeff * sqrt_t * (c.t_dust - t);
  {  // [CII] 158
    const double b = exp64(-lf.t_ul[0] * inv_t);
    const double q = lf.cii_ce * inv_sqrt_t * b * c.n_e + 8.0e-10 * w.p007 * c.n_hi +
                     4.9e-10 * w.p012 * c.n_h2;
    const double r_lu = lf.g_ratio[0] * q * b;
    net -= c.n_cp_nh * (r_lu / (r_lu + lf.a[0] + q)) * lf.e[0];
  }
  const double e039 = w.p039;
  net -= c.n_o_nh * line64(9.2e-12 * w.p067 * c.n_hi + 4.5e-12 * w.p064 * c.n_h2 +
                               1.4e-8 * e039 * c.n_e, lf, 1, inv_t);
  net -= c.n_o_nh * line64(4.0e-12 * w.p060 * c.n_hi + 2.0e-12 * w.p058 * c.n_h2 +
                               5.0e-9 * e039 * c.n_e, lf, 2, inv_t);
  {
    const double t03 = w.p030;
    const double q = 1.0e-10 * t03 * c.n_hi + 5.0e-11 * t03 * c.n_h2 + 2.0e-6 * inv_sqrt_t * c.n_e;
    net -= c.n_c_nh * (line64(q, lf, 3, inv_t) + line64(q, lf, 4, inv_t));
  }
  {  // CO ladder: sum_J A h nu r_lu / (r_lu + A + gamma), the fractions of
     // up to 8 levels combined over a common denominator (one division per
     // group instead of one per level)
    const double gn = 3.3e-11 * (0.1 * sqrt_t) * c.n_h2;
    const int nlev = co_levels_below(5.0 * t, co);
    const double q1 = exp64(-theta2 * inv_t);
    double qj = q1, bj = 1.0, sum = 0.0;
    for (int k0 = 0; k0 < nlev; k0 += 8) {
      const int k1 = k0 + 8 < nlev ? k0 + 8 : nlev;
      double num = 0.0, den = 1.0;
      for (int k = k0; k < k1; ++k) {
        bj *= qj;  // exp(-T_u(J) / T), J = k + 1
        qj *= q1;
        const double gam = gn * co[k].j_factor;
        const double r_lu = co[k].g_ratio * gam * bj;
        const double d = r_lu + co[k].a_co + gam;
        num = fma(num, d, r_lu * co[k].ahv * den);
        den *= d;
      }
      sum += num / den;
    }
    net -= c.n_co * sum;
  }
  if (t >= 100.0) {
    double x = fmin(fmax(lt / kLn10, 2.0), 4.5);
    double llh = -24.311 + x * (3.5692 + x * (-11.332 + x * (15.738 + x * (-10.581 +
                 x * (3.5803 + x * -0.48365)))));
    double llh2 = -24.311 + x * (4.6585 + x * (-14.272 + x * (19.779 + x * (-13.255 +
                  x * (4.4840 + x * -0.60504)))));
    double l0 = exp64(llh * kLn10) * c.n_hi + exp64(llh2 * kLn10) * c.n_h2;
    double lte = exp64((-19.703 + 0.5 * x) * kLn10);
    net -= c.n_h2 * l0 * lte / fmax(l0 + lte, 1e-50);
  }
  if (t >= 3000.0) net -= c.n_hi * c.n_e * (2.41e-6 * inv_sqrt_t * 0.486 * exp64(-1.18e5 * inv_t)) *
                          10.2 * kEVtoErg;
  {
    double gg_cool = c.gg_coeff * sqrt_t * (t - c.t_dust);
    if (gg_cool > 0.0) net -= gg_cool;
  }
  net -= c.n_cp_nh * c.n_e * (4.67e-12 * exp64(-0.6 * (lt - kLn300))) * kKBoltz * t;
  return net;
}

// Out of line for the mixed root, which calls it from several places: one
// copy keeps the mixed thermal kernel within the instruction cache.  The
// plain root inlines the body.
__device__ __noinline__ double net_heating_fast64(double t, const ThermalCtx& c,
                                                  const LineFast& lf,
                                                  const CoLevel* __restrict__ co,
                                                  double theta2) {
  return net_heating_mixed64_body(t, c, lf, co, theta2);
}

// ------------------------------------------- warp-cooperative FP64 net heating
// The five fine-structure lines and the 40 CO levels as one table of
// two-level lines, so that 32 lanes can evaluate one cell's lines with the
// same instructions (entry e on lane e % 32):
//   q = c1 T^a1 n_HI + c2 T^a2 n_H2 + c3 T^a3 exp(d3 / T) n_e,
//   r = g q exp(-t_ul / T),   term = n_x r / (r + a + q) e,
// n_x = n_C+ / n_H (0), n_O / n_H (1), n_C / n_H (2), n_CO (3).  Entries 0-4:
// [CII] 158, [OI] 63, [OI] 145, [CI] 609, [CI] 370 (their collision rates as
// in net_heating_fast64_body, the (T / 100)^a factors folded into c); 5-44:
// CO levels J = 1-40 (q = 3.3e-12 (1 + 0.1 J) T^0.5 n_H2; active below the
// ladder's break).
struct CoopLine {
  double c1, a1, c2, a2, c3, a3, d3, g, t_ul, a, e;
  int species;
};
constexpr int kCoopLines = 45;

__host__ __device__ inline CoopLine coop_line(int e, const LineFast& lf, const CoLevel* co) {
  CoopLine L{};
  const double l100 = 4.605170185988091368;  // ln 100
  if (e >= 5) {
    const CoLevel& v = co[e - 5];
    L.c2 = 3.3e-12 * v.j_factor;
    L.a2 = 0.5;
    L.g = v.g_ratio;
    L.t_ul = v.t_u;
    L.a = v.a_co;
    L.e = v.ahv;
    L.species = 3;
    return L;
  }
  L.g = lf.g_ratio[e];
  L.t_ul = lf.t_ul[e];
  L.a = lf.a[e];
  L.e = lf.e[e];
  if (e == 0) {
    L.c1 = 8.0e-10 * exp(-0.07 * l100); L.a1 = 0.07;
    L.c2 = 4.9e-10 * exp(-0.12 * l100); L.a2 = 0.12;
    L.c3 = lf.cii_ce; L.a3 = -0.5; L.d3 = -lf.t_ul[0];
    L.species = 0;
  } else if (e <= 2) {
    L.c1 = e == 1 ? 9.2e-12 : 4.0e-12; L.a1 = e == 1 ? 0.67 : 0.60;
    L.c2 = e == 1 ? 4.5e-12 : 2.0e-12; L.a2 = e == 1 ? 0.64 : 0.58;
    L.c3 = (e == 1 ? 1.4e-8 : 5.0e-9) * exp(-0.39 * l100); L.a3 = 0.39;
    L.species = 1;
  } else {
    L.c1 = 1.0e-10 * exp(-0.3 * l100); L.a1 = 0.3;
    L.c2 = 5.0e-11 * exp(-0.3 * l100); L.a2 = 0.3;
    L.c3 = 2.0e-6; L.a3 = -0.5;
    L.species = 2;
  }
  return L;
}

// Table entry L's cooling term at T (lt = ln T, inv_t = 1 / T).
__device__ __forceinline__ double coop_term(const CoopLine& L, double lt, double inv_t,
                                            const ThermalCtx& c) {
  double q = L.c2 * exp64(L.a2 * lt) * c.n_h2;
  if (L.c1 != 0.0) {
    q += L.c1 * exp64(L.a1 * lt) * c.n_hi;
    q += L.c3 * exp64(fma(L.d3, inv_t, L.a3 * lt)) * c.n_e;
  }
  const double r = L.g * q * exp64(-L.t_ul * inv_t);
  const double nx = L.species == 3 ? c.n_co
                    : (L.species == 0 ? c.n_cp_nh : (L.species == 1 ? c.n_o_nh : c.n_c_nh));
  return nx * (r / (r + L.a + q)) * L.e;
}

// The net heating's terms outside the table, given the table's sum `lines`.
__device__ __forceinline__ double coop_rest(double t, double lt, double sqrt_t, double inv_t,
                                            const ThermalCtx& c, double lines) {
  const double inv_sqrt_t = sqrt_t * inv_t;
  double net = c.gamma_fixed + c.gg_coeff * sqrt_t * (c.t_dust - t) - lines;
  if (t >= 100.0) {
    double x = fmin(fmax(lt / kLn10, 2.0), 4.5);
    double llh = -24.311 + x * (3.5692 + x * (-11.332 + x * (15.738 + x * (-10.581 +
                 x * (3.5803 + x * -0.48365)))));
    double llh2 = -24.311 + x * (4.6585 + x * (-14.272 + x * (19.779 + x * (-13.255 +
                  x * (4.4840 + x * -0.60504)))));
    double l0 = exp64(llh * kLn10) * c.n_hi + exp64(llh2 * kLn10) * c.n_h2;
    double lte = exp64((-19.703 + 0.5 * x) * kLn10);
    net -= c.n_h2 * l0 * lte / fmax(l0 + lte, 1e-50);
  }
  if (t >= 3000.0) net -= c.n_hi * c.n_e * (2.41e-6 * inv_sqrt_t * 0.486 * exp64(-1.18e5 * inv_t)) *
                          10.2 * kEVtoErg;
  {
    double gg_cool = c.gg_coeff * sqrt_t * (t - c.t_dust);
    if (gg_cool > 0.0) net -= gg_cool;
  }
  net -= c.n_cp_nh * c.n_e * (4.67e-12 * exp64(-0.6 * (lt - kLn300))) * kKBoltz * t;
  return net;
}

#ifdef __CUDA_ARCH__
// The FP64 net heating of one cell at t, evaluated by all 32 lanes of a
// warp together and returned to every lane: each lane takes the table
// entries lane and lane + 32 (the CO Boltzmann factors from exp64 directly
// rather than by recurrence), the remaining terms are computed on every
// lane, the line terms are summed by a butterfly and lane 0's sum is
// broadcast, so that every lane holds the same value.  Same terms as
// net_heating_fast64_body; the summation order differs (relative difference
// ~1e-15 of the terms).  On GB300 a warp's FP64 instruction holds its
// scheduler's FP64 unit as long with one active lane as with 32, so a
// warp evaluating one cell this way finishes ~5x sooner than a lane
// evaluating it alone: the thermal kernel uses it when the list is short.
__device__ __noinline__ double net_heating_coop64(double t, const ThermalCtx& c,
                                                  const CoopLine* __restrict__ tab,
                                                  const CoLevel* __restrict__ co,
                                                  double theta2) {
  const int lane = threadIdx.x & 31;
  const double lt = log(t);
  const double sqrt_t = sqrt(t);
  const double inv_t = 1.0 / t;
  const int nlev = co_levels_below(5.0 * t, co);
  double part = 0.0;
  for (int e = lane; e < kCoopLines; e += 32) {
    if (e >= 5 && e - 5 >= nlev) continue;
    part += coop_term(tab[e], lt, inv_t, c);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  part = __shfl_sync(0xffffffffu, part, 0);
  (void)theta2;
  return coop_rest(t, lt, sqrt_t, inv_t, c, part);
}
#elif defined(__CUDACC__)
// nvcc's host pass: the device definition above is the one that runs
__device__ __noinline__ double net_heating_coop64(double t, const ThermalCtx& c,
                                                  const CoopLine* __restrict__ tab,
                                                  const CoLevel* __restrict__ co,
                                                  double theta2);
#else
// Host builds (the CPU tests): the same terms, the table summed in order.
inline double net_heating_coop64(double t, const ThermalCtx& c, const CoopLine* tab,
                                 const CoLevel* co, double theta2) {
  const double lt = log(t);
  const double sqrt_t = sqrt(t);
  const double inv_t = 1.0 / t;
  const int nlev = co_levels_below(5.0 * t, co);
  double part = 0.0;
  for (int e = 0; e < kCoopLines; ++e)
    if (e < 5 || e - 5 < nlev) part += coop_term(tab[e], lt, inv_t, c);
  (void)theta2;
  return coop_rest(t, lt, sqrt_t, inv_t, c, part);
}
#endif

// Per-cell FP32 coefficients, scaled by 1 / Gamma_fixed.
struct ThermalCtx32 {
  float gg, td, ne, nhi, nh2, cii, o63, o145, ci609, ci370, co, h2, lya, rec;
};

__device__ __forceinline__ ThermalCtx32 make_ctx32(const ThermalCtx& c, const LineFast& lf,
                                                   const CoLevel* co, double* scale) {
  double K = 1.0 / fmax(c.gamma_fixed, 1e-300);
  *scale = K;
  ThermalCtx32 f;
  f.gg = (float)(c.gg_coeff * K);
  f.td = (float)c.t_dust;
  f.ne = (float)c.n_e;
  f.nhi = (float)c.n_hi;
  f.nh2 = (float)c.n_h2;
  f.cii = (float)(c.n_cp_nh * lf.e[0] * K);
  f.o63 = (float)(c.n_o_nh * lf.e[1] * K);
  f.o145 = (float)(c.n_o_nh * lf.e[2] * K);
  f.ci609 = (float)(c.n_c_nh * lf.e[3] * K);
  f.ci370 = (float)(c.n_c_nh * lf.e[4] * K);
  f.co = (float)(c.n_co * co[0].ahv * K);
  f.h2 = (float)(c.n_h2 * K);
  f.lya = (float)(c.n_hi * c.n_e * 10.2 * kEVtoErg * K);
  f.rec = (float)(c.n_cp_nh * c.n_e * kKBoltz * K);
  return f;
}

__device__ __forceinline__ float line32(float q, float a_ul, float t_ul, float g_ratio,
                                        float inv_t) {
  float r_lu = g_ratio * q * expf(-t_ul * inv_t);
  return r_lu / (r_lu + a_ul + q);
}

// The temperature-only parts of the FP32 twin that need FP64 work, for one
// node of the bisection tree (its midpoint t): the H2 cooling factors
// 10^llh, 10^llh2, 10^lte (FP64 polynomial fits that cancel to ~1e-2 in
// FP32) and the branch points (CO levels below the ladder's break, T >= 100
// K, T >= 3000 K).  The bisection evaluates at these nodes only, so its FP32
// evaluations run without an FP64 instruction.
struct BisectNode {
  float lh, lh2, lte;
  int info;  // levels below the CO break | 256 (T >= 100 K) | 512 (T >= 3000 K)
};

__device__ inline void h2_cooling_factors(double x, double* lh, double* lh2, double* lte) {
  const double llh = -24.311 + x * (3.5692 + x * (-11.332 + x * (15.738 + x * (-10.581 +
                     x * (3.5803 + x * -0.48365)))));
  const double llh2 = -24.311 + x * (4.6585 + x * (-14.272 + x * (19.779 + x * (-13.255 +
                      x * (4.4840 + x * -0.60504)))));
  *lh = exp(llh * kLn10);
  *lh2 = exp(llh2 * kLn10);
  *lte = exp((-19.703 + 0.5 * x) * kLn10);
}

__device__ inline BisectNode bisect_node(double t, const CoLevel* __restrict__ co) {
  BisectNode nd;
  nd.info = co_levels_below(5.0 * t, co) | (t >= 100.0 ? 256 : 0) | (t >= 3000.0 ? 512 : 0);
  double lh = 0.0, lh2 = 0.0, lte = 0.0;
  if (t >= 100.0) h2_cooling_factors(fmin(fmax(log10(t), 2.0), 4.5), &lh, &lh2, &lte);
  nd.lh = (float)lh;
  nd.lh2 = (float)lh2;
  nd.lte = (float)lte;
  return nd;
}

// FP32 net heating / Gamma_fixed and the sum of |terms|.
// Branch points (the CO ladder break, T >= 100 K, T >= 3000 K) are decided
// on the FP64 temperature t64 so the FP32 and FP64 functions switch terms at
// the same temperatures.  With nd (a bisection node at t64) the branch
// points and the H2 factors come from the node table.
__device__ __noinline__ float net_heating32(double t64, const ThermalCtx32& f,
                                               const float* __restrict__ lines32,
                                               const float* __restrict__ co32,
                                               const CoLevel* __restrict__ co, float* S,
                                               const BisectNode* __restrict__ nd = nullptr) {
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
  int info;
  float lh = 0.0f, lh2 = 0.0f, lte = 0.0f;
  if (nd) {
    info = nd->info;
    lh = nd->lh;
    lh2 = nd->lh2;
    lte = nd->lte;
  } else {
    info = co_levels_below(5.0 * t64, co) | (t64 >= 100.0 ? 256 : 0) | (t64 >= 3000.0 ? 512 : 0);
    if (info & 256) {
      const double x = fmin(fmax((double)lt / kLn10, 2.0), 4.5);
      const double llh = -24.311 + x * (3.5692 + x * (-11.332 + x * (15.738 + x * (-10.581 +
                         x * (3.5803 + x * -0.48365)))));
      const double llh2 = -24.311 + x * (4.6585 + x * (-14.272 + x * (19.779 + x * (-13.255 +
                          x * (4.4840 + x * -0.60504)))));
      lte = exp2f((float)((-19.703 + 0.5 * x) * 3.321928094887362));
      lh = exp2f((float)(llh * 3.321928094887362));
      lh2 = exp2f((float)(llh2 * 3.321928094887362));
    }
  }
  {
    const float g0 = 3.3e-11f * (0.1f * sqrt_t);
    const int nlev = info & 255;
    float sum = 0.0f;
    for (int k = 0; k < nlev; ++k) {
      const float* L = co32 + 5 * k;  // T_u, A, g_ratio, j_factor, ahv / ahv_1
      float gam = g0 * L[3] * f.nh2;
      float r_lu = L[2] * gam * expf(-L[0] * inv_t);
      sum += r_lu / (r_lu + L[1] + gam) * L[4];
    }
    cool += f.co * sum;
  }
  if (info & 256) {
    const float l0 = lh * f.nhi + lh2 * f.nh2;
    cool += f.h2 * (l0 * (lte / fmaxf(l0 + lte, 1e-37f)));
  }
  if (info & 512) cool += f.lya * (2.41e-6f / sqrt_t * 0.486f * expf(-1.18e5f * inv_t));
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
__device__ __forceinline__ double root_plain(const ThermalCtx& c, const LineFast& lp,
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
// the remaining error by ~1e-11 T); a step past an end of the bracket first
// tests for a root within tol of that end (one FP64 evaluation at tol/2
// inside it: a root there would otherwise be reached by bisection, ~20
// evaluations); else a two-point FP64 check for a jump of the net heating at
// T, else the safeguarded FP64 iteration of root_plain to tol.
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

// COOP: every lane of the warp runs this for the same cell (the control flow
// is then uniform) and each FP64 evaluation is net_heating_coop64 over the
// warp, with the table `coop`.
template <bool COOP = false>
__device__ __forceinline__ double root_mixed(const ThermalCtx& c, const LineFast& lf,
                                             const CoLevel* __restrict__ co, double theta2,
                                             const float* __restrict__ lines32,
                                             const float* __restrict__ co32,
                                             const double* __restrict__ mid_tab,
                                             const BisectNode* __restrict__ node_tab, double tol,
                                             int max_it, double t_warm, double delta,
                                             int* node_io, float* margin_io, int* status,
                                             int* n64, const CoopLine* coop = nullptr) {
  auto eval64 = [&](double x) -> double {
    if constexpr (COOP) return net_heating_coop64(x, c, coop, co, theta2);
    else return net_heating_fast64(x, c, lf, co, theta2);
  };
  double K;
  const ThermalCtx32 f32 = make_ctx32(c, lf, co, &K);
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
      float v = net_heating32(t_mid, f32, lines32, co32, co, &S, node_tab + node);
      bool pos;
      if (fabsf(v) > kCertify * S) {
        pos = v > 0.0f;
        margin = fminf(margin, fabsf(v) / S);
      } else {
        const double f = eval64(t_mid);
        pos = f > 0.0;
        ++evals;
        margin = fminf(margin, S > 0.0f ? (float)(fabs(f) / (double)S) : 0.0f);
      }
      if (pos) { t_lo = t_mid; node = 2 * node + 1; } else { t_hi = t_mid; node = 2 * node; }
    }
    *node_io = node;
    *margin_io = margin == margin ? margin : 0.0f;
  }
  // After the bracket: every FP64 evaluation of the finish below goes
  // through one call site in one loop, so the threads of a warp that are in
  // different phases (pinned check, jump tests, Newton polish, safeguarded
  // iteration) evaluate together; a warp then costs the largest number of
  // evaluations among its threads, not the sum over the phases they visit.
  enum {
    kPinned,    // warm root pinned at 10 K / 1e5 K: one evaluation at t
    kNearChk,   // test for a discontinuity within 1e-3 t (no evaluation)
    kNearA,     // sign at a = d (1 - tol/2) ...
    kNearB,     // ... and at b = d (1 + tol/2)
    kPrep,      // FP32 slope of T's continuous piece (no evaluation)
    kNewton,    // up to three FP64 Newton steps
    kJumpA,     // jump of the net heating at t: sign at t (1 - tol/2) ...
    kJumpB,     // ... and at t (1 + tol/2)
    kSafe,      // safeguarded Newton / bisection to tol
    kDone
  };
  double t, a = 0.0, b = 0.0, d_jump = 0.0, fa = 0.0, slope = 0.0, res = 0.0;
  double dx_old = 0.0, dx = 0.0;
  int ph, k = 0, st = 1;
  bool at_lo = false, tried_lo = false, tried_hi = false;
  // (closed: a root returned on a discontinuity can be a bracket end, e.g.
  // 100 K, a node of the bisection tree)
  if (t_warm >= t_lo && t_warm <= t_hi) {
    t = t_warm;
    // a root pinned at an end of [10, 1e5] K (the net heating keeps one
    // sign over the whole range, every decision went that way): a warm start
    // within tol of that end that keeps the sign leaves the root between the
    // end and t -- one FP64 evaluation instead of the polish below
    at_lo = t_lo == 10.0 && t <= 10.0 * (1.0 + tol);
    const bool at_hi = t_hi == 1e5 && t >= 1e5 * (1.0 - tol);
    ph = (at_lo || at_hi) ? kPinned : kNearChk;
  } else {
    t = sqrt(t_lo * t_hi);
    for (int q = 0; q < 4; ++q) {  // FP32 Newton inside the bracket
      float S;
      const float v = net_heating32(t, f32, lines32, co32, co, &S);
      const double dv = slope32(t, f32, lines32, co32, co, theta2);
      double tn = t - (double)v / dv;
      if (!(tn > t_lo && tn < t_hi)) break;
      bool small = fabs(tn - t) <= 1e-6 * t;
      t = tn;
      if (small) break;
    }
    ph = kNearChk;
  }
  while (ph != kDone) {
    if (ph == kNearChk) {  // a root on a discontinuity next to t: sign change across it
      double d_lo, d_hi;
      jumps_around(t, co, theta2, &d_lo, &d_hi);
      d_jump = (t - d_lo <= d_hi - t) ? d_lo : d_hi;
      if (fabs(t - d_jump) <= 1e-3 * t && d_jump >= t_lo && d_jump <= t_hi) {
        a = d_jump * (1.0 - 0.5 * tol);
        b = d_jump * (1.0 + 0.5 * tol);
        ph = kNearA;
      } else {
        ph = kPrep;
      }
    }
    if (ph == kPrep) {
      if (!(t > t_lo && t < t_hi)) t = sqrt(t_lo * t_hi);
      slope = slope32(t, f32, lines32, co32, co, theta2) / K;
      k = 0;
      ph = kNewton;
    }
    const double x = (ph == kNearA || ph == kJumpA) ? a : (ph == kNearB || ph == kJumpB) ? b : t;
    const double f = eval64(x);
    ++evals;
    switch (ph) {
      case kPinned:
        if (at_lo ? !(f > 0.0) : (f > 0.0)) {
          st = 0;
          res = t;
          ph = kDone;
          break;
        }
        if (f > 0.0) t_lo = t; else t_hi = t;
        t = sqrt(t_lo * t_hi);
        ph = kNearChk;
        break;
      case kNearA:
      case kJumpA:
        fa = f;
        ph = ph == kNearA ? kNearB : kJumpB;
        break;
      case kNearB:
      case kJumpB: {
        if (fa > 0.0 && !(f > 0.0)) {
          st = 0;
          res = ph == kNearB ? d_jump : t;
          ph = kDone;
          break;
        }
        double lo2 = t_lo, hi2 = t_hi;
        if (fa > 0.0) lo2 = fmax(lo2, a); else hi2 = fmin(hi2, a);
        if (f > 0.0) lo2 = fmax(lo2, b); else hi2 = fmin(hi2, b);
        if (lo2 < hi2) { t_lo = lo2; t_hi = hi2; }
        if (ph == kNearB) {
          ph = kPrep;
        } else {
          if (!(t > t_lo && t < t_hi)) t = sqrt(t_lo * t_hi);
          dx_old = t_hi - t_lo;
          dx = dx_old;
          k = 0;
          res = t;
          ph = max_it > 0 ? kSafe : kDone;
        }
        break;
      }
      case kNewton: {  // up to three FP64 Newton steps
        if (f > 0.0) t_lo = fmax(t_lo, t); else t_hi = fmin(t_hi, t);
        if (f == 0.0 || t_hi - t_lo <= tol * t) {  // (the latter: closed by an end check)
          st = 0;
          res = t;
          ph = kDone;
          break;
        }
        const double tn = t - f / slope;
        if (!(slope < 0.0 && tn > t_lo && tn < t_hi)) {
          // a step past an end of the bracket: the root may sit within tol of
          // that end (10 K, a discontinuity at a node such as 100 K, or a
          // node the outer iteration has pushed the cell's balance onto); one
          // evaluation at tol/2 inside that end settles it, once per end
          const double e_lo = t_lo * (1.0 + 0.5 * tol), e_hi = t_hi * (1.0 - 0.5 * tol);
          if (slope < 0.0 && tn <= t_lo && !tried_lo && e_lo < t_hi) {
            tried_lo = true;
            t = e_lo;
          } else if (slope < 0.0 && tn >= t_hi && !tried_hi && e_hi > t_lo) {
            tried_hi = true;
            t = e_hi;
          } else {
            ph = kJumpA;
          }
        } else {
          const bool small = fabs(tn - t) <= fmax(1e-8, tol) * t;
          t = tn;
          if (small) {
            st = 0;
            res = t;
            ph = kDone;
          } else if (++k == 3) {
            ph = kJumpA;
          }
        }
        if (ph == kJumpA) {  // jump of the net heating at t: sign change across t (1 +- tol / 2)
          a = t * (1.0 - 0.5 * tol);
          b = t * (1.0 + 0.5 * tol);
        }
        break;
      }
      default: {  // kSafe
        if (f > 0.0) t_lo = t; else t_hi = t;
        if (f == 0.0) {
          st = 0;
          res = t;
          ph = kDone;
          break;
        }
        double tn = t - f / slope;
        const double e_lo = t_lo * (1.0 + 0.5 * tol), e_hi = t_hi * (1.0 - 0.5 * tol);
        if (slope < 0.0 && tn <= t_lo && !tried_lo && e_lo < t_hi) {  // end checks as above
          tried_lo = true;
          dx_old = dx;
          tn = e_lo;
        } else if (slope < 0.0 && tn >= t_hi && !tried_hi && e_hi > t_lo) {
          tried_hi = true;
          dx_old = dx;
          tn = e_hi;
        } else if (!(slope < 0.0) || !(tn > t_lo && tn < t_hi) ||
                   fabs(2.0 * f) > fabs(dx_old * slope)) {
          dx_old = dx;
          tn = 0.5 * (t_lo + t_hi);
        } else {
          dx_old = dx;
        }
        dx = tn - t;
        t = tn;
        res = t;
        if (fabs(dx) <= tol * t || t_hi - t_lo <= tol * t) {
          st = 0;
          ph = kDone;
        } else if (++k >= max_it) {
          ph = kDone;
        }
        break;
      }
    }
  }
  *status = st;
  *n64 = evals;
  return res;
}

}  // namespace p3d
