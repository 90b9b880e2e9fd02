// p3d_common.cuh -- shared definitions for the sm_103a kernels of prism3d_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace p3d {

// CGS constants (prism3d/utils/constants.py, rust/src/constants.rs).
constexpr double kHPlanck = 6.62607015e-27;
constexpr double kKBoltz = 1.380649e-16;
constexpr double kEVtoErg = 1.602176634e-12;
constexpr double kAVperNH = 5.34e-22;
constexpr double kXOTotal = 2.94e-4;
constexpr double kFHabing = 1.6e-3;
constexpr double kEFUVMean = 10.0 * 1.602176634e-12;

// Fine-structure line parameters [freq, A, T_ul, g_u, g_l] in the order the
// reference's solve_thermal_vec receives them (rust/src/thermal.rs:297-300).
struct LineParams {
  double cii[5];
  double oi63[5];
  double oi145[5];
  double ci[10];
};

// Line constants of the five fine-structure lines in the order CII 158,
// OI 63, OI 145, CI 609, CI 370 (from LineParams [freq, A, T_ul, g_u, g_l]),
// formed once on the host so the FP64 evaluation divides by none of them:
// A, T_ul, g_u / g_l, A h nu, and the [CII] electron-excitation prefactor
// 8.63e-6 x 2.15 / g_l (times b / sqrt(T)).
struct LineFast {
  double a[5], t_ul[5], g_ratio[5], e[5];
  double cii_ce;
};

__host__ __device__ inline LineFast make_line_fast(const LineParams& lp) {
  const double* L[5] = {lp.cii, lp.oi63, lp.oi145, lp.ci, lp.ci + 5};
  LineFast f;
  for (int k = 0; k < 5; ++k) {
    f.a[k] = L[k][1];
    f.t_ul[k] = L[k][2];
    f.g_ratio[k] = L[k][3] / L[k][4];
    f.e[k] = L[k][1] * kHPlanck * L[k][0];
  }
  f.cii_ce = 8.63e-6 / lp.cii[4] * 2.15;
  return f;
}

// CO rotational ladder J_u = 1..40 (rust/src/thermal.rs:13-41): T_u, A,
// g_u/g_l, 1 + 0.1 J, A h nu.  Filled once per device by the host.
struct CoLevel {
  double t_u, a_co, g_ratio, j_factor, ahv;
};

// Per-cell thermal context (rust/src/thermal.rs:286-295).
struct ThermalCtx {
  double gamma_fixed, gg_coeff, t_dust, n_e, n_hi, n_h2, n_co, n_cp_nh, n_o_nh, n_c_nh;
};

// Device-side error word: kernels OR flags into it; the host reads it after
// the work that could raise it.
enum : unsigned int {
  kErrNone = 0u,
  kErrNewtonLimit = 1u,   // a bounded Newton loop ended unconverged
  kErrNonFinite = 2u,     // a non-finite value reached an output
  kErrBadIndex = 4u,      // an index check failed (access skipped)
};

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Fixed launch shape: grid-stride loops with at most kMaxBlocksPerSM blocks
// per SM on the 152-SM GB300.
constexpr int kThreads = 256;
inline unsigned grid_for(int64_t n, int sms, int per_sm = 8) {
  int64_t b = ceil_div(n, kThreads);
  int64_t cap = (int64_t)sms * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace p3d
