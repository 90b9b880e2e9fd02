// p3d_newton.cuh -- batched per-cell implicit chemistry for the reduced network.
//
// Unknowns y = (x_HI, x_H2, x_C+, x_C, x_CO).  Rows:
//   0  dx_H2/dt = R x_HI - (k_pd + R_cr) x_H2          (rate equation)
//   1  x_HI + 2 x_H2 - 1 = 0                           (H conservation)
//   2  dx_C+/dt = k_ci x_C - a n_H (x_C+ + x_HCO+) x_C+ + k_co x_CO
//   3  dx_CO/dt = k_OH(x_H2) x_C - k_co x_CO
//   4  x_C+ + x_C + x_CO - X_C = 0                     (C conservation)
// i.e. the right-hand side of rust/src/chemistry.rs:35-49 with its two
// renormalisations written as constraints.  k_pd = kpd0 f_H2(N_H2) with
// N_H2 = u_h2 + ds n_H x_H2 (the cell's own half layer of its selected ray
// solved implicitly), k_co = kco0 f_CO(N_CO, N_H2) + 6 zeta.
//
// Pseudo-transient continuation: backward-Euler steps (1/dt) dy - J dy = f on
// the rate rows, constraints imposed exactly; the first step is pure Newton
// (1/dt = 0), a step that would make a species non-positive is retried with
// 1/dt = fastest rate / 10 (then x4), accepted steps divide 1/dt by `growth`.
// The unknowns are the relative changes w_i = dy_i / y_i (columns scaled by
// y), so species many orders below their element total keep relative
// precision.  Converged when every |w_i| <= rtol and every rate residual <=
// rtol of its production + destruction.  The 5x5 system is row-equilibrated
// and factorised with partial pivoting in registers: in FP64 (plain path) or
// in FP32 with FP64 residuals and two steps of iterative refinement (mixed
// path).
#pragma once

#include "p3d_common.cuh"
#include "p3d_phys.cuh"

namespace p3d {

// u_h2 / u_co: shielding columns of the selected ray at the start of the
// outer iteration; ds_own > 0 adds the cell's own H2 half layer
// ds_own n_H x_H2 to u_h2 inside the solve (implicit self-shielding).
struct ChemCell {
  double n_h, kci, acp, rh2, rcr, xc, hcop;
  double kpd0, kco0, kco_cr, u_h2, u_co, ds, b_dop;
  double fh2_fix, kpd_fix, kco_fix;  // used when ds == 0 (see chem_prepare)
  double koh_s = 1.0;                // multiplier of the C + OH -> CO rate
};

// Shielding factors and the photo rates they set, once per cell when the
// columns are fixed for the whole solve.
// FAST: the mixed path's form of the CO shielding (fsh_co).
template <bool FAST = false>
__device__ __forceinline__ void chem_prepare(ChemCell& p) {
  if (p.ds > 0.0) return;
  double d1, dh;
  p.fh2_fix = fsh_h2<FAST>(p.u_h2, p.b_dop, &d1);
  p.kpd_fix = p.kpd0 * p.fh2_fix;
  p.kco_fix = p.kco0 * fsh_co<FAST>(p.u_co, p.u_h2, &dh) + p.kco_cr;
}

__device__ __forceinline__ void chem5_eval(const ChemCell& p, const double* y, double* f,
                                           double (*J)[5], double* sc, double* fh2_out) {
  double x_hi = y[0], h = y[1], cp = y[2], c = y[3], co = y[4];
  double s = 10.0 * h;
  double x_oh = 1e-9 + 9e-8 * fmin(fmax(s, 0.0), 1.0);
  double dxoh = (s > 0.0 && s < 1.0) ? 9e-7 : 0.0;
  double koh = 1e-10 * p.koh_s * x_oh * p.n_h;
  double an = p.acp * p.n_h;
  double xe = cp + p.hcop;
  double f1, kpd, kco, dkpd_h = 0.0, dkco_h = 0.0;
  if (p.ds > 0.0) {  // own H2 half layer inside the solve
    double nh2 = p.u_h2 + p.ds * p.n_h * h;
    double d1, dh;
    f1 = fsh_h2(nh2, p.b_dop, &d1);
    double f2 = fsh_co(p.u_co, nh2, &dh);
    kpd = p.kpd0 * f1;
    kco = p.kco0 * f2 + p.kco_cr;
    dkpd_h = p.kpd0 * d1 * p.ds * p.n_h;
    dkco_h = p.kco0 * dh * p.ds * p.n_h;
  } else {  // shielding fixed by the columns of the iteration
    f1 = p.fh2_fix;
    kpd = p.kpd_fix;
    kco = p.kco_fix;
  }
  *fh2_out = f1;
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int k = 0; k < 5; ++k) J[r][k] = 0.0;
  f[0] = p.rh2 * x_hi - (kpd + p.rcr) * h;
  f[1] = x_hi + 2.0 * h - 1.0;
  f[2] = p.kci * c - an * xe * cp + kco * co;
  f[3] = koh * c - kco * co;
  f[4] = cp + c + co - p.xc;
  J[0][0] = p.rh2;
  J[0][1] = -(kpd + p.rcr) - h * dkpd_h;
  J[1][0] = 1.0;
  J[1][1] = 2.0;
  J[2][1] = co * dkco_h;
  J[2][2] = -an * (xe + cp);
  J[2][3] = p.kci;
  J[2][4] = kco;
  J[3][1] = 1e-10 * p.koh_s * dxoh * p.n_h * c - co * dkco_h;
  J[3][3] = koh;
  J[3][4] = -kco;
  J[4][2] = 1.0;
  J[4][3] = 1.0;
  J[4][4] = 1.0;
  sc[0] = p.rh2 * x_hi + (kpd + p.rcr) * h;
  sc[1] = 1.0;
  sc[2] = p.kci * c + an * xe * cp + kco * co;
  sc[3] = koh * c + kco * co;
  sc[4] = p.xc;
}

// In-register LU with partial pivoting; returns false on a zero pivot.
template <typename R>
__device__ __forceinline__ bool lu5(R (*A)[5], int* perm) {
#pragma unroll
  for (int k = 0; k < 5; ++k) perm[k] = k;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    int piv = k;
    R best = fabs(A[k][k]);
#pragma unroll
    for (int r = k + 1; r < 5; ++r)
      if (fabs(A[r][k]) > best) { best = fabs(A[r][k]); piv = r; }
    if (!(best > R(0))) return false;
    if (piv != k) {
#pragma unroll
      for (int c = 0; c < 5; ++c) { R t = A[k][c]; A[k][c] = A[piv][c]; A[piv][c] = t; }
      int t = perm[k]; perm[k] = perm[piv]; perm[piv] = t;
    }
    R inv = R(1) / A[k][k];
#pragma unroll
    for (int r = k + 1; r < 5; ++r) {
      R m = A[r][k] * inv;
      A[r][k] = m;
#pragma unroll
      for (int c = k + 1; c < 5; ++c) A[r][c] -= m * A[k][c];
    }
  }
  return true;
}

template <typename R>
__device__ __forceinline__ void lu5_solve(const R (*LU)[5], const int* perm, const double* b,
                                          double* x) {
  R y[5];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    R s = (R)b[perm[r]];
#pragma unroll
    for (int c = 0; c < r; ++c) s -= LU[r][c] * y[c];
    y[r] = s;
  }
#pragma unroll
  for (int r = 4; r >= 0; --r) {
    R s = y[r];
#pragma unroll
    for (int c = r + 1; c < 5; ++c) s -= LU[r][c] * y[c];
    y[r] = s / LU[r][r];
  }
#pragma unroll
  for (int r = 0; r < 5; ++r) x[r] = (double)y[r];
}

// Solve A d = b (A, b row-equilibrated).  MIXED: factor and solve in FP32;
// the Newton iteration around it evaluates the nonlinear residual f in FP64,
// so each iteration refines the previous one's FP32 solve (the iteration
// converges to the FP64 root; the contraction per step is the FP32 solve's
// relative error, ~1e-6).
template <bool MIXED>
__device__ __forceinline__ bool solve5(const double (*A)[5], const double* b, double* d) {
  if (!MIXED) {
    double LU[5][5];
    int perm[5];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) LU[r][c] = A[r][c];
    if (!lu5<double>(LU, perm)) return false;
    lu5_solve<double>(LU, perm, b, d);
    return true;
  } else {
    float LU[5][5];
    int perm[5];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) LU[r][c] = (float)A[r][c];
    if (!lu5<float>(LU, perm)) return false;
    lu5_solve<float>(LU, perm, b, d);
    return true;
  }
}

// Species advanced by each rate row (-1: constraint row).
__device__ __forceinline__ constexpr int ode_species(int r) {
  return r == 0 ? 1 : (r == 2 ? 2 : (r == 3 ? 4 : -1));
}

// Returns 0 converged, 1 iteration limit.  y in-out; *fh2 = f_H2 at the
// final y; *iters = iterations used.
template <bool MIXED>
__device__ __forceinline__ int chem_steady_cell(const ChemCell& p, double* y, int max_iter,
                                                double rtol, double growth, double* fh2,
                                                int* iters) {
  double inv_dt = 0.0;
  int it;
  int status = 1;
  for (it = 0; it < max_iter; ++it) {
    double f[5], J[5][5], d[5], sc[5], yn[5];
    chem5_eval(p, y, f, J, sc, fh2);
    bool ok;
    if (MIXED) {
      // FP32 system: columns scaled by y, rows equilibrated, FP64 residual
      float A[5][5], b[5];
      int perm[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        int os = ode_species(r);
        float m = 0.0f;
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          double a = (os >= 0) ? -J[r][c] + (c == os ? inv_dt : 0.0) : J[r][c];
          A[r][c] = (float)(a * y[c]);
          m = fmaxf(m, fabsf(A[r][c]));
        }
        float inv = 1.0f / m;
#pragma unroll
        for (int c = 0; c < 5; ++c) A[r][c] *= inv;
        // the row's FP64 residual scaled by the same FP32 factor as its
        // matrix row (an FP64 multiply, not a division, for the FP64 pipe)
        b[r] = (float)((os >= 0 ? f[r] : -f[r]) * (double)inv);
      }
      double bd[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) bd[r] = b[r];
      ok = lu5<float>(A, perm);
      if (ok) lu5_solve<float>(A, perm, bd, d);
    } else {
      double A[5][5], b[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        int os = ode_species(r);
        double m = 0.0;
        if (os >= 0) {
#pragma unroll
          for (int c = 0; c < 5; ++c) A[r][c] = -J[r][c];
          A[r][os] += inv_dt;
          b[r] = f[r];
        } else {
#pragma unroll
          for (int c = 0; c < 5; ++c) A[r][c] = J[r][c];
          b[r] = -f[r];
        }
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          A[r][c] *= y[c];
          m = fmax(m, fabs(A[r][c]));
        }
        double inv = 1.0 / m;
#pragma unroll
        for (int c = 0; c < 5; ++c) A[r][c] *= inv;
        b[r] *= inv;
      }
      ok = solve5<false>(A, b, d);
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      if (!(d[r] > -1.0)) ok = false;
      yn[r] = y[r] * (1.0 + d[r]);
    }
    if (!ok) {
      double lam = fmax(fabs(J[0][1]), fmax(fabs(J[2][2]), fabs(J[3][4])));
      inv_dt = (inv_dt == 0.0) ? lam / 10.0 + 1e-30 : inv_dt * 4.0;
      continue;
    }
    bool conv = true;
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      if (fabs(d[r]) > rtol) conv = false;
      if (ode_species(r) >= 0 && fabs(f[r]) > rtol * sc[r]) conv = false;
    }
#pragma unroll
    for (int r = 0; r < 5; ++r) y[r] = yn[r];
    if (conv) {
      status = 0;
      ++it;
      break;
    }
    inv_dt /= growth;
  }
  if (p.ds > 0.0) {  // f_H2 at the final state (fixed by the columns otherwise)
    double f[5], J[5][5], sc[5];
    chem5_eval(p, y, f, J, sc, fh2);
  } else {
    *fh2 = p.fh2_fix;
  }
  *iters = it;
  return status;
}

}  // namespace p3d
