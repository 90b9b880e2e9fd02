// p3d_network.cu -- full chemical network on the device: RHS and constrained
// steady state, one warp per cell.
//
// The network is data: a reaction table with the rate laws of
// ChemistrySolver._rhs (prism3d/chemistry/solver.py:69-143) over the
// reactions of build_pdr_network() (prism3d/chemistry/network.py:186-896).
// p3d_network_create compiles the table into term lists:
//   F terms  per species, the (reaction, +-1) pairs in the reference's
//            accumulation order (reaction order; reactants, then products),
//   J terms  per non-zero Jacobian entry, the (reaction, partial, +-1)
//            triples,
// so that one warp evaluates F and J of a cell without atomics and with a
// fixed summation order.
//
// Steady state (replaces the BDF windows of solver.py:145-225): Newton /
// pseudo-transient continuation in relative variables w = dy / y on
//   F_i(y) = 0                       for the ordinary species rows,
//   sum_i c_ei y_i = total_e         one row per element (H, C, O, S, Si,
//                                    Fe, He; totals of the initial state),
//   y_e = sum of cations             the electron row (charge neutrality as
//                                    solver.py:380-386 imposes it).
// The element row replaces the equation of the most abundant single-element
// species of that element, so the replaced equations hold at the solution.
// Rows are equilibrated by their largest entry.  Lane r owns row r; the LU
// factorisation uses implicit partial pivoting (warp arg-max, pivot row
// broadcast from shared memory).  MIXED factorises in FP32 and refines the
// FP32 solution twice with FP64 residuals of the FP64 matrix; F, J and the
// convergence test stay FP64 in both paths.
//
// Post-processing (reference species layout only): the analytic H+/e-
// correction (solver.py:227-281) and the conservation fix-up
// (solver.py:345-388) in the reference's operation order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/prism3d_gb300.h"
#include "p3d_capi_internal.cuh"
#include "p3d_common.cuh"

namespace p3d {
namespace net {

constexpr int kMaxSpecies = 32;
constexpr int kMaxReactions = 96;
constexpr int kMaxElements = 8;
constexpr int kMaxPivots = 8;
constexpr int kMaxFTerms = 768;
constexpr int kMaxJEntries = 1024;
constexpr int kMaxJTerms = 2048;
constexpr int kWarps = 4;  // warps (cells in flight) per block
constexpr int kLd = 33;    // padded row stride of the per-warp matrices
constexpr double kFloor = 1e-30;
constexpr double kGrowth = 2.0;
constexpr double kYTest = 1e-25;  // abundances at or below are not tested
constexpr int kRefine = 2;
constexpr double kRefineBelow = 0.5;  // refine when the last step was below
constexpr int kSwitch64 = 100;  // mixed: FP64 factorisation from this iteration on

// Reference species layout (solver.py:28-36).
enum RefIdx : int {
  kE = 0, kH = 1, kH2 = 2, kHp = 3, kHm = 4, kH2p = 5, kH3p = 6, kCp = 7, kC = 8, kCO = 9,
  kCH = 10, kCHp = 11, kCH2p = 12, kO = 13, kOp = 14, kOH = 15, kOHp = 16, kH2O = 17,
  kH2Op = 18, kH3Op = 19, kO2 = 20, kCOp = 21, kHCOp = 22, kS = 23, kSp = 24, kSi = 25,
  kSip = 26, kFe = 27, kFep = 28, kHe = 29, kHep = 30
};

struct Table {
  int ns, nr, nel, e_index, post_ok, nj;
  double pah_total, c_total, o_total;
  int rtype[kMaxReactions];
  int r0[kMaxReactions], r1[kMaxReactions];
  int shield[kMaxReactions];
  double a[kMaxReactions], b[kMaxReactions], g[kMaxReactions];
  int f_start[kMaxSpecies + 1];
  int16_t f_j[kMaxFTerms];
  int8_t f_s[kMaxFTerms];
  int16_t je_row[kMaxJEntries], je_col[kMaxJEntries];
  int je_start[kMaxJEntries + 1];
  int16_t jt_j[kMaxJTerms];
  int8_t jt_q[kMaxJTerms], jt_s[kMaxJTerms];
  double el[kMaxElements][kMaxSpecies];
  int piv_start[kMaxElements + 1];
  int piv[kMaxElements * kMaxPivots];
  double cation[kMaxSpecies];
};

// Per-warp shared memory.
struct Warp {
  double A[kMaxSpecies][kLd];
  float L[kMaxSpecies][kLd];
  double rate[kMaxReactions];
  double dr[kMaxReactions][3];
  double y[kMaxSpecies];
  double w[kMaxSpecies];
  double tot[kMaxElements];
  int perm[kMaxSpecies];
  int pivrow[kMaxElements];
};

struct Cond {
  double n_h, t, g0, a_v, zeta, fh2, fco;
};

__device__ __forceinline__ Cond load_cond(const double* __restrict__ cond, int64_t c) {
  const double* p = cond + 7 * c;
  return Cond{p[0], p[1], p[2], p[3], p[4], p[5], p[6]};
}

// Rate coefficient of reaction j (solver.py:101-127), without the n_H and
// abundance factors of the rate.
__device__ __forceinline__ double rate_coeff(const Table& T, int j, const Cond& c) {
  const int tp = T.rtype[j];
  const double a = T.a[j], b = T.b[j], g = T.g[j];
  if (tp == P3D_RX_TWO_BODY) {
    const double tc = fmin(fmax(c.t, 10.0), 41000.0);
    return a * pow(tc / 300.0, b) * exp(-g / tc);
  }
  if (tp == P3D_RX_PHOTO) {
    double k = a * c.g0 * exp(-g * c.a_v);
    if (T.shield[j] == 1) k *= c.fh2;
    else if (T.shield[j] == 2) k *= c.fco;
    return k;
  }
  if (tp == P3D_RX_CR) return a * c.zeta;
  return a * pow(c.t / 300.0, b);  // grain surface
}

// x(PAH-) and its derivative with respect to y_e (solver.py:76-88).
__device__ __forceinline__ void pah_minus(const Table& T, double y_e, const Cond& c, double* x,
                                          double* dx) {
  const double n_e = fmax(y_e, 1e-10) * c.n_h;
  if (c.g0 > 0.0 && n_e > 0.0) {
    const double psi = c.g0 * sqrt(c.t) / n_e;
    const double fm = fmax(500.0 / (psi + 500.0) * 0.5, 0.0);
    *x = T.pah_total * fm;
    *dx = (y_e > 1e-10) ? T.pah_total * (0.5 * 500.0 * psi / ((psi + 500.0) * (psi + 500.0)) / y_e)
                        : 0.0;
  } else {
    *x = T.pah_total * 0.4;
    *dx = 0.0;
  }
}

// Rates and partial derivatives of the lane's reactions (j = lane + 32 m)
// from the floored abundances in W.y; k[m] are the lane's coefficients.
__device__ __forceinline__ void eval_rates(const Table& T, Warp& W, const double k[3],
                                           const Cond& c, int lane, bool jac) {
  double pm, dpm;
  pah_minus(T, W.y[T.e_index], c, &pm, &dpm);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const int j = lane + 32 * m;
    if (j >= T.nr) break;
    const int tp = T.rtype[j], i0 = T.r0[j], i1 = T.r1[j];
    double r, p0 = 0.0, p1 = 0.0, p2 = 0.0;
    if (tp == P3D_RX_TWO_BODY) {
      const double xa = i0 >= 0 ? W.y[i0] : (i0 == P3D_NET_PAH_MINUS ? pm : 0.0);
      const double xb = i1 >= 0 ? W.y[i1] : (i1 == P3D_NET_PAH_MINUS ? pm : 0.0);
      r = k[m] * xa * xb * c.n_h;
      if (jac) {
        p0 = k[m] * xb * c.n_h;
        p1 = k[m] * xa * c.n_h;
        if (i0 == P3D_NET_PAH_MINUS) p2 = k[m] * xb * dpm * c.n_h;
        else if (i1 == P3D_NET_PAH_MINUS) p2 = k[m] * xa * dpm * c.n_h;
      }
    } else if (tp == P3D_RX_GRAIN_SURFACE) {
      r = k[m] * W.y[i0] * c.n_h * 0.5;
      p0 = k[m] * c.n_h * 0.5;
    } else {
      r = k[m] * (i0 >= 0 ? W.y[i0] : 0.0);
      p0 = k[m];
    }
    W.rate[j] = r;
    if (jac) {
      W.dr[j][0] = p0;
      W.dr[j][1] = p1;
      W.dr[j][2] = p2;
    }
  }
}

// F_r and the sum of |terms| (production + destruction) of species r.
__device__ __forceinline__ void eval_f(const Table& T, const Warp& W, int r, double* f,
                                       double* sc) {
  double acc = 0.0, s = 0.0;
  for (int t = T.f_start[r]; t < T.f_start[r + 1]; ++t) {
    const double v = W.rate[T.f_j[t]];
    if (T.f_s[t] > 0) acc += v;
    else acc -= v;
    s += v;
  }
  *f = acc;
  *sc = s;
}

// Pivot search: one warp reduction of a 32-bit key per column.  The key is
// the high word of |a| (FP64: sign, exponent, 20 mantissa bits; FP32: the
// whole |a|) with its low 5 bits replaced by 31 - lane, so the maximum picks
// the largest magnitude to 2^-15 relative (FP64) or 2^-18 (FP32) and the
// lowest lane on ties.  Excluded lanes pass key 0.  Returns the pivot lane,
// or -1 if every candidate is zero.
__device__ __forceinline__ int pivot_lane(unsigned int mag_bits, bool cand, int lane) {
  const unsigned int key = cand ? ((mag_bits & ~31u) | (unsigned int)(31 - lane)) : 0u;
  const unsigned int m = __reduce_max_sync(0xffffffffu, key);
  return (m & ~31u) ? 31 - (int)(m & 31u) : -1;
}

__device__ __forceinline__ unsigned int mag_hi(double a) {
  return (unsigned int)(__double_as_longlong(a) >> 32) & 0x7fffffffu;
}

__device__ __forceinline__ unsigned int mag32(float a) { return __float_as_uint(a) & 0x7fffffffu; }

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

// Solve with FP64 LU in place of W.A; b is the lane's right-hand side, the
// solution unknown r ends in lane r.  Returns false on a zero pivot.
__device__ bool lu_solve64(Warp& W, int ns, int lane, double b, double* x) {
  int my = lane < ns ? -1 : (1 << 20);
  for (int k = 0; k < ns; ++k) {
    const int p = pivot_lane(my < 0 ? mag_hi(W.A[lane][k]) : 0u, my < 0, lane);
    if (p < 0) return false;
    if (lane == p) my = k;
    if (lane == 0) W.perm[k] = p;
    const double bp = __shfl_sync(0xffffffffu, b, p);
    const double piv = W.A[p][k];
    if (my < 0) {
      const double l = W.A[lane][k] / piv;
      W.A[lane][k] = l;
      for (int j = k + 1; j < ns; ++j) W.A[lane][j] = fma(-l, W.A[p][j], W.A[lane][j]);
      b = fma(-l, bp, b);
    }
    __syncwarp();
  }
  double xr = 0.0;
  for (int k = ns - 1; k >= 0; --k) {
    const int p = W.perm[k];
    const double xk = __shfl_sync(0xffffffffu, lane == p ? b / W.A[lane][k] : 0.0, p);
    if (lane == k) xr = xk;
    if (my >= 0 && my < k) b = fma(-W.A[lane][k], xk, b);
  }
  *x = xr;
  return true;
}

// FP32 LU of W.L (no right-hand side); my = pivot step of the lane's row.
__device__ bool lu_factor32(Warp& W, int ns, int lane, int* my_out) {
  int my = lane < ns ? -1 : (1 << 20);
  for (int k = 0; k < ns; ++k) {
    const int p = pivot_lane(my < 0 ? mag32(W.L[lane][k]) : 0u, my < 0, lane);
    if (p < 0) return false;
    if (lane == p) my = k;
    if (lane == 0) W.perm[k] = p;
    const float piv = W.L[p][k];
    if (my < 0) {
      const float l = W.L[lane][k] / piv;
      W.L[lane][k] = l;
      for (int j = k + 1; j < ns; ++j) W.L[lane][j] = fmaf(-l, W.L[p][j], W.L[lane][j]);
    }
    __syncwarp();
  }
  *my_out = my;
  return true;
}

__device__ float lu_apply32(const Warp& W, int ns, int lane, int my, float b) {
  for (int k = 0; k < ns; ++k) {
    const int p = W.perm[k];
    const float bp = __shfl_sync(0xffffffffu, b, p);
    if (my > k && my < ns) b = fmaf(-W.L[lane][k], bp, b);
  }
  float xr = 0.f;
  for (int k = ns - 1; k >= 0; --k) {
    const int p = W.perm[k];
    const float xk = __shfl_sync(0xffffffffu, lane == p ? b / W.L[lane][k] : 0.f, p);
    if (lane == k) xr = xk;
    if (my >= 0 && my < k) b = fmaf(-W.L[lane][k], xk, b);
  }
  return xr;
}

// solver.py:227-281 then :345-388, one lane, reference operation order.
__device__ void post_process(const Table& T, double* y, const Cond& c) {
  {
    const double x_h = y[kH], x_cp = y[kCp];
    const double r_form = c.zeta * 0.46 * x_h;
    const double tc = fmax(c.t, 10.0);
    const double alpha = 2.753e-14 * pow(tc / 300.0, -0.745) + 1.0e-14 * sqrt(tc / 100.0);
    const double qa = alpha * c.n_h;
    const double qb = alpha * c.n_h * x_cp;
    const double qc = -r_form;
    if (qa > 0.0) {
      const double disc = qb * qb - 4.0 * qa * qc;
      if (disc >= 0.0) {
        double xhp = (-qb + sqrt(disc)) / (2.0 * qa);
        xhp = fmax(xhp, kFloor);
        if (x_cp < 1e-6) {
          y[kHp] = xhp;
          const int ions[16] = {kHp, kCp, kH3p, kHCOp, kSp, kSip, kFep, kOp,
                                kH2p, kOHp, kH2Op, kH3Op, kCHp, kCH2p, kCOp, kHep};
          double n_pos = 0.0;
          for (int q = 0; q < 16; ++q) n_pos += y[ions[q]];
          y[kE] = fmax(n_pos, kFloor);
        }
      }
    }
  }
  {
    const double h_major = y[kH] + 2.0 * y[kH2];
    const int hs[12] = {kHp, kHm, kH2p, kH3p, kOH, kOHp, kH2O, kH2Op, kH3Op, kCH, kCHp, kHCOp};
    const double hm[12] = {1, 1, 2, 3, 1, 1, 2, 2, 3, 1, 1, 1};
    double h_minor = 0.0;
    for (int q = 0; q < 12; ++q) h_minor += y[hs[q]] * hm[q];
    if (h_major > 0.0) {
      const double s = fmin(fmax(fmax(1.0 - h_minor, 0.9) / h_major, 0.8), 1.2);
      y[kH] *= s;
      y[kH2] *= s;
    }
    const double c_tot = T.c_total;
    const double c_major = y[kCp] + y[kC] + y[kCO];
    const int cs[5] = {kCH, kCHp, kCH2p, kCOp, kHCOp};
    double c_minor = 0.0;
    for (int q = 0; q < 5; ++q) c_minor += y[cs[q]];
    if (c_major > 0.0) {
      const double s = fmin(fmax(fmax(c_tot - c_minor, c_tot * 0.9) / c_major, 0.8), 1.2);
      y[kCp] *= s;
      y[kC] *= s;
      y[kCO] *= s;
    }
    double o_mol = y[kCO] + y[kOH] + y[kH2O] + y[kOp] + y[kOHp] + y[kH2Op] + y[kH3Op] + y[kCOp] +
                   y[kHCOp];
    o_mol += 2.0 * y[kO2];
    y[kO] = fmax(T.o_total - o_mol, kFloor);
    const int ions[16] = {kHp, kCp, kSp, kSip, kFep, kOp, kH2p, kH3p,
                          kOHp, kH2Op, kH3Op, kCHp, kCH2p, kCOp, kHCOp, kHep};
    double n_pos = 0.0;
    for (int q = 0; q < 16; ++q) n_pos += y[ions[q]];
    y[kE] = fmax(n_pos, kFloor);
    for (int q = 0; q < 31; ++q) y[q] = fmax(y[q], kFloor);
  }
}

__device__ __forceinline__ int next_cell(int* counter, int lane) {
  int c = 0;
  if (lane == 0) c = atomicAdd(counter, 1);
  return __shfl_sync(0xffffffffu, c, 0);
}

__global__ void __launch_bounds__(kWarps * 32)
    rhs_kernel(const Table* __restrict__ tab, int64_t n, const double* __restrict__ cond,
               const double* __restrict__ x, double* __restrict__ dxdt) {
  extern __shared__ __align__(16) unsigned char smem[];
  Warp& W = reinterpret_cast<Warp*>(smem)[threadIdx.x >> 5];
  const Table& T = *tab;
  const int lane = threadIdx.x & 31, ns = T.ns;
  for (int64_t cell = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5); cell < n;
       cell += (int64_t)gridDim.x * kWarps) {
    const Cond c = load_cond(cond, cell);
    double k[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) k[m] = (lane + 32 * m < T.nr) ? rate_coeff(T, lane + 32 * m, c) : 0.0;
    if (lane < ns) W.y[lane] = fmax(x[cell * ns + lane], kFloor);
    __syncwarp();
    eval_rates(T, W, k, c, lane, false);
    __syncwarp();
    if (lane < ns) {
      double f, sc;
      eval_f(T, W, lane, &f, &sc);
      dxdt[cell * ns + lane] = f;
    }
    __syncwarp();
  }
}

template <bool MIXED>
__global__ void __launch_bounds__(kWarps * 32)
    steady_kernel(const Table* __restrict__ tab, int64_t n, const double* __restrict__ cond,
                  double* __restrict__ x, int post, int max_iter, double rtol,
                  int32_t* __restrict__ status, int32_t* __restrict__ iters, int* counter,
                  unsigned int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  Warp& W = reinterpret_cast<Warp*>(smem)[threadIdx.x >> 5];
  const Table& T = *tab;
  const int lane = threadIdx.x & 31, ns = T.ns, nel = T.nel;
  const bool row = lane < ns;
  for (int64_t cell = next_cell(counter, lane); cell < n; cell = next_cell(counter, lane)) {
    const Cond c = load_cond(cond, cell);
    double k[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) k[m] = (lane + 32 * m < T.nr) ? rate_coeff(T, lane + 32 * m, c) : 0.0;
    double y = row ? fmax(x[cell * ns + lane], kFloor) : 0.0;
    if (row) W.y[lane] = y;
    __syncwarp();
    // element totals of the initial state (lane e)
    if (lane < nel) {
      double tot = 0.0;
      for (int i = 0; i < ns; ++i) tot += T.el[lane][i] * W.y[i];
      W.tot[lane] = tot;
    }
    double inv_dt = 0.0, wprev = 1.0;
    int it = 0;
    bool conv = false;
    while (it < max_iter) {
      eval_rates(T, W, k, c, lane, true);
      // pivot species of each element: the most abundant single-element one
      if (lane < nel) {
        int best = T.piv[T.piv_start[lane]];
        double bv = -1.0;
        for (int q = T.piv_start[lane]; q < T.piv_start[lane + 1]; ++q) {
          const int s = T.piv[q];
          const double v = T.el[lane][s] * W.y[s];
          if (v > bv) { bv = v; best = s; }
        }
        W.pivrow[lane] = best;
      }
      if (row)
        for (int j = 0; j < ns; ++j) W.A[lane][j] = 0.0;
      __syncwarp();
      double f = 0.0, sc = 0.0;
      if (row) eval_f(T, W, lane, &f, &sc);
      for (int e = lane; e < T.nj; e += 32) {
        double v = 0.0;
        for (int t = T.je_start[e]; t < T.je_start[e + 1]; ++t) {
          const double d = W.dr[T.jt_j[t]][T.jt_q[t]];
          if (T.jt_s[t] > 0) v += d;
          else v -= d;
        }
        W.A[T.je_row[e]][T.je_col[e]] = -v;
      }
      __syncwarp();
      double jd = row ? fabs(W.A[lane][lane]) : 0.0;
      int el_row = -1;
      for (int e = 0; e < nel; ++e)
        if (W.pivrow[e] == lane) el_row = e;
      bool ode = row && el_row < 0 && lane != T.e_index;
      double d = 0.0;
      if (ode) {
        W.A[lane][lane] += inv_dt;
        d = f;
      } else if (row && el_row >= 0) {
        double s = 0.0;
        for (int j = 0; j < ns; ++j) {
          W.A[lane][j] = T.el[el_row][j];
          s += T.el[el_row][j] * W.y[j];
        }
        d = W.tot[el_row] - s;
      } else if (row) {
        double s = 0.0;
        for (int j = 0; j < ns; ++j) {
          W.A[lane][j] = T.cation[j];
          s += T.cation[j] * W.y[j];
        }
        W.A[lane][lane] = -1.0;
        d = y - s;
      }
      __syncwarp();
      // column scaling by y (relative variables), then row scaling by the
      // power of two at the row's largest magnitude (exact; the largest
      // entry lands in [1, 2)).  The magnitude scan runs on the high words
      // and also flags Inf/NaN.
      bool finite = true;
      if (row) {
        unsigned int mx = 0u;
        for (int j = 0; j < ns; ++j) {
          const double a = W.A[lane][j] * W.y[j];
          W.A[lane][j] = a;
          mx = max(mx, mag_hi(a));
        }
        finite = mx < 0x7ff00000u && isfinite(d);
        double inv = 1.0;
        if (mx >= 0x00100000u) {
          const int biased = min(max(2046 - (int)(mx >> 20), 1), 2046);
          inv = __longlong_as_double((long long)biased << 52);
        }
        for (int j = 0; j < ns; ++j) {
          const double a = W.A[lane][j] * inv;
          W.A[lane][j] = a;
          if (MIXED && it < kSwitch64) W.L[lane][j] = (float)a;
        }
        d *= inv;
      }
      const bool res_ok = !ode || fabs(f) <= rtol * sc || y <= kYTest;
      const double lam = warp_max(jd);
      __syncwarp();
      bool ok = __all_sync(0xffffffffu, finite);
      double wr = 0.0;
      if (ok) {
        if (MIXED && it < kSwitch64) {
          int my;
          ok = lu_factor32(W, ns, lane, &my);
          if (ok) {
            wr = (double)lu_apply32(W, ns, lane, my, (float)d);
            // refinement only once the iteration is close to the root: the
            // pseudo-time steps before do not need an exact direction
            const int n_ref = wprev < kRefineBelow ? kRefine : 0;
            for (int rep = 0; rep < n_ref; ++rep) {
              if (row) W.w[lane] = wr;
              __syncwarp();
              double res = d;
              if (row)
                for (int j = 0; j < ns; ++j) res = fma(-W.A[lane][j], W.w[j], res);
              __syncwarp();
              wr += (double)lu_apply32(W, ns, lane, my, (float)res);
            }
          }
        } else {
          ok = lu_solve64(W, ns, lane, d, &wr);
        }
      }
      // a step that would make an abundance above kYTest non-positive is
      // rejected; smaller ones go to the floor
      ok = __all_sync(0xffffffffu, ok && (!row || (isfinite(wr) && (wr > -1.0 || y <= kYTest))));
      const bool step_ok = !row || fabs(wr) <= rtol || y <= kYTest;
      ++it;
      if (!ok) {
        inv_dt = (inv_dt == 0.0) ? lam / 10.0 + 1e-30 : inv_dt * 4.0;
        continue;
      }
      wprev = warp_max(row && y > kYTest ? fabs(wr) : 0.0);
      if (row) {
        y = fmax(y * (1.0 + fmax(wr, -1.0)), kFloor);
        W.y[lane] = y;
      }
      __syncwarp();
      conv = __all_sync(0xffffffffu, res_ok && step_ok);
      if (conv) break;
      inv_dt /= kGrowth;
    }
    if (lane == 0) {
      if (status) status[cell] = conv ? 0 : 1;
      if (iters) iters[cell] = it;
      if (!conv) atomicOr(err, kErrNewtonLimit);
      if (post && T.post_ok) post_process(T, W.y, c);
    }
    __syncwarp();
    if (row) x[cell * ns + lane] = W.y[lane];
    __syncwarp();
  }
}

}  // namespace net
}  // namespace p3d

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct p3d_network {
  int device = -1;
  int sms = 0;
  int blocks_per_sm[2] = {0, 0};
  cudaStream_t stream = nullptr;
  p3d::net::Table host;
  p3d::net::Table* table = nullptr;
  int* counter = nullptr;
  unsigned int* err = nullptr;
  // grow-only staging for the host-buffer entry points
  void* stage[4] = {};
  size_t cap[4] = {};
};

namespace p3d {
namespace net {

static size_t smem_bytes() { return sizeof(Warp) * kWarps; }

static int stage(p3d_network* h, int k, size_t bytes, void** out) {
  if (h->cap[k] < bytes) {
    if (h->stage[k]) {
      cudaStreamSynchronize(h->stream);
      cudaFree(h->stage[k]);
      h->stage[k] = nullptr;
      h->cap[k] = 0;
    }
    cudaError_t e = cudaMalloc(&h->stage[k], bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(P3D_ENOMEM, "network staging cudaMalloc(%zu): %s", bytes,
                       cudaGetErrorString(e));
    }
    h->cap[k] = bytes;
  }
  *out = h->stage[k];
  return P3D_OK;
}

static int check_device(const p3d_network* h) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != h->device)
    return set_error(P3D_EINVAL, "network was created on device %d, current device is %d",
                     h->device, dev);
  return P3D_OK;
}

// Term lists of the table (see the file header).
static int compile(p3d::net::Table& T, int ns, int nr, const int32_t* rtype, const double* alpha,
                   const double* beta, const double* gamma, const int32_t* reac,
                   const int32_t* prod, const int32_t* shield, int nel, const double* elc,
                   const int32_t* charge, int e_index) {
  memset(&T, 0, sizeof(T));
  T.ns = ns;
  T.nr = nr;
  T.nel = nel;
  T.e_index = e_index;
  for (int j = 0; j < nr; ++j) {
    if (rtype[j] < P3D_RX_TWO_BODY || rtype[j] > P3D_RX_GRAIN_SURFACE)
      return set_error(P3D_EINVAL, "reaction %d: unknown type %d", j, rtype[j]);
    T.rtype[j] = rtype[j];
    T.a[j] = alpha[j];
    T.b[j] = beta[j];
    T.g[j] = gamma[j];
    T.shield[j] = shield ? shield[j] : 0;
    for (int m = 0; m < 2; ++m) {
      const int i = reac[2 * j + m];
      if (i >= ns || i < P3D_NET_PAH_MINUS)
        return set_error(P3D_EINVAL, "reaction %d: reactant index %d", j, i);
    }
    for (int m = 0; m < 4; ++m) {
      const int i = prod[4 * j + m];
      if (i >= ns || i < P3D_NET_UNTRACKED)
        return set_error(P3D_EINVAL, "reaction %d: product index %d", j, i);
    }
    T.r0[j] = reac[2 * j];
    T.r1[j] = reac[2 * j + 1];
    if (rtype[j] != P3D_RX_TWO_BODY && T.r0[j] == P3D_NET_PAH_MINUS)
      return set_error(P3D_EINVAL, "reaction %d: PAH- only in two-body reactions", j);
    if (rtype[j] == P3D_RX_GRAIN_SURFACE && T.r0[j] < 0)
      return set_error(P3D_EINVAL, "reaction %d: grain-surface reaction needs a tracked reactant", j);
  }
  // F terms: per species, in reaction order, reactants then products
  int nf = 0;
  for (int i = 0; i < ns; ++i) {
    T.f_start[i] = nf;
    for (int j = 0; j < nr; ++j) {
      for (int m = 0; m < 2; ++m)
        if (reac[2 * j + m] == i) {
          if (nf >= kMaxFTerms) return set_error(P3D_EINVAL, "network too large (F terms)");
          T.f_j[nf] = (int16_t)j;
          T.f_s[nf++] = -1;
        }
      for (int m = 0; m < 4; ++m)
        if (prod[4 * j + m] == i) {
          if (nf >= kMaxFTerms) return set_error(P3D_EINVAL, "network too large (F terms)");
          T.f_j[nf] = (int16_t)j;
          T.f_s[nf++] = 1;
        }
    }
  }
  T.f_start[ns] = nf;
  // J terms: entry (row i, column c) <- +-dr[j][q]
  struct Term { int j, q, s; };
  std::map<std::pair<int, int>, std::vector<Term>> ent;
  for (int j = 0; j < nr; ++j) {
    int col[3] = {-1, -1, -1};
    if (T.rtype[j] == P3D_RX_TWO_BODY) {
      col[0] = T.r0[j] >= 0 ? T.r0[j] : -1;
      col[1] = T.r1[j] >= 0 ? T.r1[j] : -1;
      if (T.r0[j] == P3D_NET_PAH_MINUS || T.r1[j] == P3D_NET_PAH_MINUS) col[2] = e_index;
    } else {
      col[0] = T.r0[j] >= 0 ? T.r0[j] : -1;
    }
    for (int q = 0; q < 3; ++q) {
      if (col[q] < 0) continue;
      for (int m = 0; m < 2; ++m)
        if (reac[2 * j + m] >= 0) ent[{reac[2 * j + m], col[q]}].push_back({j, q, -1});
      for (int m = 0; m < 4; ++m)
        if (prod[4 * j + m] >= 0) ent[{prod[4 * j + m], col[q]}].push_back({j, q, 1});
    }
  }
  int ne = 0, nt = 0;
  for (auto& kv : ent) {
    if (ne >= kMaxJEntries || nt + (int)kv.second.size() > kMaxJTerms)
      return set_error(P3D_EINVAL, "network too large (Jacobian terms)");
    T.je_row[ne] = (int16_t)kv.first.first;
    T.je_col[ne] = (int16_t)kv.first.second;
    T.je_start[ne] = nt;
    for (const Term& t : kv.second) {
      T.jt_j[nt] = (int16_t)t.j;
      T.jt_q[nt] = (int8_t)t.q;
      T.jt_s[nt++] = (int8_t)t.s;
    }
    ++ne;
  }
  T.je_start[ne] = nt;
  T.nj = ne;
  // element rows and their candidate pivot species (made of that element alone)
  int np = 0;
  for (int e = 0; e < nel; ++e) {
    T.piv_start[e] = np;
    for (int i = 0; i < ns; ++i) {
      T.el[e][i] = elc[(size_t)e * ns + i];
      if (T.el[e][i] < 0.0) return set_error(P3D_EINVAL, "negative element count");
    }
    for (int i = 0; i < ns; ++i) {
      if (!(T.el[e][i] > 0.0)) continue;
      bool alone = true;
      for (int e2 = 0; e2 < nel; ++e2)
        if (e2 != e && elc[(size_t)e2 * ns + i] > 0.0) alone = false;
      if (alone && i != e_index) {
        if (np - T.piv_start[e] >= kMaxPivots) break;
        T.piv[np++] = i;
      }
    }
    if (np == T.piv_start[e])
      return set_error(P3D_EINVAL, "element %d has no species made of it alone", e);
  }
  T.piv_start[nel] = np;
  for (int i = 0; i < ns; ++i) T.cation[i] = charge[i] > 0 ? (double)charge[i] : 0.0;
  return P3D_OK;
}

template <bool MIXED>
static int launch_steady(p3d_network* h, int64_t n, const double* cond, double* x, int post,
                         int max_iter, double rtol, int32_t* status, int32_t* iters,
                         cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(h->counter, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_fail(e, "network counter reset");
  int64_t blocks = ceil_div(n, kWarps);
  const int64_t cap = (int64_t)h->sms * h->blocks_per_sm[MIXED ? 1 : 0];
  if (blocks > cap) blocks = cap;
  steady_kernel<MIXED><<<(unsigned)blocks, kWarps * 32, smem_bytes(), s>>>(
      h->table, n, cond, x, post, max_iter, rtol, status, iters, h->counter, h->err);
  e = cudaGetLastError();
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "network steady launch");
}

}  // namespace net
}  // namespace p3d

using namespace p3d;
using namespace p3d::net;

extern "C" {

int p3d_network_create(p3d_network_t** out, int32_t n_species, int32_t n_reactions,
                       const int32_t* rtype, const double* alpha, const double* beta,
                       const double* gamma, const int32_t* reactants, const int32_t* products,
                       const int32_t* shield, int32_t n_elements, const double* element_counts,
                       const int32_t* charge, int32_t e_index, double pah_total,
                       int32_t reference_layout, double c_total, double o_total) {
  if (!out) return set_error(P3D_EINVAL, "null handle pointer");
  *out = nullptr;
  if (n_species < 1 || n_species > kMaxSpecies)
    return set_error(P3D_EINVAL, "n_species=%d outside [1, %d]", n_species, kMaxSpecies);
  if (n_reactions < 1 || n_reactions > kMaxReactions)
    return set_error(P3D_EINVAL, "n_reactions=%d outside [1, %d]", n_reactions, kMaxReactions);
  if (n_elements < 0 || n_elements > kMaxElements)
    return set_error(P3D_EINVAL, "n_elements=%d outside [0, %d]", n_elements, kMaxElements);
  if (e_index < 0 || e_index >= n_species)
    return set_error(P3D_EINVAL, "e_index=%d outside the species", e_index);
  if (!rtype || !alpha || !beta || !gamma || !reactants || !products || !charge ||
      (n_elements > 0 && !element_counts))
    return set_error(P3D_EINVAL, "null array");
  if (reference_layout && n_species != 31)
    return set_error(P3D_EINVAL, "reference layout has 31 species, got %d", n_species);
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  p3d_network* h = new p3d_network();
  rc = compile(h->host, n_species, n_reactions, rtype, alpha, beta, gamma, reactants, products,
               shield, n_elements, element_counts, charge, e_index);
  if (rc) {
    delete h;
    return rc;
  }
  h->host.pah_total = pah_total;
  h->host.post_ok = reference_layout ? 1 : 0;
  h->host.c_total = c_total;
  h->host.o_total = o_total;
  h->device = st->device;
  h->sms = st->sms;
  h->stream = st->stream;
  cudaError_t e;
  if ((e = cudaMalloc(&h->table, sizeof(Table))) != cudaSuccess ||
      (e = cudaMalloc(&h->counter, sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&h->err, sizeof(unsigned int))) != cudaSuccess) {
    cudaGetLastError();
    p3d_network_destroy(h);
    return set_error(P3D_ENOMEM, "network cudaMalloc: %s", cudaGetErrorString(e));
  }
  const size_t sm = smem_bytes();
  if ((e = cudaFuncSetAttribute(steady_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sm)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(steady_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sm)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(rhs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sm)) != cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&h->blocks_per_sm[0],
                                                         steady_kernel<false>, kWarps * 32, sm)) !=
          cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&h->blocks_per_sm[1],
                                                         steady_kernel<true>, kWarps * 32, sm)) !=
          cudaSuccess) {
    p3d_network_destroy(h);
    return cuda_fail(e, "network kernel attributes");
  }
  if (h->blocks_per_sm[0] < 1 || h->blocks_per_sm[1] < 1) {
    p3d_network_destroy(h);
    return set_error(P3D_ECUDA, "network kernels do not fit on an SM");
  }
  if ((e = cudaMemcpyAsync(h->table, &h->host, sizeof(Table), cudaMemcpyHostToDevice,
                           h->stream)) != cudaSuccess ||
      (e = cudaMemsetAsync(h->err, 0, sizeof(unsigned int), h->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) {
    p3d_network_destroy(h);
    return cuda_fail(e, "network table upload");
  }
  *out = h;
  return P3D_OK;
}

int p3d_network_info(const p3d_network_t* h, int32_t* n_species, int32_t* reference_layout) {
  if (!h) return set_error(P3D_EINVAL, "null network");
  if (n_species) *n_species = h->host.ns;
  if (reference_layout) *reference_layout = h->host.post_ok;
  return P3D_OK;
}

int p3d_network_destroy(p3d_network_t* h) {
  if (!h) return P3D_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->table);
  cudaFree(h->counter);
  cudaFree(h->err);
  for (int k = 0; k < 4; ++k) cudaFree(h->stage[k]);
  delete h;
  return P3D_OK;
}

int p3d_network_rhs_dev(p3d_network_t* h, int64_t n, const double* cond, const double* x,
                        double* dxdt, void* stream) {
  if (!h) return set_error(P3D_EINVAL, "null network");
  int rc = check_device(h);
  if (rc) return rc;
  if (n < 0) return set_error(P3D_EINVAL, "n < 0");
  if (n == 0) return P3D_OK;
  if (!cond || !x || !dxdt) return set_error(P3D_EINVAL, "null array");
  int64_t blocks = ceil_div(n, kWarps);
  const int64_t cap = (int64_t)h->sms * h->blocks_per_sm[0];
  if (blocks > cap) blocks = cap;
  rhs_kernel<<<(unsigned)blocks, kWarps * 32, smem_bytes(), (cudaStream_t)stream>>>(
      h->table, n, cond, x, dxdt);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "network rhs launch");
}

int p3d_network_rhs(p3d_network_t* h, int64_t n, const double* cond, const double* x,
                    double* dxdt) {
  if (!h) return set_error(P3D_EINVAL, "null network");
  int rc = check_device(h);
  if (rc) return rc;
  if (n < 0) return set_error(P3D_EINVAL, "n < 0");
  if (n == 0) return P3D_OK;
  if (!cond || !x || !dxdt) return set_error(P3D_EINVAL, "null array");
  const size_t nc = sizeof(double) * 7 * (size_t)n, nx = sizeof(double) * h->host.ns * (size_t)n;
  void *dc, *dx, *df;
  if ((rc = stage(h, 0, nc, &dc)) || (rc = stage(h, 1, nx, &dx)) || (rc = stage(h, 2, nx, &df)))
    return rc;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(dc, cond, nc, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(dx, x, nx, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess)
    return cuda_fail(e, "network rhs H2D");
  if ((rc = p3d_network_rhs_dev(h, n, (const double*)dc, (const double*)dx, (double*)df,
                                h->stream)))
    return rc;
  if ((e = cudaMemcpyAsync(dxdt, df, nx, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
    return cuda_fail(e, "network rhs D2H");
  return sync_check(h->stream, "network rhs");
}

int p3d_network_steady_dev(p3d_network_t* h, int64_t n, const double* cond, double* x,
                           int32_t mixed, int32_t post, int32_t max_iter, double rtol,
                           int32_t* status, int32_t* iters, void* stream) {
  if (!h) return set_error(P3D_EINVAL, "null network");
  int rc = check_device(h);
  if (rc) return rc;
  if (n < 0) return set_error(P3D_EINVAL, "n < 0");
  if (n > (int64_t)INT32_MAX) return set_error(P3D_EINVAL, "n=%lld above 2^31-1", (long long)n);
  if (max_iter < 1) return set_error(P3D_EINVAL, "max_iter=%d < 1", max_iter);
  if (!(rtol > 0.0)) return set_error(P3D_EINVAL, "rtol must be > 0");
  if (post && !h->host.post_ok)
    return set_error(P3D_EINVAL, "post-processing needs the reference species layout");
  if (n == 0) return P3D_OK;
  if (!cond || !x) return set_error(P3D_EINVAL, "null array");
  cudaStream_t s = (cudaStream_t)stream;
  return mixed ? launch_steady<true>(h, n, cond, x, post, max_iter, rtol, status, iters, s)
               : launch_steady<false>(h, n, cond, x, post, max_iter, rtol, status, iters, s);
}

int p3d_network_steady(p3d_network_t* h, int64_t n, const double* cond, double* x, int32_t mixed,
                       int32_t post, int32_t max_iter, double rtol, int32_t* status,
                       int32_t* iters) {
  if (!h) return set_error(P3D_EINVAL, "null network");
  int rc = check_device(h);
  if (rc) return rc;
  if (n < 0) return set_error(P3D_EINVAL, "n < 0");
  if (n == 0) return P3D_OK;
  if (!cond || !x) return set_error(P3D_EINVAL, "null array");
  const size_t nc = sizeof(double) * 7 * (size_t)n, nx = sizeof(double) * h->host.ns * (size_t)n;
  const size_t ni = sizeof(int32_t) * (size_t)n;
  void *dc, *dx, *ds;
  if ((rc = stage(h, 0, nc, &dc)) || (rc = stage(h, 1, nx, &dx)) || (rc = stage(h, 3, 2 * ni, &ds)))
    return rc;
  int32_t* dst = (int32_t*)ds;
  int32_t* dit = dst + n;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(dc, cond, nc, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(dx, x, nx, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
      (e = cudaMemsetAsync(h->err, 0, sizeof(unsigned int), h->stream)) != cudaSuccess)
    return cuda_fail(e, "network steady H2D");
  if ((rc = p3d_network_steady_dev(h, n, (const double*)dc, (double*)dx, mixed, post, max_iter,
                                   rtol, dst, dit, h->stream)))
    return rc;
  unsigned int err = 0;
  if ((e = cudaMemcpyAsync(x, dx, nx, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess ||
      (status && (e = cudaMemcpyAsync(status, dst, ni, cudaMemcpyDeviceToHost, h->stream)) !=
                     cudaSuccess) ||
      (iters && (e = cudaMemcpyAsync(iters, dit, ni, cudaMemcpyDeviceToHost, h->stream)) !=
                    cudaSuccess) ||
      (e = cudaMemcpyAsync(&err, h->err, sizeof(err), cudaMemcpyDeviceToHost, h->stream)) !=
          cudaSuccess)
    return cuda_fail(e, "network steady D2H");
  if ((rc = sync_check(h->stream, "network steady"))) return rc;
  if (err & kErrNewtonLimit)
    return set_error(P3D_ECONVERGE, "network steady state: some cells not converged in %d iterations",
                     max_iter);
  return P3D_OK;
}

}  // extern "C"
