// p3d_steady_kernels.cuh -- kernels of the device-resident steady-state driver.
//
// One outer iteration reproduces the physics and ordering of
// PDRSolver3D.run() (prism3d/solver_3d.py:262-376) on the whole grid:
//   1. columns: N_H2 and N_CO along each cell's selected FUV ray;
//   2. grid-mean T for the H2 shielding Doppler width (solver_3d.py:302);
//   3. one fused per-cell kernel: shielding, PE heating, T_dust, H2
//      formation, chemistry to steady state (backward-Euler / Newton with the
//      cell's own H2 column solved implicitly), damping, thermal-balance
//      root, per-cell T update, convergence measure.
// G0, A_V, N_H, the cosmic-ray rate and the selected ray depend on density
// only (fuv_rt_3d.py:284-292: A_V uses N_H), so they are computed once by
// the full ray march at reset and folded into per-cell constants.
//
// Two precisions share the kernels: PLAIN (FP64 everywhere, fixed work per
// cell, one host synchronisation per iteration) and MIXED (FP32 LU with FP64
// residual + refinement, FP32 bisection with FP64-certified signs and an
// FP64 Newton polish of the thermal root, warm starts, iterations captured
// in a CUDA graph and checked every few launches).
#pragma once

#include "p3d_common.cuh"
#include "p3d_newton.cuh"
#include "p3d_pe.cuh"
#include "p3d_phys.cuh"
#include "p3d_rt.cuh"
#include "p3d_steady.cuh"
#include "p3d_thermal.cuh"
#include "p3d_thermal_fast.cuh"

namespace p3d {

// CO ladder and FP32 line tables for this translation unit (filled at
// p3d_steady_create).
__constant__ CoLevel c_co_ss[40];
__constant__ float c_lines32[20];
__constant__ float c_co32[200];
// FP64 geometric-bisection tree of [10, 1e5] K: node k (1..1023) holds
// sqrt(lo * hi) of its bracket, children 2k (net <= 0) and 2k + 1.
__device__ double g_bisect_mid[1024];
// per node: the FP32 twin's temperature-only FP64 parts (p3d_thermal_fast.cuh)
__device__ BisectNode g_bisect_node[1024];

// the two-level line table of the warp-cooperative net heating
__device__ CoopLine g_coop_lines[kCoopLines];

__global__ void ss_coop_table_kernel(LineFast lf) {
  const int e = threadIdx.x;
  if (blockIdx.x == 0 && e < kCoopLines) g_coop_lines[e] = coop_line(e, lf, c_co_ss);
}

__global__ void ss_bisect_table_kernel() {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double lo[1024], hi[1024];
  lo[1] = 10.0;
  hi[1] = 1e5;
  for (int k = 1; k < 1024; ++k) {
    double m = sqrt(lo[k] * hi[k]);
    g_bisect_mid[k] = m;
    g_bisect_node[k] = bisect_node(m, c_co_ss);
    if (2 * k + 1 < 1024) {
      lo[2 * k] = lo[k];
      hi[2 * k] = m;
      lo[2 * k + 1] = m;
      hi[2 * k + 1] = hi[k];
    }
  }
  g_bisect_mid[0] = 0.0;
  g_bisect_node[0] = BisectNode{0.0f, 0.0f, 0.0f, 0};
}

// Column layers (per unit ds) of a cell: 2 n x_H2 and n x_CO, the products
// fuv_rt_3d.py:335-337 forms (before its factor ds).  Kept beside the
// abundances by every kernel that writes them, so the column scans read two
// values per cell and multiply nothing.
__device__ __forceinline__ double col_layer_h2(double n, double x_h2) {
  return __dmul_rn(__dmul_rn(n, x_h2), 2.0);
}
__device__ __forceinline__ double col_layer_co(double n, double x_co) {
  return __dmul_rn(n, x_co);
}

__global__ void ss_layers_kernel(int64_t n, SteadyDev d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    d.l2[i] = col_layer_h2(d.dens[i], d.x_h2[i]);
    d.l3[i] = col_layer_co(d.dens[i], d.x_co[i]);
  }
}

// After a grain step every cell's PE heating and H2 formation change, so
// the fixed point moves: forget the last solve's change (the worklist solves
// every cell again), its bisection decisions (the root's inputs moved in a
// way the replay test does not see) and the T-update brackets, as the
// reference restarts its per-cell damping for every dust step
// (solver_3d.py:252-254).  State and warm-start roots are kept.
__global__ void ss_dust_restart_kernel(int64_t n, SteadyDev d) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    d.chg_last[i] = INFINITY;
    d.bis_node[i] = 0;
    d.t_prev[i] = 0.0;
    d.r_prev[i] = 0.0;
    d.t_lo[i] = 0.0;
    d.t_hi[i] = INFINITY;
    d.span[i] = INFINITY;
  }
}

// ----------------------------------------------------------------- setup
__global__ void __launch_bounds__(kThreads)
ss_setup_kernel(int64_t n, SteadyDev d, SteadyParams p, const double* __restrict__ ray_ds,
                const int* __restrict__ ray_fam) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double g0 = d.g0[i], av = d.av[i], nh = d.nh_col[i];
    int r = d.ray[i];
    bool okr = (r >= 0 && r < p.n_rays);
    d.ds[i] = okr ? ray_ds[r] : 0.0;
    d.fam[i] = okr ? (int8_t)ray_fam[r] : (int8_t)-1;
    double e374 = exp(-3.74 * av);
    d.kpd0[i] = 4.43e-11 * g0 * e374;
    d.uv0[i] = g0 * e374;
    d.kci[i] = 2.56e-10 * g0 * exp(-3.02 * av);
    d.kco0[i] = 1.71e-10 * g0 * exp(-3.53 * av);
    d.hci0[i] = 3.0e-10 * g0 * exp(-3.0 * av);
    d.zeta[i] = cr_rate(nh, p.zeta0);
    d.td_rad[i] = tdust_rad(g0, av);
    // analytic initial abundances (solver_3d.py:155-191)
    double lg = log10(fmax(g0, 0.1));
    double fh2 = 0.5 * (1.0 + tanh((av - (1.5 + 0.3 * lg)) / 0.8));
    double xh2 = fmin(fmax(fh2 * 0.5, 1e-6), 0.5);
    double xhi = fmin(fmax(1.0 - 2.0 * xh2, 1e-6), 1.0);
    double fco = 0.5 * (1.0 + tanh((av - (3.0 + 0.2 * lg)) / 1.0));
    double X = p.x_c_total;
    double xco = fmin(fmax(X * fco * 0.95, 1e-10), X);
    double xc = fmin(fmax(X * fco * 0.05, 1e-10), X);
    double xcp = fmin(fmax(X * (1.0 - fco), 1e-10), X);
    double cs = xcp + xc + xco;
    double sc = cs > 0.0 ? X / cs : 1.0;
    xcp *= sc;
    xc *= sc;
    xco *= sc;
    d.x_hi[i] = xhi;
    d.x_h2[i] = xh2;
    d.x_cp[i] = xcp;
    d.x_c[i] = xc;
    d.x_co[i] = xco;
    d.l2[i] = col_layer_h2(d.dens[i], xh2);
    d.l3[i] = col_layer_co(d.dens[i], xco);
    d.x_o[i] = fmax(p.x_o_total - xco, 1e-10);
    d.x_e[i] = fmax(xcp + p.x_hcop, 1e-10);
    d.t_gas[i] = p.t_init;
    d.f_nano[i] = p.f_nano;
    d.e_g[i] = p.e_g;
    d.t_prev[i] = 0.0;
    d.r_prev[i] = 0.0;
    d.t_lo[i] = 0.0;
    d.t_hi[i] = INFINITY;
    d.span[i] = INFINITY;
    d.t_root[i] = 0.0;
    d.u_h2_last[i] = -1.0;
    d.u_co_last[i] = -1.0;
    d.b_last[i] = -1.0;
    d.chg_last[i] = INFINITY;
    d.flags[i] = 0;
    d.bis_node[i] = 0;
    d.bis_margin[i] = 0.0f;
    d.fh2_slope[i] = INFINITY;
    // set by each cell's first chemistry solve; NaN until then (a get()
    // before run() shows them as not yet computed)
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    d.gamma_pe[i] = nan;
    d.t_dust[i] = nan;
    d.rh2_cell[i] = nan;
    d.fh2[i] = nan;
  }
}

// Selected-ray columns (fuv_rt_3d.py:297-392 restricted to each cell's
// selected ray): for every pencil along an axis and each direction, the
// running sums of the layers 2 n x_H2 and n x_CO from the illuminated end;
// cells whose selected ray belongs to that (axis, direction) family take
// ds x (upstream sum + half their own layer) (with own_implicit the own H2
// half layer is left out and added inside the chemistry solve).
//
// One launch covers all three axes, and each pencil is read once per axis
// for both directions:
//  * x and y (strided pencils): a block owns 32 pencils that are adjacent in
//    memory (consecutive k), one lane per pencil, so every warp load is a
//    256-byte contiguous row.  The pencil is cut into chunks of kColChunk
//    cells, dealt round-robin to the block's 8 warps: pass 1 stores each
//    chunk's two layer sums in shared memory, two warps turn them into the
//    carries into every chunk (exclusive sums from the front and from the
//    back), pass 2 re-reads the chunk (an L1 hit) and writes the cells of
//    both families, walking only the directions some cell of the chunk
//    selected.
//  * z (contiguous pencils): a warp per pencil, 4 consecutive cells per lane
//    and 128 cells per step; lane sums, then a warp shuffle scan (up for the
//    forward carry, down for the backward one).
// The layers 2 n x_H2 and n x_CO come precomputed (col_layer_h2/_co): on
// GB300 the scan is bound by the FP64 pipe, not by HBM, so it multiplies
// nothing and adds each layer once per running sum.  Sums are exact-order
// sequential only inside a chunk; the columns agree with a sequential
// cumulative sum to rounding (they feed the shielding factors, whose
// reference form the tests compare to 1e-12).  Layers are >= 0, so no clamp
// at 0 is needed.
constexpr int kColChunk = 8;    // cells per chunk of a strided pencil
constexpr int kColWarps = 8;    // warps per block
constexpr int kColLanesZ = 4;   // consecutive cells per lane on the z axis

// The worklist's column test of cell c against its columns at its last
// solve (ss_mark_kernel used to make it from u_h2 / u_h2_last / u_co /
// u_co_last; the pass that writes the columns makes it now, so the mark
// kernel reads one byte).
struct ColQuiet {
  const double* __restrict__ h2_last;
  const double* __restrict__ co_last;
  uint8_t* __restrict__ moved;
  double tol;
};

__device__ __forceinline__ void col_store(int own_implicit, int64_t c, double dsc, double s2,
                                          double s3, double l2, double l3,
                                          double* __restrict__ u_h2,
                                          double* __restrict__ u_co, const ColQuiet& q) {
  const double uh2 = own_implicit ? dsc * s2 : dsc * fma(0.5, l2, s2);
  const double uco = dsc * fma(0.5, l3, s3);
  u_h2[c] = uh2;
  u_co[c] = uco;
  q.moved[c] = !(fabs(uh2 - q.h2_last[c]) <= q.tol * fabs(uh2) &&
                 fabs(uco - q.co_last[c]) <= q.tol * fabs(uco));
}

// Shared memory of one strided-axis block: chunk sums and the carries from
// the front and from the back, nck x 32 doubles each for both layers,
// nck = chunks of the longer of the x and y pencils.
inline size_t columns_smem_bytes(int64_t nx, int64_t ny) {
  const int64_t len = nx > ny ? nx : ny;
  return sizeof(double) * 6 * 32 * (size_t)ceil_div(len, kColChunk);
}

// Blocks of each part of the launch: x tiles, y tiles, then z warps.
struct ColumnsGrid {
  int64_t nbx, nby, nbz;
};
inline ColumnsGrid columns_grid(int64_t nx, int64_t ny, int64_t nz) {
  const int64_t kt = ceil_div(nz, 32);
  return {ny * kt, nx * kt, ceil_div(nx * ny, kColWarps)};
}

// Number of column tiles: x tiles, y tiles, z pencils (col_dirty's layout).
inline int64_t column_tiles(int64_t nx, int64_t ny, int64_t nz) {
  const int64_t kt = ceil_div(nz, 32);
  return ny * kt + nx * kt + nx * ny;
}

// Marks the column tiles of the listed cells, whose layers the chemistry of
// this iteration rewrites, for the next column pass -- or, for a list longer
// than max_list, has that pass recompute every tile.
__global__ void ss_col_mark_kernel(int64_t nx, int64_t ny, int64_t nz,
                                   const int32_t* __restrict__ list,
                                   uint8_t* __restrict__ dirty, SteadyGlobals* g,
                                   int64_t max_list) {
  const int64_t count = (int64_t)g->n_active;
  const bool all = count > max_list;
  if (blockIdx.x == 0 && threadIdx.x == 0) g->cols_all = all ? 1 : 0;
  if (all) return;
  const int64_t kt = ceil_div(nz, 32);
  uint8_t* dx = dirty;
  uint8_t* dy = dx + ny * kt;
  uint8_t* dz = dy + nx * kt;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = list[e];
    const int64_t i = c / (ny * nz), j = (c / nz) % ny, k = c % nz;
    dx[j * kt + k / 32] = 1;
    dy[i * kt + k / 32] = 1;
    dz[i * ny + j] = 1;
  }
}

// Star mode: the point-source columns come from their own kernels, so the
// worklist's column test (as col_store makes it) is made here for every cell.
__global__ void ss_col_moved_kernel(int64_t n, const double* __restrict__ u_h2,
                                    const double* __restrict__ u_co, ColQuiet q) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double uh2 = u_h2[i], uco = u_co[i];
    q.moved[i] = !(fabs(uh2 - q.h2_last[i]) <= q.tol * fabs(uh2) &&
                   fabs(uco - q.co_last[i]) <= q.tol * fabs(uco));
  }
}

// force: every tile (else those marked in `dirty`, or all when g->cols_all);
// a tile's mark is cleared when it is recomputed.  A tile left out keeps its
// columns from the last pass, computed from the same layers.
__global__ void __launch_bounds__(32 * kColWarps)
ss_columns_kernel(int own_implicit, int64_t nx, int64_t ny, int64_t nz, int64_t nbx,
                  int64_t nby, const double* __restrict__ lay2, const double* __restrict__ lay3,
                  const int8_t* __restrict__ fam, const double* __restrict__ ds,
                  double* __restrict__ u_h2, double* __restrict__ u_co,
                  uint8_t* __restrict__ dirty, const SteadyGlobals* __restrict__ g, int force,
                  ColQuiet cq) {
  extern __shared__ double col_sh[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t b = blockIdx.x;
  const bool every = force || g->cols_all;
  if (b < nbx + nby) {
    // x tile b, y tile b - nbx: dirty + b either way (x tiles first)
    if (!every && !dirty[b]) return;
    __syncthreads();  // every thread has read the mark before it is cleared
    if (threadIdx.x == 0) dirty[b] = 0;
    const int axis = b < nbx ? 0 : 1;
    const int64_t t = axis == 0 ? b : b - nbx;
    const int64_t kt = ceil_div(nz, 32);
    const int64_t outer = t / kt;  // j (x pencils) or i (y pencils)
    const int64_t k = (t - outer * kt) * 32 + lane;
    const bool live = k < nz;
    const int64_t len = axis == 0 ? nx : ny;
    const int64_t stride = axis == 0 ? ny * nz : nz;
    const int64_t base = axis == 0 ? outer * nz + k : outer * ny * nz + k;
    const int nck = (int)ceil_div(len, kColChunk);
    double* tot2 = col_sh;             // chunk sums
    double* tot3 = tot2 + 32 * nck;
    double* fc2 = tot3 + 32 * nck;     // carries from the front
    double* fc3 = fc2 + 32 * nck;
    double* bc2 = fc3 + 32 * nck;      // carries from the back
    double* bc3 = bc2 + 32 * nck;
    for (int c = w; c < nck; c += kColWarps) {  // pass 1: chunk sums
      double s2 = 0.0, s3 = 0.0;
      if (live) {
#pragma unroll
        for (int u = 0; u < kColChunk; ++u) {
          const int64_t tt = (int64_t)c * kColChunk + u;
          if (tt < len) {
            s2 += lay2[base + tt * stride];
            s3 += lay3[base + tt * stride];
          }
        }
      }
      tot2[32 * c + lane] = s2;
      tot3[32 * c + lane] = s3;
    }
    __syncthreads();
    if (w == 0) {
      double a2 = 0.0, a3 = 0.0;
      for (int c = 0; c < nck; ++c) {
        fc2[32 * c + lane] = a2;
        fc3[32 * c + lane] = a3;
        a2 += tot2[32 * c + lane];
        a3 += tot3[32 * c + lane];
      }
    } else if (w == 1) {
      double a2 = 0.0, a3 = 0.0;
      for (int c = nck - 1; c >= 0; --c) {
        bc2[32 * c + lane] = a2;
        bc3[32 * c + lane] = a3;
        a2 += tot2[32 * c + lane];
        a3 += tot3[32 * c + lane];
      }
    }
    __syncthreads();
    if (!live) return;
    const int8_t want_f = (int8_t)(axis * 2 + 1), want_b = (int8_t)(axis * 2);
    for (int c = w; c < nck; c += kColWarps) {  // pass 2: writes
      const int64_t t0 = (int64_t)c * kColChunk;
      const int n_u = (int)(len - t0 < kColChunk ? len - t0 : kColChunk);
      const int64_t c0 = base + t0 * stride;
      unsigned need_f = 0u, need_b = 0u;  // cells of the chunk selecting each direction
      for (int u = 0; u < n_u; ++u) {
        const int8_t f = fam[c0 + u * stride];
        need_f |= (unsigned)(f == want_f) << u;
        need_b |= (unsigned)(f == want_b) << u;
      }
      if (need_f) {
        double f2 = fc2[32 * c + lane], f3 = fc3[32 * c + lane];
        for (int u = 0; u < n_u; ++u) {
          const int64_t cell = c0 + u * stride;
          const double a2 = lay2[cell], a3 = lay3[cell];
          if ((need_f >> u) & 1u) col_store(own_implicit, cell, ds[cell], f2, f3, a2, a3, u_h2, u_co, cq);
          f2 += a2;
          f3 += a3;
        }
      }
      if (need_b) {
        double b2 = bc2[32 * c + lane], b3 = bc3[32 * c + lane];
        for (int u = n_u - 1; u >= 0; --u) {
          const int64_t cell = c0 + u * stride;
          const double a2 = lay2[cell], a3 = lay3[cell];
          if ((need_b >> u) & 1u) col_store(own_implicit, cell, ds[cell], b2, b3, a2, a3, u_h2, u_co, cq);
          b2 += a2;
          b3 += a3;
        }
      }
    }
    return;
  }
  // z axis: one warp per contiguous pencil
  const int64_t pz = (b - nbx - nby) * kColWarps + w;
  if (pz >= nx * ny) return;
  uint8_t* dzp = dirty + nbx + nby + pz;
  if (!every && !*dzp) return;
  __syncwarp();  // every lane has read the mark before it is cleared
  if (lane == 0) *dzp = 0;
  const int64_t base = pz * nz;
  constexpr int kStep = 32 * kColLanesZ;
  const int8_t want_f = 5, want_b = 4;
  for (int dir = 1; dir >= 0; --dir) {  // forward pass, then backward
    double carry2 = 0.0, carry3 = 0.0;
    const int64_t nstep = ceil_div(nz, kStep);
    for (int64_t st = 0; st < nstep; ++st) {
      const int64_t c0 = (dir ? st : nstep - 1 - st) * kStep + kColLanesZ * lane;
      double l2[kColLanesZ], l3[kColLanesZ];
      int8_t fv[kColLanesZ];
      double s2 = 0.0, s3 = 0.0;
#pragma unroll
      for (int u = 0; u < kColLanesZ; ++u) {
        const int64_t tt = c0 + u;
        l2[u] = tt < nz ? lay2[base + tt] : 0.0;
        l3[u] = tt < nz ? lay3[base + tt] : 0.0;
        fv[u] = tt < nz ? fam[base + tt] : (int8_t)-1;
        s2 += l2[u];
        s3 += l3[u];
      }
      // inclusive scan of the lane sums in the pass direction, then one lane
      // shift for the exclusive sums (no subtraction, which would cancel)
      double e2 = s2, e3 = s3;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double a2 = dir ? __shfl_up_sync(0xffffffffu, e2, o)
                              : __shfl_down_sync(0xffffffffu, e2, o);
        const double a3 = dir ? __shfl_up_sync(0xffffffffu, e3, o)
                              : __shfl_down_sync(0xffffffffu, e3, o);
        const bool in = dir ? lane >= o : lane + o < 32;
        if (in) {
          e2 += a2;
          e3 += a3;
        }
      }
      const double all2 = __shfl_sync(0xffffffffu, e2, dir ? 31 : 0);
      const double all3 = __shfl_sync(0xffffffffu, e3, dir ? 31 : 0);
      double x2 = dir ? __shfl_up_sync(0xffffffffu, e2, 1) : __shfl_down_sync(0xffffffffu, e2, 1);
      double x3 = dir ? __shfl_up_sync(0xffffffffu, e3, 1) : __shfl_down_sync(0xffffffffu, e3, 1);
      if (dir ? lane == 0 : lane == 31) {
        x2 = 0.0;
        x3 = 0.0;
      }
      double r2 = carry2 + x2, r3 = carry3 + x3;
      const int8_t want = dir ? want_f : want_b;
#pragma unroll
      for (int v = 0; v < kColLanesZ; ++v) {
        const int u = dir ? v : kColLanesZ - 1 - v;
        if (fv[u] == want)
          col_store(own_implicit, base + c0 + u, ds[base + c0 + u], r2, r3, l2[u], l3[u],
                    u_h2, u_co, cq);
        r2 += l2[u];
        r3 += l3[u];
      }
      carry2 += all2;
      carry3 += all3;
    }
  }
}

// ------------------------------------------------------------ reductions
__global__ void ss_sum_kernel(int64_t n, const double* __restrict__ x, double* __restrict__ part) {
  __shared__ double sh[kThreads / 32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += x[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) t += sh[w];
    part[blockIdx.x] = t;
  }
}

// The block partial sums added in order by one thread: the mean T (and so
// the Doppler width every cell's H2 shielding sees) is the same on every run
// and unchanged from the order the plain path's tests were pinned with (a
// tree order moves it by an ulp, enough to flip which few cells chatter on a
// bisection node at tol 1e-11).
__global__ void ss_finalize_kernel(int nparts, const double* __restrict__ part, int64_t n,
                                   SteadyGlobals* g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[b];
  double tm = s / (double)n;
  g->t_mean = tm;
  g->b_dop = sqrt(2.0 * kKBoltz * tm / (2.0 * kMH)) / 1e5;
  g->dmax_bits = 0ull;
  g->evals64 = 0ull;
  g->chem_fail = 0u;
  g->therm_fail = 0u;
  g->n_gt[0] = g->n_gt[1] = g->n_gt[2] = 0u;
  g->n_active = 0u;
  g->therm_next = 0u;
  g->chem_next = 0u;
}

__device__ __forceinline__ void block_max_atomic(double v, unsigned long long* dst) {
  __shared__ double sh[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, sh[w]);
    // non-negative doubles order like their bit patterns
    if (m > 0.0) atomicMax(dst, (unsigned long long)__double_as_longlong(m));
  }
}

// ------------------------------------------------- per-cell T update
// r = G - T_in changes sign at a fixed point of the outer map; each cell
// keeps the largest T_in with r > 0 (lo) and the smallest with r < 0 (hi).
// With a bracket: secant step through the last two (T_in, r) pairs, or the
// geometric midpoint when it leaves the bracket.  Without one: the damped
// step (1 - w_T) r, limited to `span`, which starts at twice the width of
// the last lost bracket and grows x4 per step.  A bracket narrower than
// 4e-12 T makes the cell hop across it each iteration: a genuine jump keeps
// it, a bracket made stale by the rest of the grid breaks.
__device__ __forceinline__ double t_update(double t_in, double G, double w_t, double& tp,
                                           double& rp, double& lo, double& hi, double& span) {
  double r = G - t_in;
  double lo_n = r > 0.0 ? fmax(lo, t_in) : lo;
  double hi_n = r < 0.0 ? fmin(hi, t_in) : hi;
  bool bad = lo_n >= hi_n;
  bool had = (lo > 0.0) && isfinite(hi);
  if (bad && had) span = fmax(2.0 * (hi - lo), 1e-9 * t_in);
  if (bad) {
    lo = r > 0.0 ? t_in : 0.0;
    hi = r < 0.0 ? t_in : INFINITY;
  } else {
    lo = lo_n;
    hi = hi_n;
  }
  bool valid = (lo > 0.0) && isfinite(hi);
  double den = r - rp;
  double ts = t_in - r * (t_in - tp) / den;
  bool ok_sec = isfinite(ts) && (den != 0.0) && (tp > 0.0);
  double mid = sqrt(lo * (valid ? hi : 1.0));
  bool inside = ok_sec && ts > lo && ts < hi;
  double step = fmin(fmax((1.0 - w_t) * r, -span), span);
  if (!valid) span *= 4.0;
  double tn = valid ? (inside ? ts : mid) : t_in + step;
  // collapsed bracket: hop just across it, so the next residual re-checks
  // the jump (a bracket left over from an earlier map then breaks)
  if (valid && hi - lo <= 4e-12 * t_in) tn = (t_in <= lo) ? hi * (1.0 + 1e-12) : lo * (1.0 - 1e-12);
  if (r == 0.0) tn = t_in;
  tp = t_in;
  rp = r;
  return tn;
}

// ----------------------------------------------------------- cell kernel
// ------------------------------------------------------------ worklist
// A cell is solved this iteration unless (mixed path, from the fourth
// iteration on) its last solve changed it by <= quiet_tol and its inputs
// have moved little since: its selected-ray columns by <= quiet_in_tol, and
// its H2 self-shielding factor by <= quiet_b_tol.  The factor is the one
// input the Doppler width b (set by the grid-mean T, which drifts while the
// last cells settle) reaches; its relative change is |db / b| times the
// slope |d ln f_H2 / d ln b| kept from the last solve, so a drift of the mean
// T wakes only the cells in the H2 transition, where f_H2 depends on b (not
// those where it is ~1 or set by its damping-wing term).  Then the cell is
// at its fixed point to about the tolerance and keeps its state -- provided
// its last thermal residual |G - T| / T was small as well: a T update
// confined to a stale bracket, or hopping across a collapsed one, takes
// ~1e-12 steps while G - T stays large, and only further solves break that
// bracket (cells whose T sits on a discontinuity of the thermal balance are
// therefore solved every iteration, as on the plain path).  Solved cells are
// appended to a dense list (one atomic per warp), so the chemistry and
// thermal kernels run full warps of active cells.
template <bool MIXED>
__global__ void __launch_bounds__(kThreads)
ss_mark_kernel(int64_t n, SteadyDev d, SteadyParams p, SteadyGlobals* g) {
  const double b_dop = g->b_dop;
  const int iter = g->iter;
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < n;
       base += stride) {
    const int64_t i = base + lane;
    bool active = i < n;
    if (active && MIXED && iter > 2) {
      // last change <= quiet_tol and residual <= quiet_r_tol (q_self), its
      // columns within quiet_in_tol of their values at that solve (!q_moved)
      if (d.q_self[i] && !d.q_moved[i]) {
        const double b_last = d.b_last[i];
        if (b_last == b_dop ||
            fabs(b_dop - b_last) * (double)d.fh2_slope[i] <= p.quiet_b_tol * b_dop)
          active = false;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, active);
    if (m) {
      unsigned pos = 0;
      if (lane == 0) pos = atomicAdd(&g->n_active, (unsigned)__popc(m));
      pos = __shfl_sync(0xffffffffu, pos, 0);
      if (active) d.list[pos + __popc(m & ((1u << lane) - 1u))] = (int32_t)i;
    }
  }
}

// Dust coupling, rates, steady-state chemistry, damping.  Cells k < count of
// the list (plain path: every cell, no list).
template <bool MIXED>
__global__ void __launch_bounds__(kThreads)
ss_chem_kernel(int64_t n, SteadyDev d, SteadyParams p, SteadyGlobals* g,
               const double* __restrict__ a_nano, const double* __restrict__ a_rest) {
  const double b_dop = g->b_dop;
  const int iter = g->iter;
  const int64_t count = MIXED ? (int64_t)g->n_active : n;
  unsigned int my_fail = 0u;
  const int lane = threadIdx.x & 31;
  // warps past the list's batches of 32 take none (as the thermal kernel)
  const bool queue = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) < (count + 31) / 32;
  while (queue) {  // 32 cells per warp from a global counter (as the thermal kernel)
    unsigned int base = 0u;
    if (lane == 0) base = atomicAdd(&g->chem_next, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((int64_t)base >= count) break;
    const int64_t k = (int64_t)base + lane;
    if (k >= count) continue;
    const int64_t i = MIXED ? (int64_t)d.list[k] : k;
    const double nh = d.dens[i];
    const double tg = d.t_gas[i];
    const double xe0 = d.x_e[i];
    double y_old[5] = {d.x_hi[i], d.x_h2[i], d.x_cp[i], d.x_c[i], d.x_co[i]};
    // dust coupling at the current T (solver_3d.py:509-530)
    const double fn = d.f_nano[i];
    const double gpe = pe_cell(p.pe, a_nano, a_rest, d.g0[i], tg, xe0, nh, fn, d.e_g[i]);
    const double td = tdust(d.td_rad[i], nh, tg);
    const double rh2 = h2_form<MIXED>(tg, td, fn, p.sigma_nano, p.sigma_lc, p.sigma_sil);
    const double zeta = d.zeta[i];
    // chemistry (solver_3d.py:549-557 rates; steady state of chemistry.rs:35-49)
    ChemCell cc;
    cc.n_h = nh;
    cc.kci = d.kci[i] * p.rs[3];
    // (T / 300)^-0.6; the mixed path from a logarithm and exp64 (as fsh_co)
    cc.acp = 4.67e-12 * (MIXED ? exp64(-0.6 * log(tg / 300.0)) : pow(tg / 300.0, -0.6)) *
             p.rs[4];
    cc.rh2 = rh2 * nh * 0.5 * p.rs[0];
    cc.rcr = 2.5 * zeta * 0.1 * p.rs[2];
    cc.xc = p.x_c_total;
    cc.hcop = p.x_hcop;
    cc.kpd0 = d.kpd0[i] * p.rs[1];
    cc.kco0 = d.kco0[i] * p.rs[5];
    cc.kco_cr = 6.0 * zeta * p.rs[6];
    cc.koh_s = p.rs[7];
    cc.u_h2 = d.u_h2[i];
    cc.u_co = d.u_co[i];
    cc.ds = p.h2_implicit ? d.ds[i] : 0.0;
    cc.b_dop = b_dop;
    chem_prepare<MIXED>(cc);
    double y[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) y[c] = fmax(y_old[c], 1e-30);
    double fh2 = 1.0;
    int citers = 0;
    // inexact chemistry while the cell is still moving (as the thermal root):
    // the Newton tolerance follows 1% of the cell's last relative change, at
    // most 1e-6, back to chem_rtol as it settles; a cell's first solve is
    // exact
    const double cl = d.chg_last[i];
    const double rtol_c = (MIXED && isfinite(cl) && !p.exact_roots)
                              ? fmax(p.chem_rtol, fmin(1e-6, 0.01 * cl))
                              : p.chem_rtol;
    int cst = chem_steady_cell<MIXED>(cc, y, p.chem_max_iter, rtol_c, 4.0, &fh2, &citers);
    my_fail += (unsigned)cst;
    double x[5];
    const bool damp = iter > 0 && p.w_chem > 0.0;
    double m = 0.0;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      x[c] = damp ? p.w_chem * y_old[c] + (1.0 - p.w_chem) * y[c] : y[c];
      m = fmax(m, fabs(x[c] - y_old[c]) / fmax(y_old[c], 1e-20));
    }
    d.x_hi[i] = x[0];
    d.x_h2[i] = x[1];
    d.x_cp[i] = x[2];
    d.x_c[i] = x[3];
    d.x_co[i] = x[4];
    d.l2[i] = col_layer_h2(nh, x[1]);
    d.l3[i] = col_layer_co(nh, x[4]);
    d.x_o[i] = fmax(p.x_o_total - y[4], 1e-30);
    d.x_e[i] = fmax(y[2] + p.x_hcop, 1e-30);
    d.fh2[i] = fh2;
    // the column the shielding factor saw (chem_prepare / chem5_eval)
    const double nh2_sh = cc.ds > 0.0 ? cc.u_h2 + cc.ds * nh * y[1] : cc.u_h2;
    d.fh2_slope[i] = (float)fsh_h2_dlnb(nh2_sh, b_dop, fh2);
    d.gamma_pe[i] = gpe;
    d.t_dust[i] = td;
    d.rh2_cell[i] = rh2;
    d.chg_spec[i] = m;
  }
  for (int o = 16; o > 0; o >>= 1) my_fail += __shfl_xor_sync(0xffffffffu, my_fail, o);
  if ((threadIdx.x & 31) == 0 && my_fail) atomicAdd(&g->chem_fail, my_fail);
}

// Thermal context of cell i (solver_3d.py:693-754) from the state its last
// chemistry solve left: Gamma_PE, T_dust, R_H2 and f_H2 of that solve.
__device__ __forceinline__ ThermalCtx steady_thermal_ctx(const SteadyDev& d, int64_t i) {
  const double nh = d.dens[i];
  const double x0 = d.x_hi[i], x1 = d.x_h2[i], x3 = d.x_c[i];
  const double zeta = d.zeta[i];
  const double rh2 = d.rh2_cell[i];
  ThermalCtx c;
  const double uv = d.uv0[i] * d.fh2[i];
  double gf = d.gamma_pe[i];
  gf += 3.3e-11 * uv * x1 * nh * (0.4 * kEVtoErg);
  gf += rh2 * x0 * (nh * nh) * (1.5 * kEVtoErg);
  gf += 3.0e-10 * uv * x1 * nh * (2.0 * kEVtoErg) * (nh / (nh + 3e4));
  gf += zeta * (x0 + 2.0 * x1) * nh * (20.0 * kEVtoErg);
  gf += d.hci0[i] * x3 * nh * kEVtoErg;
  c.gamma_fixed = gf;
  const double mu = x1 > 0.5 ? 2.0 : 1.0;
  c.gg_coeff = 2.0 * 0.35 * 1e-21 * (nh * nh) * (mu == 2.0 ? kGgSpeedMu2 : kGgSpeedMu1) * kKBoltz;
  c.t_dust = d.t_dust[i];
  c.n_e = d.x_e[i] * nh;
  c.n_hi = x0 * nh;
  c.n_h2 = x1 * nh;
  c.n_co = d.x_co[i] * nh;
  c.n_cp_nh = d.x_cp[i] * nh;
  c.n_o_nh = d.x_o[i] * nh;
  c.n_c_nh = x3 * nh;
  return c;
}

// Diagnostics Gamma (which == 0) or Lambda (1) at each cell's current T
// (solver_3d.py:891-892) with the context of its last solve.
__global__ void __launch_bounds__(kThreads)
ss_heating_cooling_kernel(int64_t n, SteadyDev d, SteadyParams p, int which,
                          double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const ThermalCtx c = steady_thermal_ctx(d, i);
    double g, l;
    heating_cooling64(d.t_gas[i], c, p.lines, c_co_ss, &g, &l);
    out[i] = which ? l : g;
  }
}

// |now - before| / |now| to FP32 precision (0 when both are 0).
__device__ __forceinline__ double rel_change32(double now, double before) {
  return (double)(fabsf((float)(now - before)) / fmaxf(fabsf((float)now), 1e-30f));
}

// Thermal context (solver_3d.py:693-754), thermal root, per-cell T update and
// convergence measure of cell i.  COOP: all lanes of the warp run it for the
// same cell (FP64 net heating over the warp); only `lead` stores and counts.
template <bool MIXED, bool COOP>
__device__ __forceinline__ void thermal_cell(int64_t i, const SteadyDev& d, const SteadyParams& p,
                                             double b_dop, bool lead, double& my_max,
                                             unsigned int* my_gt, unsigned int& my_fail,
                                             unsigned long long& my_evals) {
  const double tg = d.t_gas[i];
  const ThermalCtx c = steady_thermal_ctx(d, i);
  int tst = 0, nev = 0;
  double troot;
  int node = 0;
  float margin = 0.0f;
  if (p.fix_t) {
    troot = tg;
  } else if (MIXED) {
    // largest relative change of the root's inputs since the cell's last
    // thermal solve: species, T (context), H2/CO columns, Doppler width (the
    // ratios in FP32: delta only meets 1/300 of a certified margin, and an
    // FP32 division costs the FP64 pipe two conversions where an FP64 one
    // costs it a dozen instructions)
    const double tp0 = d.t_prev[i];
    double delta = fmax(d.chg_spec[i], tp0 > 0.0 ? rel_change32(tg, tp0) : INFINITY);
    delta = fmax(delta, rel_change32(d.u_h2[i], d.u_h2_last[i]));
    delta = fmax(delta, rel_change32(d.u_co[i], d.u_co_last[i]));
    delta = fmax(delta, rel_change32(b_dop, d.b_last[i]));
    node = d.bis_node[i];
    margin = d.bis_margin[i];
    // inexact roots while the cell is still moving: the root tolerance
    // follows 1% of its last relative change (at most 1e-4), back to
    // therm_tol_mixed as it settles; a cell's first solve is exact
    const double cl = d.chg_last[i];
    const double rtol_t = (isfinite(cl) && !p.exact_roots)
                              ? fmax(p.therm_tol_mixed, fmin(1e-4, 0.01 * cl))
                              : p.therm_tol_mixed;
    troot = root_mixed<COOP>(c, p.lf, c_co_ss, p.theta2, c_lines32, c_co32, g_bisect_mid,
                             g_bisect_node, rtol_t, p.therm_max_iter, d.t_root[i], delta, &node,
                             &margin, &tst, &nev, g_coop_lines);
  } else {
    troot = root_plain(c, p.lf, c_co_ss, p.theta2, p.therm_tol, p.therm_max_iter, &tst, &nev);
  }
  double tp = d.t_prev[i], rp = d.r_prev[i], lo = d.t_lo[i], hi = d.t_hi[i], sp = d.span[i];
  double tn = t_update(tg, troot, p.w_t, tp, rp, lo, hi, sp);
  double m = fmax(d.chg_spec[i], fabs(tn - tg) / tg);
  if (!(m == m)) m = INFINITY;
  if (!lead) return;
  if (MIXED && !p.fix_t) {
    d.bis_node[i] = (int16_t)node;
    d.bis_margin[i] = margin;
  }
  my_evals += (unsigned long long)nev;
  my_fail += (unsigned)tst;
  my_max = fmax(my_max, m);
  my_gt[0] += m > p.count_thr[0];
  my_gt[1] += m > p.count_thr[1];
  my_gt[2] += m > p.count_thr[2];
  d.t_root[i] = troot;
  d.t_gas[i] = tn;
  d.t_prev[i] = tp;
  d.r_prev[i] = rp;
  d.t_lo[i] = lo;
  d.t_hi[i] = hi;
  d.span[i] = sp;
  d.u_h2_last[i] = d.u_h2[i];
  d.u_co_last[i] = d.u_co[i];
  d.b_last[i] = b_dop;
  d.chg_last[i] = m;
  d.q_self[i] = m <= p.quiet_tol && fabs(rp) <= p.quiet_r_tol * tp;
  d.q_moved[i] = 0;
}

// q_self of every cell from its last change and residual under this run's
// tolerances (run() start: a reset, set, dust step or another tolerance may
// have changed them since they were formed).
__global__ void ss_quiet_init_kernel(int64_t n, SteadyDev d, SteadyParams p) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d.q_self[i] = d.chg_last[i] <= p.quiet_tol && fabs(d.r_prev[i]) <= p.quiet_r_tol * d.t_prev[i];
}

// __maxnreg__ 80 (6 resident blocks of 128 threads per SM instead of 4 at
// the 124 registers the compiler picks): the thermal launches of the tail are
// latency-bound and gain from more warps despite a few spills (a 1.9% shorter
// 128^3 solve; 96 registers gained 0.3%).
template <bool MIXED>
__global__ void __maxnreg__(80)
ss_thermal_kernel(int64_t n, SteadyDev d, SteadyParams p, SteadyGlobals* g) {
  const double b_dop = g->b_dop;
  const int64_t count = MIXED ? (int64_t)g->n_active : n;
  double my_max = 0.0;
  unsigned int my_gt[3] = {0u, 0u, 0u};
  unsigned int my_fail = 0u;
  unsigned long long my_evals = 0ull;
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (MIXED && count <= (int64_t)p.coop_max) {
    // a short list (the last outer iterations): one cell per warp.  The
    // launch then lasts as long as the slowest cell's chain of FP64
    // evaluations, and on GB300 a warp's FP64 instruction holds its
    // scheduler's FP64 unit as long with one active lane as with 32: the
    // warp evaluates the cell's net heating together (net_heating_coop64).
    bool queue = gwarp < count;
    while (queue) {
      unsigned int base = 0u;
      if (lane == 0) base = atomicAdd(&g->therm_next, 1u);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((int64_t)base >= count) break;
      thermal_cell<MIXED, true>((int64_t)d.list[base], d, p, b_dop, lane == 0, my_max, my_gt,
                                my_fail, my_evals);
    }
  } else {
    // Warps take 32 cells (mixed: list entries) at a time from a global
    // counter, so the uneven root-finding work spreads over all warps until
    // none is left.  Warps past the list's batches of 32 take none: in the
    // last outer iterations a few thousand listed cells meet a grid sized
    // for every cell, and each idle warp's queue atomic would queue up on
    // the counter.
    const bool queue = gwarp < (count + 31) / 32;
    while (queue) {
      unsigned int base = 0u;
      if (lane == 0) base = atomicAdd(&g->therm_next, 32u);
      base = __shfl_sync(0xffffffffu, base, 0);
      if ((int64_t)base >= count) break;
      const int64_t k = (int64_t)base + lane;
      if (k >= count) continue;
      thermal_cell<MIXED, false>(MIXED ? (int64_t)d.list[k] : k, d, p, b_dop, true, my_max, my_gt,
                                 my_fail, my_evals);
    }
  }
  block_max_atomic(my_max, &g->dmax_bits);
  for (int o = 16; o > 0; o >>= 1) {
    my_evals += __shfl_xor_sync(0xffffffffu, my_evals, o);
    my_fail += __shfl_xor_sync(0xffffffffu, my_fail, o);
#pragma unroll
    for (int k = 0; k < 3; ++k) my_gt[k] += __shfl_xor_sync(0xffffffffu, my_gt[k], o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (my_evals) atomicAdd(&g->evals64, my_evals);
    if (my_fail) atomicAdd(&g->therm_fail, my_fail);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (my_gt[k]) atomicAdd(&g->n_gt[k], my_gt[k]);
  }
}

// N_H2 (which = 1) or N_CO (which = 0) of the selected ray for output; with
// own_implicit the H2 column excludes the cell's own half layer (solved inside
// the chemistry) and it is added here.
__global__ void ss_columns_out_kernel(int64_t n, int which, int own_implicit,
                                      const double* __restrict__ dens,
                                      const double* __restrict__ xh2,
                                      const double* __restrict__ ds,
                                      const double* __restrict__ u_h2,
                                      const double* __restrict__ u_co, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = which ? u_h2[i] + (own_implicit ? ds[i] * dens[i] * xh2[i] : 0.0) : u_co[i];
}

// hist[kHistCols it ...] = (largest relative change, chemistry failures,
// thermal failures, cells changing more than count_thr[0..2], FP64
// net-heating evaluations, mean T, cells solved) of iteration `it`; then
// advance the counter.
__global__ void ss_record_kernel(SteadyGlobals* g, double* hist, int max_hist) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int it = g->iter;
    if (it >= 0 && it < max_hist) {
      double* h = hist + (int64_t)kHistCols * it;
      h[0] = __longlong_as_double((long long)g->dmax_bits);
      h[1] = (double)g->chem_fail;
      h[2] = (double)g->therm_fail;
      h[3] = (double)g->n_gt[0];
      h[4] = (double)g->n_gt[1];
      h[5] = (double)g->n_gt[2];
      h[6] = (double)g->evals64;
      h[7] = g->t_mean;
      h[8] = (double)g->n_active;  // plain path: 0 (no list; every cell solved)
    }
    g->iter = it + 1;
  }
}

__global__ void ss_reset_globals_kernel(SteadyGlobals* g) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    g->t_mean = 0.0;
    g->b_dop = 0.0;
    g->dmax_bits = 0ull;
    g->evals64 = 0ull;
    g->chem_fail = 0u;
    g->therm_fail = 0u;
    g->n_gt[0] = g->n_gt[1] = g->n_gt[2] = 0u;
    g->n_active = 0u;
  g->therm_next = 0u;
  g->chem_next = 0u;
    g->iter = 0;
  }
}

// ------------------------------------------------------------ refinement
// Reference species layout of the full network (prism3d/chemistry/solver.py:28-36).
constexpr int kNetSpecies = 31;
constexpr int kNetE = 0, kNetH = 1, kNetH2 = 2, kNetCp = 7, kNetC = 8, kNetCO = 9, kNetO = 13,
              kNetOH = 15, kNetH2O = 17, kNetHCOp = 22;

// Conditions (n x 7) and initial abundances (n x 31) of the refinement pass.
__global__ void ss_refine_gather_kernel(int64_t n, SteadyDev d, SteadyParams p, double b_dop,
                                        double* __restrict__ cond, double* __restrict__ x31) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double nh = d.dens[i];
    const double nh2 = p.h2_implicit ? d.u_h2[i] + d.ds[i] * nh * d.x_h2[i] : d.u_h2[i];
    double d1, dh;
    double* c = cond + 7 * i;
    c[0] = nh;
    c[1] = d.t_gas[i];
    c[2] = d.g0[i];
    c[3] = d.av[i];
    c[4] = d.zeta[i];
    c[5] = fsh_h2(nh2, b_dop, &d1);
    c[6] = fsh_co(d.u_co[i], nh2, &dh);
    double* x = x31 + (int64_t)kNetSpecies * i;
    for (int k = 0; k < kNetSpecies; ++k) x[k] = 1e-30;
    x[kNetE] = d.x_e[i];
    x[kNetH] = d.x_hi[i];
    x[kNetH2] = d.x_h2[i];
    x[kNetCp] = d.x_cp[i];
    x[kNetC] = d.x_c[i];
    x[kNetCO] = d.x_co[i];
    x[kNetO] = d.x_o[i];
    const double lg = log10(fmax(d.g0[i], 0.1));
    const double fh2_ic = 0.5 * (1.0 + tanh((d.av[i] - (1.5 + 0.3 * lg)) / 0.8));
    x[kNetOH] = 1e-9 + 9e-8 * fmin(fmax(fh2_ic, 0.0), 1.0);
    x[kNetH2O] = 1e-8;
    x[kNetHCOp] = p.x_hcop;
  }
}

// Write the refined abundances back and set T_gas to the thermal root with
// them (dust coupling and PE heating at the current T).
__global__ void __launch_bounds__(kThreads)
ss_refine_scatter_kernel(int64_t n, SteadyDev d, SteadyParams p, const double* __restrict__ x31,
                         const double* __restrict__ a_nano, const double* __restrict__ a_rest,
                         unsigned int* n_fail) {
  unsigned int fails = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double* x = x31 + (int64_t)kNetSpecies * i;
    const double x0 = x[kNetH], x1 = x[kNetH2], x3 = x[kNetC], xe = x[kNetE];
    d.x_hi[i] = x0;
    d.x_h2[i] = x1;
    d.x_cp[i] = x[kNetCp];
    d.x_c[i] = x3;
    d.x_co[i] = x[kNetCO];
    d.x_o[i] = x[kNetO];
    d.x_e[i] = xe;
    const double nh = d.dens[i];
    d.l2[i] = col_layer_h2(nh, x1);
    d.l3[i] = col_layer_co(nh, x[kNetCO]);
    const double tg = d.t_gas[i];
    const double fn = d.f_nano[i];
    const double gpe = pe_cell(p.pe, a_nano, a_rest, d.g0[i], tg, xe, nh, fn, d.e_g[i]);
    const double td = tdust(d.td_rad[i], nh, tg);
    const double rh2 = h2_form(tg, td, fn, p.sigma_nano, p.sigma_lc, p.sigma_sil);
    const double zeta = d.zeta[i];
    const double uv = d.uv0[i] * d.fh2[i];
    ThermalCtx c;
    double gf = gpe;
    gf += 3.3e-11 * uv * x1 * nh * (0.4 * kEVtoErg);
    gf += rh2 * x0 * (nh * nh) * (1.5 * kEVtoErg);
    gf += 3.0e-10 * uv * x1 * nh * (2.0 * kEVtoErg) * (nh / (nh + 3e4));
    gf += zeta * (x0 + 2.0 * x1) * nh * (20.0 * kEVtoErg);
    gf += d.hci0[i] * x3 * nh * kEVtoErg;
    c.gamma_fixed = gf;
    const double mu = x1 > 0.5 ? 2.0 : 1.0;
    c.gg_coeff = 2.0 * 0.35 * 1e-21 * (nh * nh) * (mu == 2.0 ? kGgSpeedMu2 : kGgSpeedMu1) * kKBoltz;
    c.t_dust = td;
    c.n_e = xe * nh;
    c.n_hi = x0 * nh;
    c.n_h2 = x1 * nh;
    c.n_co = x[kNetCO] * nh;
    c.n_cp_nh = x[kNetCp] * nh;
    c.n_o_nh = x[kNetO] * nh;
    c.n_c_nh = x3 * nh;
    int tst = 0, nev = 0;
    const double troot = root_plain(c, p.lf, c_co_ss, p.theta2, p.therm_tol,
                                    p.therm_max_iter, &tst, &nev);
    fails += (unsigned)tst;
    d.t_gas[i] = troot;
    d.t_root[i] = troot;
    d.gamma_pe[i] = gpe;
    d.t_dust[i] = td;
    d.chg_last[i] = INFINITY;  // the mixed path re-solves every cell next
  }
  for (int o = 16; o > 0; o >>= 1) fails += __shfl_xor_sync(0xffffffffu, fails, o);
  if ((threadIdx.x & 31) == 0 && fails) atomicAdd(n_fail, fails);
}

}  // namespace p3d
