// p3d_steady.cu -- device-resident steady-state driver (kernels in
// p3d_steady_kernels.cuh) and its host runtime behind the C ABI.
//
// Owns the per-cell device arrays of one grid, the library stream and, for
// the mixed path, a CUDA graph holding `kGraphIters` outer iterations that
// is relaunched until the convergence history read back after each launch
// drops below the tolerance.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/prism3d_gb300.h"
#include "p3d_capi_internal.cuh"
#include "p3d_common.cuh"
#include "p3d_pe.cuh"
#include "p3d_rt.cuh"
#include "p3d_steady.cuh"
#include "p3d_steady_kernels.cuh"
#include "p3d_adjoint.cuh"

namespace p3d {

constexpr int kGraphIters = 8;
constexpr int kMaxHist = 1 << 16;

struct SteadySolver {
  DeviceState* st = nullptr;
  int64_t nx = 0, ny = 0, nz = 0, n = 0;
  double cell = 0.0;
  RaySet rays;
  // point source (solver_3d.py:270-276): the field and the per-iteration
  // H2 / CO columns come from the star instead of the external ray set
  int star = 0;
  double star_pos[3] = {0.0, 0.0, 0.0}, star_lum = 0.0;
  SteadyParams par;
  SteadyDev d;
  std::vector<void*> allocs;
  double* dens = nullptr;
  double *nh2_full = nullptr, *nco_full = nullptr, *scratch = nullptr;
  double *a_nano = nullptr, *a_rest = nullptr;
  double *ray_ds = nullptr;
  int* ray_fam = nullptr;
  double* parts = nullptr;
  int nparts = 0;
  SteadyGlobals* glob = nullptr;
  double* hist = nullptr;
  double* hist_host = nullptr;  // pinned
  cudaGraphExec_t graph = nullptr;
  int graph_mixed = -1;
  SteadyParams graph_par;
  int64_t iters_done = 0;
  // launch shape of the per-cell chemistry / thermal kernels (threads per
  // block, blocks per SM of the grid-stride loop); p3d_steady_autotune sets
  // it.  Default: the shape it picks on GB300 for the 128^3 slab (more
  // blocks than fit an SM: the work queue hands cells to the blocks resident)
  int cell_threads = 128, cell_per_sm = 16;
  int64_t launches = 0;  // kernels launched since the last reset
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;  // reset .. end of last run
  double last_dmax = INFINITY;

  template <typename T>
  int alloc(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(e, "steady cudaMalloc");
    }
    allocs.push_back(q);
    *p = (T*)q;
    return P3D_OK;
  }

  ~SteadySolver() {
    if (graph) cudaGraphExecDestroy(graph);
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_stop) cudaEventDestroy(ev_stop);
    if (st) cudaStreamSynchronize(st->stream);
    for (void* q : allocs) cudaFree(q);
    if (hist_host) cudaFreeHost(hist_host);
  }
};

// Grid of the per-cell kernels: grid-stride loops, at most per_sm blocks of
// `threads` threads per SM.
static unsigned cell_grid(int64_t n, int sms, int threads, int per_sm) {
  int64_t b = ceil_div(n, threads);
  const int64_t cap = (int64_t)sms * per_sm;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

// Selected-ray N_H2 / N_CO columns of every cell: one launch, both directions
// of each axis per pencil read (ss_columns_kernel).
// Lists longer than this have the next column pass recompute every tile
// (marking them would cost more than it saves).
constexpr int64_t kColMarkMax = 1 << 16;

static void launch_columns(SteadySolver* s, const SteadyParams& par, cudaStream_t str,
                           bool force) {
  const SteadyDev& d = s->d;
  if (s->star) {  // columns towards the star (the cell's own half layer included)
    launch_point_source(s->nx, s->ny, s->nz, s->dens, d.x_h2, d.x_co, s->star_pos, s->star_lum,
                        s->cell, 1, nullptr, nullptr, nullptr, d.u_h2, d.u_co, s->st->sms, str);
    ss_col_moved_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(
        s->n, d.u_h2, d.u_co, ColQuiet{d.u_h2_last, d.u_co_last, d.q_moved, par.quiet_in_tol});
    return;
  }
  const ColumnsGrid g = columns_grid(s->nx, s->ny, s->nz);
  ss_columns_kernel<<<(unsigned)(g.nbx + g.nby + g.nbz), 32 * kColWarps,
                      columns_smem_bytes(s->nx, s->ny), str>>>(
      par.h2_implicit, s->nx, s->ny, s->nz, g.nbx, g.nby, d.l2, d.l3, d.fam, d.ds, d.u_h2,
      d.u_co, d.col_dirty, s->glob, force ? 1 : 0,
      ColQuiet{d.u_h2_last, d.u_co_last, d.q_moved, par.quiet_in_tol});
}

static int launch_iteration(SteadySolver* s, bool mixed, const SteadyParams& par,
                            cudaStream_t str) {
  const SteadyDev& d = s->d;
  // mixed: only the column tiles whose layers the last chemistry rewrote
  launch_columns(s, par, str, !mixed);
  ss_sum_kernel<<<s->nparts, kThreads, 0, str>>>(s->n, d.t_gas, s->parts);
  ss_finalize_kernel<<<1, 32, 0, str>>>(s->nparts, s->parts, s->n, s->glob);
  const int bt = s->cell_threads;
  const unsigned grid = cell_grid(s->n, s->st->sms, bt, s->cell_per_sm);
  if (mixed) {
    ss_mark_kernel<true><<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(s->n, d, par,
                                                                              s->glob);
    ss_col_mark_kernel<<<grid_for(kColMarkMax, s->st->sms, 1), kThreads, 0, str>>>(
        s->nx, s->ny, s->nz, d.list, d.col_dirty, s->glob, kColMarkMax);
    ss_chem_kernel<true><<<grid, bt, 0, str>>>(s->n, d, par, s->glob, s->a_nano, s->a_rest);
    ss_thermal_kernel<true><<<grid, bt, 0, str>>>(s->n, d, par, s->glob);
  } else {
    ss_chem_kernel<false><<<grid, bt, 0, str>>>(s->n, d, par, s->glob, s->a_nano, s->a_rest);
    ss_thermal_kernel<false><<<grid, bt, 0, str>>>(s->n, d, par, s->glob);
  }
  ss_record_kernel<<<1, 32, 0, str>>>(s->glob, s->hist, kMaxHist);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "steady iteration launch");
}

// kernels of one mixed iteration with the ray-set columns (the plain path
// launches two fewer; the point-source columns take four launches, not one)
constexpr int kLaunchesPerIteration = 8;
static int launches_per_iteration(const SteadySolver* s, bool mixed) {
  return kLaunchesPerIteration - (mixed ? 0 : 2) + (s->star ? 3 : 0);
}

}  // namespace p3d

using namespace p3d;

struct p3d_steady {
  SteadySolver s;
};

extern "C" {

int p3d_steady_create(p3d_steady_t** out, int64_t nx, int64_t ny, int64_t nz,
                      const double* density, const double* g0_ext, int64_t n_g0,
                      double cell_size, const double* dirs, const double* weights,
                      int64_t n_rays, double zeta0, double x_c_total, double x_o_total,
                      double t_init, const double* pe_table, int64_t n_bins, double log_psi_min,
                      double log_psi_step, int64_t n_psi, double eg_min, double eg_step,
                      int64_t n_eg, const double* bin_sigma_abs, const double* bin_dn_da_da,
                      const double* bin_is_nano, const double* h2_sigmas, const double* cii,
                      const double* oi63, const double* oi145, const double* ci) {
  if (!out) return set_error(P3D_EINVAL, "null handle pointer");
  *out = nullptr;
  if (nx <= 0 || ny <= 0 || nz <= 0) return set_error(P3D_EINVAL, "grid must be non-empty");
  // the worklist holds 32-bit cell indices
  if (nx > INT32_MAX / ny || nx * ny > INT32_MAX / nz)
    return set_error(P3D_EINVAL, "grid of %lld x %lld x %lld cells exceeds 2^31 - 1 cells",
                     (long long)nx, (long long)ny, (long long)nz);
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if (!density || !g0_ext || !dirs || !weights || !pe_table || !bin_sigma_abs ||
      !bin_dn_da_da || !bin_is_nano || !h2_sigmas || !cii || !oi63 || !oi145 || !ci)
    return set_error(P3D_EINVAL, "null argument");
  if (n_psi < 2 || n_eg < 2 || n_bins < 1) return set_error(P3D_EINVAL, "bad PE table shape");
  p3d_steady* h = new p3d_steady();
  SteadySolver* s = &h->s;
  s->st = st;
  s->nx = nx; s->ny = ny; s->nz = nz; s->n = nx * ny * nz;
  const int64_t n = s->n;
  s->cell = cell_size;
  if ((rc = build_rayset(dirs, weights, n_rays, g0_ext, n_g0, cell_size, &s->rays))) {
    delete h;
    return rc;
  }
  SteadyParams& p = s->par;
  p.zeta0 = zeta0; p.x_c_total = x_c_total; p.x_o_total = x_o_total; p.x_hcop = 1e-10;
  p.t_init = t_init; p.f_nano = 1.0; p.e_g = 0.1;
  p.sigma_nano = h2_sigmas[0]; p.sigma_lc = h2_sigmas[1]; p.sigma_sil = h2_sigmas[2];
  p.w_chem = 0.5; p.w_t = 0.5; p.chem_rtol = 1e-12; p.therm_tol = 1e-12;
  p.therm_tol_mixed = 1e-10;
  p.chem_max_iter = 200; p.therm_max_iter = 80; p.n_rays = (int)n_rays;
  p.h2_implicit = 0;
  for (int k = 0; k < 8; ++k) p.rs[k] = 1.0;
  p.fix_t = 0;
  p.exact_roots = 0;
  // one cell per warp up to ~7 cells per FP64 unit (608 schedulers): above
  // that, 32 cells per warp keep the units busier (128^3 slab: 4096 cells
  // best, 2048 and 8192 within 1%)
  p.coop_max = 4096;
  p.quiet_tol = p.quiet_in_tol = p.quiet_b_tol = p.quiet_r_tol = 0.0;
  p.pe = PeGrid{log_psi_min, log_psi_step, eg_min, eg_step, (int)n_psi, (int)n_eg};
  memcpy(p.lines.cii, cii, sizeof(p.lines.cii));
  memcpy(p.lines.oi63, oi63, sizeof(p.lines.oi63));
  memcpy(p.lines.oi145, oi145, sizeof(p.lines.oi145));
  memcpy(p.lines.ci, ci, sizeof(p.lines.ci));
  p.lf = make_line_fast(p.lines);
  SteadyDev& d = s->d;
  double** dbl[] = {&s->dens, &d.g0, &d.av, &d.nh_col, &s->nh2_full, &s->nco_full, &d.ds,
                    &d.kpd0, &d.uv0, &d.kci, &d.kco0, &d.hci0, &d.zeta, &d.td_rad, &d.t_gas,
                    &d.x_hi, &d.x_h2, &d.x_cp, &d.x_c, &d.x_co, &d.x_o, &d.x_e, &d.l2, &d.l3, &d.f_nano, &d.e_g, &d.u_h2,
                    &d.u_co, &d.t_prev, &d.r_prev, &d.t_lo, &d.t_hi, &d.span, &d.t_root, &d.u_h2_last, &d.u_co_last, &d.b_last, &d.chg_last, &d.rh2_cell, &d.chg_spec, &d.fh2,
                    &d.gamma_pe, &d.t_dust, &s->scratch};
  for (double** q : dbl)
    if ((rc = s->alloc(q, n))) { delete h; return rc; }
  d.dens = s->dens;
  if ((rc = s->alloc(&d.ray, n)) || (rc = s->alloc(&d.fam, n)) || (rc = s->alloc(&d.flags, n)) ||
      (rc = s->alloc(&d.list, n)) || (rc = s->alloc(&d.bis_node, n)) ||
      (rc = s->alloc(&d.bis_margin, n)) || (rc = s->alloc(&d.fh2_slope, n)) ||
      (rc = s->alloc(&d.col_dirty, column_tiles(nx, ny, nz))) ||
      (rc = s->alloc(&d.q_self, n)) || (rc = s->alloc(&d.q_moved, n))) {
    delete h;
    return rc;
  }
  size_t npe = (size_t)n_psi * n_eg;
  double *tab = nullptr, *bins = nullptr;
  if ((rc = s->alloc(&s->a_nano, 2 * npe)) || (rc = s->alloc(&tab, npe * n_bins)) ||
      (rc = s->alloc(&bins, 3 * n_bins)) || (rc = s->alloc(&s->ray_ds, n_rays)) ||
      (rc = s->alloc(&s->ray_fam, n_rays))) {
    delete h;
    return rc;
  }
  s->a_rest = s->a_nano + npe;
  s->nparts = 2 * st->sms;
  if ((rc = s->alloc(&s->parts, s->nparts)) || (rc = s->alloc(&s->glob, 1)) ||
      (rc = s->alloc(&s->hist, kHistCols * (size_t)kMaxHist))) {
    delete h;
    return rc;
  }
  cudaError_t e = cudaMallocHost(&s->hist_host, sizeof(double) * kHistCols * kMaxHist);
  if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaMallocHost"); }
  cudaStream_t str = st->stream;
  std::vector<double> hb(3 * n_bins), hds(n_rays);
  std::vector<int> hfam(n_rays);
  for (int64_t b = 0; b < n_bins; ++b) {
    hb[b] = bin_sigma_abs[b];
    hb[n_bins + b] = bin_dn_da_da[b];
    hb[2 * n_bins + b] = bin_is_nano[b];
  }
  for (int64_t r = 0; r < n_rays; ++r) {
    hds[r] = s->rays.ds[r];
    hfam[r] = s->rays.axis[r] * 2 + s->rays.fwd[r];
  }
  {
    CoLevel co[40];
    co_ladder_host(co);
    p.theta2 = co[0].t_u;
    float l32[20], co32[200];
    const double* L[5] = {p.lines.cii, p.lines.oi63, p.lines.oi145, p.lines.ci, p.lines.ci + 5};
    for (int k = 0; k < 5; ++k) {
      l32[4 * k] = (float)L[k][1];
      l32[4 * k + 1] = (float)L[k][2];
      l32[4 * k + 2] = (float)(L[k][3] / L[k][4]);
      l32[4 * k + 3] = (float)L[k][4];
    }
    for (int k = 0; k < 40; ++k) {
      co32[5 * k] = (float)co[k].t_u;
      co32[5 * k + 1] = (float)co[k].a_co;
      co32[5 * k + 2] = (float)co[k].g_ratio;
      co32[5 * k + 3] = (float)co[k].j_factor;
      co32[5 * k + 4] = (float)(co[k].ahv / co[0].ahv);
    }
    e = cudaMemcpyToSymbolAsync(c_co_ss, co, sizeof(co), 0, cudaMemcpyHostToDevice, str);
    if (e == cudaSuccess)
      e = cudaMemcpyToSymbolAsync(c_lines32, l32, sizeof(l32), 0, cudaMemcpyHostToDevice, str);
    if (e == cudaSuccess)
      e = cudaMemcpyToSymbolAsync(c_co32, co32, sizeof(co32), 0, cudaMemcpyHostToDevice, str);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->dens, density, sizeof(double) * n, cudaMemcpyHostToDevice, str);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(tab, pe_table, sizeof(double) * npe * n_bins, cudaMemcpyHostToDevice, str);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(bins, hb.data(), sizeof(double) * hb.size(), cudaMemcpyHostToDevice, str);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->ray_ds, hds.data(), sizeof(double) * n_rays, cudaMemcpyHostToDevice, str);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->ray_fam, hfam.data(), sizeof(int) * n_rays, cudaMemcpyHostToDevice, str);
  if (e == cudaSuccess)
    e = launch_pe_condense(tab, (int)n_bins, p.pe, bins, bins + n_bins, bins + 2 * n_bins,
                           s->a_nano, s->a_rest, str);
  if (e == cudaSuccess) {
    ss_bisect_table_kernel<<<1, 32, 0, str>>>();
    ss_coop_table_kernel<<<1, 64, 0, str>>>(p.lf);
    e = cudaGetLastError();
  }
  {
    // the strided-axis column blocks keep two chunk-sum arrays per pencil
    // tile in shared memory (16 KB for 256-cell pencils)
    const size_t sm = columns_smem_bytes(nx, ny);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess && sm > (size_t)optin)
      e = cudaErrorInvalidValue;
    if (e == cudaSuccess && sm > 48 * 1024)
      e = cudaFuncSetAttribute(ss_columns_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)sm);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  if (e != cudaSuccess) { delete h; return cuda_fail(e, "steady create"); }
  *out = h;
  return P3D_OK;
}

int p3d_steady_reset(p3d_steady_t* h) {
  if (!h) return set_error(P3D_EINVAL, "null handle");
  SteadySolver* s = &h->s;
  cudaStream_t str = s->st->stream;
  SteadyDev& d = s->d;
  if (!s->ev_start) {
    cudaEventCreate(&s->ev_start);
    cudaEventCreate(&s->ev_stop);
  }
  cudaEventRecord(s->ev_start, str);
  cudaError_t e;
  if (s->star) {
    e = launch_point_source(s->nx, s->ny, s->nz, s->dens, nullptr, nullptr, s->star_pos,
                            s->star_lum, s->cell, 0, d.g0, d.av, d.nh_col, s->nh2_full,
                            s->nco_full, s->st->sms, str);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.ray, 0xff, sizeof(int32_t) * s->n, str);
  } else {
  int err = 0;
  void* work = s->st->slot(kSlotRtWork, rt_work_bytes(s->n), &err);
  if (err) return err;
  e = launch_fuv_full(s->nx, s->ny, s->nz, s->dens, nullptr, nullptr, s->rays, work, d.g0,
                                  d.av, d.nh_col, s->nh2_full, s->nco_full, d.ray, s->st->sms,
                                  str);
  }
  if (e != cudaSuccess) return cuda_fail(e, "reset: ray march");
  ss_setup_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(s->n, d, s->par,
                                                                        s->ray_ds, s->ray_fam);
  cudaMemsetAsync(d.u_h2, 0, sizeof(double) * s->n, str);
  cudaMemsetAsync(d.u_co, 0, sizeof(double) * s->n, str);
  ss_reset_globals_kernel<<<1, 32, 0, str>>>(s->glob);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "reset launch");
  s->iters_done = 0;
  s->launches = (s->star ? 3 : rt_launch_count(s->rays)) + 2;  // ray march, setup, globals
  s->last_dmax = INFINITY;
  return P3D_OK;
}

int p3d_steady_run(p3d_steady_t* h, int mixed, int64_t max_outer, double tol, int64_t n_allow,
                   double w_chem, double w_t, int64_t* iters_out, double* dmax_out) {
  if (!h) return set_error(P3D_EINVAL, "null handle");
  if (max_outer < 0 || max_outer > kMaxHist) return set_error(P3D_EINVAL, "max_outer");
  if (!(w_chem >= 0.0 && w_chem < 1.0) || !(w_t >= 0.0 && w_t < 1.0))
    return set_error(P3D_EINVAL, "damping weights must lie in [0, 1)");
  SteadySolver* s = &h->s;
  cudaStream_t str = s->st->stream;
  if (!(tol > 0.0) || n_allow < 0) return set_error(P3D_EINVAL, "tol must be > 0, n_allow >= 0");
  SteadyParams par = s->par;
  par.w_chem = w_chem;
  par.w_t = w_t;
  par.count_thr[0] = tol * 100.0;
  par.count_thr[1] = tol;
  par.count_thr[2] = tol * 0.01;
  // a cell leaves the worklist once its last solve moved it by <= tol (the
  // convergence threshold itself) and its columns have moved by <= tol
  // since; at 1e-2 / 1e-1 tol the 128^3 slab's solve took 10% longer for
  // the same converged state (every settled cell within 1e-6 of plain FP64
  // either way)
  par.quiet_tol = tol;
  par.quiet_in_tol = tol;
  // the Doppler width reaches a cell only through f_H2: held to the columns'
  // tolerance
  par.quiet_b_tol = tol;
  // a small step alone does not make a cell settled: a T update confined to
  // a stale bracket (or hopping across a collapsed one) moves T by ~1e-12
  // while G(T) - T stays large, and only re-solving the cell breaks such a
  // bracket; its thermal residual must be small too
  par.quiet_r_tol = tol;
  auto conv = [&](const double* hrow) {
    return hrow[0] < tol || (double)hrow[4] <= (double)n_allow;
  };
  int64_t it = s->iters_done;
  const int64_t stop = s->iters_done + max_outer;
  if (stop > kMaxHist) return set_error(P3D_EINVAL, "iteration history full: reset first");
  bool done = false;
  // the first column pass of a run recomputes every tile (the state may have
  // been reset, set or refined since the last pass)
  cudaError_t e = cudaMemsetAsync(s->d.col_dirty, 1, (size_t)column_tiles(s->nx, s->ny, s->nz),
                                  str);
  // the worklist's per-cell tests under this run's tolerances (the first,
  // full column pass forms the column test)
  if (e == cudaSuccess) {
    ss_quiet_init_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(s->n, s->d, par);
    e = cudaGetLastError();
    ++s->launches;
  }
  if (e != cudaSuccess) return cuda_fail(e, "column tiles");
  // one iteration: launch, synchronise, test
  auto single = [&]() -> int {
    int rc = launch_iteration(s, mixed != 0, par, str);
    if (rc) return rc;
    cudaError_t es = cudaMemcpyAsync(s->hist_host + kHistCols * it, s->hist + kHistCols * it,
                                     sizeof(double) * kHistCols, cudaMemcpyDeviceToHost, str);
    if (es == cudaSuccess) es = cudaStreamSynchronize(str);
    if (es != cudaSuccess) return cuda_fail(es, "outer iteration");
    s->launches += launches_per_iteration(s, mixed != 0);
    s->last_dmax = s->hist_host[kHistCols * it];
    bool c = conv(s->hist_host + kHistCols * it);
    ++it;
    if (c && it > 2) done = true;
    return P3D_OK;
  };
  if (!mixed || max_outer < kGraphIters) {
    // plain path (and short mixed runs): once per iteration
    while (it < stop && !done) {
      int rc = single();
      if (rc) return rc;
    }
  } else {
    // mixed path: a graph of kGraphIters iterations, tested per launch
    if (!s->graph || s->graph_mixed != 1 || memcmp(&s->graph_par, &par, sizeof(par)) != 0) {
      if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
      cudaGraph_t g;
      e = cudaStreamBeginCapture(str, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return cuda_fail(e, "begin capture");
      for (int k = 0; k < kGraphIters; ++k) {
        int rc = launch_iteration(s, true, par, str);
        if (rc) { cudaStreamEndCapture(str, &g); return rc; }
      }
      e = cudaStreamEndCapture(str, &g);
      if (e != cudaSuccess) return cuda_fail(e, "end capture");
      e = cudaGraphInstantiate(&s->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
      s->graph_mixed = 1;
      s->graph_par = par;
    }
    while (it < stop && !done) {
      if (stop - it < kGraphIters) {  // the remainder, one at a time: max_outer is a cap
        int rc = single();
        if (rc) return rc;
        continue;
      }
      e = cudaGraphLaunch(s->graph, str);
      s->launches += (int64_t)launches_per_iteration(s, true) * kGraphIters;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->hist_host + kHistCols * it, s->hist + kHistCols * it,
                            sizeof(double) * kHistCols * kGraphIters, cudaMemcpyDeviceToHost, str);
      if (e == cudaSuccess) e = cudaStreamSynchronize(str);
      if (e != cudaSuccess) return cuda_fail(e, "mixed graph launch");
      // the device ran all kGraphIters iterations: count them all (the
      // history rows and the device's iteration counter stay in step with
      // the host's, which a later run() after a dust step relies on) and
      // test convergence on the batch's last iteration, the state returned
      const double* last = s->hist_host + kHistCols * (it + kGraphIters - 1);
      s->last_dmax = last[0];
      it += kGraphIters;
      if (conv(last) && it > 2) done = true;
    }
  }
  s->iters_done = it;
  if (s->ev_stop) cudaEventRecord(s->ev_stop, str);
  if (iters_out) *iters_out = it;
  if (dmax_out) *dmax_out = s->last_dmax;
  return done ? P3D_OK : set_error(P3D_ECONVERGE, "not converged after %lld outer iterations "
                                   "(largest relative change %.3e)", (long long)it, s->last_dmax);
}

int p3d_steady_history(p3d_steady_t* h, double* out, int64_t max_n, int64_t* n_out) {
  if (!h || !out) return set_error(P3D_EINVAL, "null argument");
  SteadySolver* s = &h->s;
  int64_t k = s->iters_done < max_n ? s->iters_done : max_n;
  cudaError_t e = cudaMemcpy(out, s->hist, sizeof(double) * kHistCols * k, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "history copy");
  if (n_out) *n_out = k;
  return P3D_OK;
}

int p3d_steady_get(p3d_steady_t* h, int field, double* host_out) {
  if (!h || !host_out) return set_error(P3D_EINVAL, "null argument");
  SteadySolver* s = &h->s;
  SteadyDev& d = s->d;
  const double* src = nullptr;
  cudaStream_t str = s->st->stream;
  switch (field) {
    case P3D_F_T_GAS: src = d.t_gas; break;
    case P3D_F_X_HI: src = d.x_hi; break;
    case P3D_F_X_H2: src = d.x_h2; break;
    case P3D_F_X_CP: src = d.x_cp; break;
    case P3D_F_X_C: src = d.x_c; break;
    case P3D_F_X_CO: src = d.x_co; break;
    case P3D_F_X_O: src = d.x_o; break;
    case P3D_F_X_E: src = d.x_e; break;
    case P3D_F_G0: src = d.g0; break;
    case P3D_F_A_V: src = d.av; break;
    case P3D_F_N_H: src = d.nh_col; break;
    case P3D_F_T_DUST: src = d.t_dust; break;
    case P3D_F_GAMMA_PE: src = d.gamma_pe; break;
    case P3D_F_ZETA: src = d.zeta; break;
    case P3D_F_F_SH_H2: src = d.fh2; break;
    case P3D_F_CHANGE: src = d.chg_last; break;
    case P3D_F_F_NANO: src = d.f_nano; break;
    case P3D_F_E_G: src = d.e_g; break;
    case P3D_F_GAMMA:
    case P3D_F_LAMBDA:
      ss_heating_cooling_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(
          s->n, d, s->par, field == P3D_F_LAMBDA ? 1 : 0, s->scratch);
      src = s->scratch;
      break;
    case P3D_F_N_H2:
    case P3D_F_N_CO: {
      ss_columns_out_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(
          s->n, field == P3D_F_N_H2 ? 1 : 0, s->par.h2_implicit, s->dens, d.x_h2, d.ds, d.u_h2,
          d.u_co, s->scratch);
      src = s->scratch;
      break;
    }
    default: return set_error(P3D_EINVAL, "unknown field %d", field);
  }
  cudaError_t e = cudaMemcpyAsync(host_out, src, sizeof(double) * s->n, cudaMemcpyDeviceToHost,
                                  str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "steady get");
}

int p3d_steady_set_point_source(p3d_steady_t* h, const double* star_pos, double l_fuv) {
  if (!h) return set_error(P3D_EINVAL, "null handle");
  SteadySolver* s = &h->s;
  if (!(l_fuv > 0.0)) {
    s->star = 0;
    return P3D_OK;
  }
  if (!star_pos) return set_error(P3D_EINVAL, "null star position");
  if (s->par.h2_implicit)
    return set_error(P3D_EINVAL, "the point-source columns include the cell's own layer");
  s->star = 1;
  for (int k = 0; k < 3; ++k) s->star_pos[k] = star_pos[k];
  s->star_lum = l_fuv;
  if (s->graph) {  // the captured iterations hold the other columns launch
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  return P3D_OK;
}

int p3d_steady_dust_step(p3d_steady_t* h) {
  if (!h) return set_error(P3D_EINVAL, "null handle");
  SteadySolver* s = &h->s;
  cudaStream_t str = s->st->stream;
  cudaError_t e = launch_dust_evolve(s->n, s->d.g0, s->dens, s->d.f_nano, s->d.e_g, s->st->sms,
                                     str);
  if (e == cudaSuccess) {
    ss_dust_restart_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(s->n, s->d);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return cuda_fail(e, "dust step launch");
  s->launches += 2;
  return P3D_OK;
}

int p3d_steady_columns(p3d_steady_t* h, double* nh2_out, double* nco_out) {
  if (!h || !nh2_out || !nco_out) return set_error(P3D_EINVAL, "null argument");
  SteadySolver* s = &h->s;
  cudaStream_t str = s->st->stream;
  launch_columns(s, s->par, str, true);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "columns launch");
  ++s->launches;
  for (int which = 1; which >= 0; --which) {
    ss_columns_out_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(
        s->n, which, s->par.h2_implicit, s->dens, s->d.x_h2, s->d.ds, s->d.u_h2, s->d.u_co,
        s->scratch);
    e = cudaMemcpyAsync(which ? nh2_out : nco_out, s->scratch, sizeof(double) * s->n,
                        cudaMemcpyDeviceToHost, str);
    if (e == cudaSuccess) e = cudaStreamSynchronize(str);
    if (e != cudaSuccess) return cuda_fail(e, "columns copy");
  }
  return P3D_OK;
}

int p3d_steady_set(p3d_steady_t* h, int field, const double* host_in) {
  if (!h || !host_in) return set_error(P3D_EINVAL, "null argument");
  SteadySolver* s = &h->s;
  SteadyDev& d = s->d;
  double* dst = nullptr;
  switch (field) {
    case P3D_F_T_GAS: dst = d.t_gas; break;
    case P3D_F_X_HI: dst = d.x_hi; break;
    case P3D_F_X_H2: dst = d.x_h2; break;
    case P3D_F_X_CP: dst = d.x_cp; break;
    case P3D_F_X_C: dst = d.x_c; break;
    case P3D_F_X_CO: dst = d.x_co; break;
    default: return set_error(P3D_EINVAL, "field %d cannot be set (T_gas and the five "
                              "chemistry unknowns can)", field);
  }
  for (int64_t i = 0; i < s->n; ++i)
    if (!(host_in[i] > 0.0) || !std::isfinite(host_in[i]))
      return set_error(P3D_EINVAL, "value %lld must be finite and > 0", (long long)i);
  cudaError_t e = cudaMemcpyAsync(dst, host_in, sizeof(double) * s->n, cudaMemcpyHostToDevice,
                                  s->st->stream);
  if (e == cudaSuccess && (field == P3D_F_X_H2 || field == P3D_F_X_CO)) {
    ss_layers_kernel<<<grid_for(s->n, s->st->sms, 8), kThreads, 0, s->st->stream>>>(s->n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st->stream);
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "steady set");
}

int p3d_steady_get_ray(p3d_steady_t* h, int32_t* host_out) {
  if (!h || !host_out) return set_error(P3D_EINVAL, "null argument");
  SteadySolver* s = &h->s;
  cudaError_t e = cudaMemcpy(host_out, s->d.ray, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "steady get ray");
}

int p3d_steady_elapsed_ms(p3d_steady_t* h, double* ms) {
  if (!h || !ms) return set_error(P3D_EINVAL, "null argument");
  SteadySolver* s = &h->s;
  if (!s->ev_start) return set_error(P3D_EINVAL, "no reset recorded");
  cudaError_t e = cudaEventSynchronize(s->ev_stop);
  float f = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&f, s->ev_start, s->ev_stop);
  if (e != cudaSuccess) return cuda_fail(e, "elapsed");
  *ms = f;
  return P3D_OK;
}

int p3d_steady_launch_count(p3d_steady_t* h, int64_t* out) {
  if (!h || !out) return set_error(P3D_EINVAL, "null argument");
  *out = h->s.launches;
  return P3D_OK;
}

int p3d_steady_kernel_times(p3d_steady_t* h, int reps, double* ms4) {
  if (!h || !ms4 || reps < 1) return set_error(P3D_EINVAL, "bad argument");
  SteadySolver* s = &h->s;
  cudaStream_t str = s->st->stream;
  const SteadyDev& d = s->d;
  SteadyParams par = s->par;
  par.count_thr[0] = par.count_thr[1] = par.count_thr[2] = 1.0;
  par.quiet_tol = 0.0;  // no compaction: every cell solved
  par.quiet_in_tol = 0.0;
  par.quiet_r_tol = 0.0;
  par.exact_roots = 1;  // the path whose FP64 work the roofline counts
  par.quiet_b_tol = 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int bt = s->cell_threads;
  const unsigned grid = cell_grid(s->n, s->st->sms, bt, s->cell_per_sm);
  for (int which = 0; which < 4; ++which) {
    cudaEventRecord(e0, str);
    for (int r = 0; r < reps; ++r) {
      if (which == 0) {
        launch_columns(s, par, str, true);
      } else if (which == 1) {
        ss_sum_kernel<<<s->nparts, kThreads, 0, str>>>(s->n, d.t_gas, s->parts);
        ss_finalize_kernel<<<1, 32, 0, str>>>(s->nparts, s->parts, s->n, s->glob);
      } else if (which == 2) {
        ss_finalize_kernel<<<1, 32, 0, str>>>(s->nparts, s->parts, s->n, s->glob);
        ss_mark_kernel<true><<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(s->n, d, par,
                                                                                  s->glob);
        ss_chem_kernel<true><<<grid, bt, 0, str>>>(s->n, d, par, s->glob, s->a_nano, s->a_rest);
        ss_thermal_kernel<true><<<grid, bt, 0, str>>>(s->n, d, par, s->glob);
      } else {
        ss_finalize_kernel<<<1, 32, 0, str>>>(s->nparts, s->parts, s->n, s->glob);
        ss_chem_kernel<false><<<grid, bt, 0, str>>>(s->n, d, par, s->glob, s->a_nano,
                                                    s->a_rest);
        ss_thermal_kernel<false><<<grid, bt, 0, str>>>(s->n, d, par, s->glob);
      }
    }
    cudaEventRecord(e1, str);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return cuda_fail(e, "kernel timing");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms4[which] = (double)ms / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return P3D_OK;
}

// Live FP64 FMA throughput of the current device: 8 independent DFMA chains
// per thread, 2 flops per DFMA, timed with CUDA events.
__global__ void fp64_peak_kernel(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

int p3d_fp64_peak_tflops(double* tflops) {
  if (!tflops) return set_error(P3D_EINVAL, "null argument");
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  int err;
  double* dummy = (double*)st->slot(20, 64, &err);
  if (err) return err;
  const int blocks = st->sms * 4, threads = 256, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp64_peak_kernel<<<blocks, threads, 0, st->stream>>>(dummy, 64, 0.999999, 1e-7);
  cudaEventRecord(e0, st->stream);
  fp64_peak_kernel<<<blocks, threads, 0, st->stream>>>(dummy, iters, 0.999999, 1e-7);
  cudaEventRecord(e1, st->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(e, "fp64 peak probe");
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return P3D_OK;
}

int p3d_steady_autotune(p3d_steady_t* h, int warm_iters, int32_t* cfg_out, double* ms_out) {
  if (!h || warm_iters < 1 || warm_iters > 64)
    return set_error(P3D_EINVAL, "autotune: null handle or warm_iters outside [1, 64]");
  SteadySolver* s = &h->s;
  cudaStream_t str = s->st->stream;
  // a representative state: warm_iters mixed iterations from the initial one
  int rc = p3d_steady_reset(h);
  if (rc) return rc;
  rc = p3d_steady_run(h, 1, warm_iters, 1e-300, 0, 0.1, 0.5, nullptr, nullptr);
  if (rc && rc != P3D_ECONVERGE) return rc;
  SteadyParams par = s->par;
  par.count_thr[0] = par.count_thr[1] = par.count_thr[2] = 1.0;
  par.quiet_tol = 0.0;  // every cell solved
  par.quiet_in_tol = 0.0;
  par.quiet_r_tol = 0.0;
  par.quiet_b_tol = 0.0;
  par.w_chem = 0.1;
  const SteadyDev& d = s->d;
  const int threads[2] = {128, 256};
  const int per_sm[6] = {2, 4, 8, 16, 32, 64};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = INFINITY;
  int bt = s->cell_threads, bp = s->cell_per_sm;
  cudaError_t e = cudaSuccess;
  for (int a = 0; a < 2 && e == cudaSuccess; ++a)
    for (int b = 0; b < 6 && e == cudaSuccess; ++b) {
      const unsigned grid = cell_grid(s->n, s->st->sms, threads[a], per_sm[b]);
      float ms = 0.f, tot = 0.f;
      for (int rep = 0; rep < 3; ++rep) {  // first launch warms, two timed
        cudaEventRecord(e0, str);
        ss_finalize_kernel<<<1, 32, 0, str>>>(s->nparts, s->parts, s->n, s->glob);
        ss_mark_kernel<true><<<grid_for(s->n, s->st->sms, 8), kThreads, 0, str>>>(s->n, d, par,
                                                                                  s->glob);
        ss_chem_kernel<true><<<grid, threads[a], 0, str>>>(s->n, d, par, s->glob, s->a_nano,
                                                           s->a_rest);
        ss_thermal_kernel<true><<<grid, threads[a], 0, str>>>(s->n, d, par, s->glob);
        cudaEventRecord(e1, str);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) break;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) tot += ms;
      }
      if (e == cudaSuccess && tot / 2 < best) {
        best = tot / 2;
        bt = threads[a];
        bp = per_sm[b];
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(e, "autotune");
  s->cell_threads = bt;
  s->cell_per_sm = bp;
  if (s->graph) {  // baked the old launch shape
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  if (cfg_out) { cfg_out[0] = bt; cfg_out[1] = bp; }
  if (ms_out) *ms_out = best;
  return p3d_steady_reset(h);
}

int p3d_steady_set_launch(p3d_steady_t* h, int threads, int blocks_per_sm) {
  if (!h) return set_error(P3D_EINVAL, "null handle");
  if (threads != 128 && threads != 256)
    return set_error(P3D_EINVAL, "launch shape: threads %d not 128 or 256", threads);
  if (blocks_per_sm < 1 || blocks_per_sm > 64)
    return set_error(P3D_EINVAL, "launch shape: blocks per SM %d outside [1, 64]", blocks_per_sm);
  SteadySolver* s = &h->s;
  s->cell_threads = threads;
  s->cell_per_sm = blocks_per_sm;
  if (s->graph) {  // baked the old launch shape
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  return P3D_OK;
}

int p3d_steady_set_coop_max(p3d_steady_t* h, int64_t max_cells) {
  if (!h) return set_error(P3D_EINVAL, "null handle");
  if (max_cells < 0) return set_error(P3D_EINVAL, "coop_max must be >= 0");
  h->s.par.coop_max = (int)(max_cells > INT32_MAX ? INT32_MAX : max_cells);
  if (h->s.graph) {  // baked the old parameters
    cudaGraphExecDestroy(h->s.graph);
    h->s.graph = nullptr;
  }
  return P3D_OK;
}

int p3d_steady_set_rate_scale(p3d_steady_t* h, const double* scale8) {
  if (!h || !scale8) return set_error(P3D_EINVAL, "null argument");
  for (int k = 0; k < 8; ++k)
    if (!(scale8[k] > 0.0) || !std::isfinite(scale8[k]))
      return set_error(P3D_EINVAL, "rate scale %d must be finite and > 0", k);
  for (int k = 0; k < 8; ++k) h->s.par.rs[k] = scale8[k];
  return P3D_OK;
}

int p3d_steady_set_fixed_temperature(p3d_steady_t* h, int fixed) {
  if (!h) return set_error(P3D_EINVAL, "null handle");
  h->s.par.fix_t = fixed ? 1 : 0;
  return P3D_OK;
}

int p3d_steady_adjoint(p3d_steady_t* h, const double* w6, double dx, int64_t max_sweeps,
                       double tol, double omega, double* grad9, double* grad_ln_nh,
                       double* loss2, int64_t* sweeps_out, int64_t* n_jump_out) {
  if (!h || !grad9 || !w6) return set_error(P3D_EINVAL, "null argument");
  if (max_sweeps < 1 || !(tol > 0.0) || !(dx > 0.0) || !(omega > 0.0 && omega <= 1.0))
    return set_error(P3D_EINVAL, "max_sweeps >= 1, tol > 0, dx > 0, 0 < omega <= 1 required");
  SteadySolver* s = &h->s;
  if (s->iters_done < 1) return set_error(P3D_EINVAL, "run the steady state before its adjoint");
  if (s->star)
    return set_error(P3D_EINVAL, "the adjoint covers the external ray-set field, not a point source");
  cudaStream_t str = s->st->stream;
  const int64_t n = s->n;
  const SteadyDev& d = s->d;
  // workspace (freed on return)
  std::vector<void*> mem;
  auto get = [&](size_t bytes) -> void* {
    void* q = nullptr;
    if (cudaMalloc(&q, bytes ? bytes : 8) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    mem.push_back(q);
    return q;
  };
  auto cleanup = [&]() {
    cudaStreamSynchronize(str);
    for (void* q : mem) cudaFree(q);
  };
  AdjArgs a;
  for (int k = 0; k < 6; ++k) a.w[k] = w6[k];
  const size_t nd = sizeof(double) * (size_t)n;
  a.jinv = (double*)get(36 * nd);
  a.jn2 = (double*)get(6 * nd);
  a.jn3 = (double*)get(6 * nd);
  a.jb = (double*)get(6 * nd);
  a.jth = (double*)get(6 * kAdjParams * nd);
  a.lam = (double*)get(6 * nd);
  a.cx2 = (double*)get(nd);
  a.cx3 = (double*)get(nd);
  a.a2 = (double*)get(nd);
  a.a3 = (double*)get(nd);
  a.qb = (double*)get(nd);
  a.jump = (int*)get(sizeof(int) * (size_t)n);
  a.teval = (double*)get(nd);
  a.dn = grad_ln_nh ? (double*)get(nd) : nullptr;
  double* qg0 = grad_ln_nh ? (double*)get(nd) : nullptr;
  double* qav = grad_ln_nh ? (double*)get(nd) : nullptr;
  double* qnh = grad_ln_nh ? (double*)get(nd) : nullptr;
  a.red = (double*)get(sizeof(double) * (size_t)s->nparts);
  a.scal = (double*)get(sizeof(double) * 2);
  a.dmax = (unsigned long long*)get(sizeof(unsigned long long));
  unsigned int* n_bad = (unsigned int*)get(sizeof(unsigned int));
  {
    const void* need[] = {a.jinv, a.jn2, a.jn3, a.jb, a.jth, a.lam, a.cx2, a.cx3, a.a2, a.a3,
                          a.qb, a.jump, a.teval, a.red, a.scal, a.dmax, n_bad};
    bool miss = false;
    for (const void* q : need) miss = miss || !q;
    if (grad_ln_nh) miss = miss || !a.dn || !qg0 || !qav || !qnh;
    if (miss) {
      cleanup();
      return set_error(P3D_ENOMEM, "adjoint workspace (%lld cells)", (long long)n);
    }
  }
  // columns and mean T of the final state
  const SteadyParams& par = s->par;
  int64_t dims[3] = {s->nx, s->ny, s->nz};
  launch_columns(s, par, str, true);
  ss_sum_kernel<<<s->nparts, kThreads, 0, str>>>(n, d.t_gas, s->parts);
  ss_finalize_kernel<<<1, 32, 0, str>>>(s->nparts, s->parts, n, s->glob);
  SteadyGlobals gl;
  cudaError_t e = cudaMemcpyAsync(&gl, s->glob, sizeof(gl), cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess) e = cudaMemsetAsync(n_bad, 0, sizeof(unsigned int), str);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.lam, 0, 6 * nd, str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "adjoint setup"); }
  const double b = gl.b_dop, dbdt = gl.b_dop / (2.0 * gl.t_mean);
  const unsigned grid = grid_for(n, s->st->sms, 4);
  adj_local_kernel<<<(unsigned)ceil_div(n, 128) < grid * 2u ? (unsigned)ceil_div(n, 128)
                                                             : grid * 2u,
                     128, 0, str>>>(n, d, par, s->a_nano, s->a_rest, b, a, n_bad);
  e = cudaGetLastError();
  if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "adjoint local launch"); }
  auto grid_sum = [&](const double* q, double* out) {
    ss_sum_kernel<<<s->nparts, kThreads, 0, str>>>(n, q, a.red);
    adj_finish_sum_kernel<<<1, 32, 0, str>>>(s->nparts, a.red, out);
  };
  // sweeps until the gradient changes by <= tol (relative to its largest
  // component) between checks
  auto gradient = [&](double* out) -> cudaError_t {
    for (int k = 0; k < kAdjParams; ++k) {
      adj_grad_kernel<<<grid, kThreads, 0, str>>>(n, a, k, a.cx2);
      grid_sum(a.cx2, a.scal + 1);
      cudaError_t e2 = cudaMemcpyAsync(out + k, a.scal + 1, sizeof(double),
                                       cudaMemcpyDeviceToHost, str);
      if (e2 != cudaSuccess) return e2;
    }
    return cudaStreamSynchronize(str);
  };
  int64_t sweeps = 0;
  double dmax = INFINITY;
  double prev[kAdjParams];
  for (int k = 0; k < kAdjParams; ++k) prev[k] = 0.0;
  const int kCheck = 20;
  while (sweeps < max_sweeps) {
    for (int k = 0; k < kCheck && sweeps < max_sweeps; ++k, ++sweeps) {
      adj_couple_kernel<<<grid, kThreads, 0, str>>>(n, d, a);
      for (int axis = 0; axis < 3; ++axis) {
        int64_t np = n / dims[axis];
        adj_scan_kernel<<<(unsigned)ceil_div(np, 128), 128, 0, str>>>(
            axis, s->nx, s->ny, s->nz, np, s->dens, d.fam, a);
      }
      grid_sum(a.qb, a.scal);
      cudaMemsetAsync(a.dmax, 0, sizeof(unsigned long long), str);
      adj_update_kernel<<<grid, kThreads, 0, str>>>(n, d, a, dx, a.scal, dbdt, omega);
    }
    e = gradient(grad9);
    if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "adjoint sweeps"); }
    double gm = 0.0, dg = 0.0;
    for (int k = 0; k < kAdjParams; ++k) {
      gm = fmax(gm, fabs(grad9[k]));
      dg = fmax(dg, fabs(grad9[k] - prev[k]));
      prev[k] = grad9[k];
    }
    dmax = gm > 0.0 ? dg / gm : dg;
    if (!std::isfinite(dmax)) break;
    if (dmax <= tol) break;
  }
  // gradient with respect to log n_H (optional)
  if (grad_ln_nh) {
    adj_couple_kernel<<<grid, kThreads, 0, str>>>(n, d, a);
    for (int axis = 0; axis < 3; ++axis) {
      int64_t np = n / dims[axis];
      adj_scan_kernel<<<(unsigned)ceil_div(np, 128), 128, 0, str>>>(
          axis, s->nx, s->ny, s->nz, np, s->dens, d.fam, a);
    }
    adj_dens_local_kernel<<<(unsigned)ceil_div(n, 128) < grid * 2u ? (unsigned)ceil_div(n, 128)
                                                                  : grid * 2u,
                            128, 0, str>>>(n, d, par, s->a_nano, s->a_rest, b, dx, a, qg0, qav,
                                           qnh);
    const RaySet& rs = s->rays;
    for (int r = 0; r < rs.n; ++r) {
      const int axis = rs.axis[r];
      int64_t np = n / dims[axis];
      adj_ray_scan_kernel<<<(unsigned)ceil_div(np, 128), 128, 0, str>>>(
          axis, rs.fwd[r], r, rs.ds[r], rs.g_ext[r] * rs.w[r], s->nx, s->ny, s->nz, np,
          s->dens, d.ray, qg0, qav, qnh, a.dn);
    }
    e = cudaMemcpyAsync(grad_ln_nh, a.dn, nd, cudaMemcpyDeviceToHost, str);
    if (e == cudaSuccess) e = cudaStreamSynchronize(str);
    if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "adjoint density gradient"); }
  }
  double lc = 0.0, lt = 0.0;
  adj_loss_kernel<<<grid, kThreads, 0, str>>>(n, d, a, dx, a.cx2, a.cx3);
  grid_sum(a.cx2, a.scal + 1);
  e = cudaMemcpyAsync(&lc, a.scal + 1, sizeof(double), cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  grid_sum(a.cx3, a.scal + 1);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&lt, a.scal + 1, sizeof(double), cudaMemcpyDeviceToHost, str);
  // jump cells
  adj_jump_count_kernel<<<grid, kThreads, 0, str>>>(n, a.jump, a.cx2);
  grid_sum(a.cx2, a.scal + 1);
  double nj = 0.0;
  unsigned int bad = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&nj, a.scal + 1, sizeof(double), cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&bad, n_bad, sizeof(bad), cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "adjoint results");
  if (loss2) { loss2[0] = lc; loss2[1] = lt / (double)n; }
  if (sweeps_out) *sweeps_out = sweeps;
  if (n_jump_out) *n_jump_out = (int64_t)nj;
  if (bad) return set_error(P3D_ECONVERGE, "adjoint: %u cells with a singular Jacobian", bad);
  if (!(dmax <= tol))
    return set_error(P3D_ECONVERGE, "adjoint sweeps did not reach tol (last relative gradient "
                     "change %.3e after %lld sweeps)", dmax, (long long)sweeps);
  return P3D_OK;
}

int p3d_steady_refine(p3d_steady_t* h, p3d_network_t* net, int32_t mixed, int32_t max_iter,
                      double rtol, double* cond_out, double* x31_out, int32_t* status_out) {
  if (!h || !net) return set_error(P3D_EINVAL, "null argument");
  int32_t ns = 0, ref = 0;
  int rc = p3d_network_info(net, &ns, &ref);
  if (rc) return rc;
  if (ns != kNetSpecies || !ref)
    return set_error(P3D_EINVAL, "refinement needs the reference 31-species network");
  SteadySolver* s = &h->s;
  if (s->iters_done < 1) return set_error(P3D_EINVAL, "run the steady state before refining it");
  cudaStream_t str = s->st->stream;
  const int64_t n = s->n;
  const SteadyDev& d = s->d;
  double *cond = nullptr, *x31 = nullptr;
  int32_t* st = nullptr;
  unsigned int* n_fail = nullptr;
  auto cleanup = [&]() {
    cudaStreamSynchronize(str);
    cudaFree(cond);
    cudaFree(x31);
    cudaFree(st);
    cudaFree(n_fail);
  };
  if (cudaMalloc(&cond, sizeof(double) * 7 * (size_t)n) != cudaSuccess ||
      cudaMalloc(&x31, sizeof(double) * kNetSpecies * (size_t)n) != cudaSuccess ||
      cudaMalloc(&st, sizeof(int32_t) * (size_t)n) != cudaSuccess ||
      cudaMalloc(&n_fail, sizeof(unsigned int)) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return set_error(P3D_ENOMEM, "refinement workspace (%lld cells)", (long long)n);
  }
  // columns and Doppler width of the current state
  const SteadyParams& par = s->par;
  launch_columns(s, par, str, true);
  ss_sum_kernel<<<s->nparts, kThreads, 0, str>>>(n, d.t_gas, s->parts);
  ss_finalize_kernel<<<1, 32, 0, str>>>(s->nparts, s->parts, n, s->glob);
  SteadyGlobals gl;
  cudaError_t e = cudaMemcpyAsync(&gl, s->glob, sizeof(gl), cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess) e = cudaMemsetAsync(n_fail, 0, sizeof(unsigned int), str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "refinement setup"); }
  const unsigned grid = grid_for(n, s->st->sms, 8);
  ss_refine_gather_kernel<<<grid, kThreads, 0, str>>>(n, d, par, gl.b_dop, cond, x31);
  if (cond_out) {
    e = cudaMemcpyAsync(cond_out, cond, sizeof(double) * 7 * (size_t)n, cudaMemcpyDeviceToHost,
                        str);
    if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "refinement conditions"); }
  }
  rc = p3d_network_steady_dev(net, n, cond, x31, mixed, 1, max_iter, rtol, st, nullptr, str);
  if (rc) { cleanup(); return rc; }
  ss_refine_scatter_kernel<<<grid, kThreads, 0, str>>>(n, d, par, x31, s->a_nano, s->a_rest,
                                                       n_fail);
  unsigned int fails = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess && x31_out)
    e = cudaMemcpyAsync(x31_out, x31, sizeof(double) * kNetSpecies * (size_t)n,
                        cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess && status_out)
    e = cudaMemcpyAsync(status_out, st, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&fails, n_fail, sizeof(fails), cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "refinement");
  s->launches += 7;
  if (fails) return set_error(P3D_ECONVERGE, "refinement: %u thermal roots not converged", fails);
  return P3D_OK;
}

int p3d_steady_column_maps(p3d_steady_t* h, double cell_size, int32_t los_axis,
                           double inclination_deg, double* maps) {
  if (!h || !maps) return set_error(P3D_EINVAL, "null argument");
  SteadySolver* s = &h->s;
  if (los_axis < 0 || los_axis > 2) return set_error(P3D_EINVAL, "los_axis must be 0, 1 or 2");
  const int64_t dims[3] = {s->nx, s->ny, s->nz};
  const int64_t npix = s->n / dims[los_axis];
  double* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * 6 * (size_t)npix);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(P3D_ENOMEM, "column maps output");
  }
  const SteadyDev& d = s->d;
  int rc = p3d_column_maps_dev(s->nx, s->ny, s->nz, s->dens, d.x_h2, d.x_co, d.x_cp, d.x_e,
                               cell_size, los_axis, inclination_deg, out, s->st->stream);
  if (!rc) {
    e = cudaMemcpyAsync(maps, out, sizeof(double) * 6 * (size_t)npix, cudaMemcpyDeviceToHost,
                        s->st->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "steady column maps");
  }
  cudaStreamSynchronize(s->st->stream);
  cudaFree(out);
  return rc;
}

int p3d_steady_destroy(p3d_steady_t* h) {
  delete h;
  return P3D_OK;
}

}  // extern "C"
