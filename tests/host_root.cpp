// Host build of the steady driver's thermal roots (prism3d_gb300/csrc/
// p3d_thermal_fast.cuh) for the CPU tests: the same source compiled by g++,
// so the mixed root's control flow (certified FP32 bisection, decision
// replay, warm start, pinned roots, FP64 polish) is checked against the
// plain root on the oracle's thermal contexts without a GPU.  Only the
// CUDA qualifiers and __ldg are mapped to host forms.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#undef __device__
#define __device__
#undef __forceinline__
#define __forceinline__ inline
#undef __noinline__
#define __noinline__ __attribute__((noinline))
#define __ldg(p) (*(p))
#include "../prism3d_gb300/csrc/p3d_thermal_fast.cuh"

using namespace p3d;

namespace {
CoLevel g_co[40];
float g_l32[20], g_co32[200];
double g_mid[1024];
BisectNode g_node[1024];
CoopLine g_coop[kCoopLines];
LineParams g_lp;
LineFast g_lf;
double g_theta2;

ThermalCtx make_ctx(const double* c10) {
  ThermalCtx c;
  c.gamma_fixed = c10[0];
  c.gg_coeff = c10[1];
  c.t_dust = c10[2];
  c.n_e = c10[3];
  c.n_hi = c10[4];
  c.n_h2 = c10[5];
  c.n_co = c10[6];
  c.n_cp_nh = c10[7];
  c.n_o_nh = c10[8];
  c.n_c_nh = c10[9];
  return c;
}
}  // namespace

// Line parameters in the solve_thermal_vec layout; co5: (40, 5) CO ladder
// rows (T_u, A, g_u/g_l, 1 + 0.1 J, A h nu).  The FP32 tables and the
// bisection tree are built as p3d_steady_create / ss_bisect_table_kernel do.
extern "C" void hr_init(const double* cii, const double* oi63, const double* oi145,
                        const double* ci, const double* co5) {
  memcpy(g_lp.cii, cii, sizeof(g_lp.cii));
  memcpy(g_lp.oi63, oi63, sizeof(g_lp.oi63));
  memcpy(g_lp.oi145, oi145, sizeof(g_lp.oi145));
  memcpy(g_lp.ci, ci, sizeof(g_lp.ci));
  for (int k = 0; k < 40; ++k) {
    g_co[k].t_u = co5[5 * k];
    g_co[k].a_co = co5[5 * k + 1];
    g_co[k].g_ratio = co5[5 * k + 2];
    g_co[k].j_factor = co5[5 * k + 3];
    g_co[k].ahv = co5[5 * k + 4];
  }
  g_theta2 = g_co[0].t_u;
  g_lf = make_line_fast(g_lp);
  const double* L[5] = {g_lp.cii, g_lp.oi63, g_lp.oi145, g_lp.ci, g_lp.ci + 5};
  for (int k = 0; k < 5; ++k) {
    g_l32[4 * k] = (float)L[k][1];
    g_l32[4 * k + 1] = (float)L[k][2];
    g_l32[4 * k + 2] = (float)(L[k][3] / L[k][4]);
    g_l32[4 * k + 3] = (float)L[k][4];
  }
  for (int k = 0; k < 40; ++k) {
    g_co32[5 * k] = (float)g_co[k].t_u;
    g_co32[5 * k + 1] = (float)g_co[k].a_co;
    g_co32[5 * k + 2] = (float)g_co[k].g_ratio;
    g_co32[5 * k + 3] = (float)g_co[k].j_factor;
    g_co32[5 * k + 4] = (float)(g_co[k].ahv / g_co[0].ahv);
  }
  double lo[1024], hi[1024];
  lo[1] = 10.0;
  hi[1] = 1e5;
  for (int k = 1; k < 1024; ++k) {
    double m = sqrt(lo[k] * hi[k]);
    g_mid[k] = m;
    g_node[k] = bisect_node(m, g_co);
    if (2 * k + 1 < 1024) {
      lo[2 * k] = lo[k];
      hi[2 * k] = m;
      lo[2 * k + 1] = m;
      hi[2 * k + 1] = hi[k];
    }
  }
  g_mid[0] = 0.0;
  for (int e = 0; e < kCoopLines; ++e) g_coop[e] = coop_line(e, g_lf, g_co);
}

// ctx: n x 10, row-major.  node / margin: in-out per cell (0 / 0 for a cell
// never solved).
extern "C" void hr_root_mixed(long n, const double* ctx, const double* t_warm,
                              const double* delta, int* node, float* margin, double tol,
                              double* t_out, int* n64, int* status) {
  for (long i = 0; i < n; ++i) {
    ThermalCtx c = make_ctx(ctx + 10 * i);
    int nd = node[i], st = 0, ev = 0;
    float mg = margin[i];
    t_out[i] = root_mixed(c, g_lf, g_co, g_theta2, g_l32, g_co32, g_mid, g_node, tol, 80, t_warm[i],
                          delta[i], &nd, &mg, &st, &ev);
    node[i] = nd;
    margin[i] = mg;
    n64[i] = ev;
    status[i] = st;
  }
}

// The same with the warp-cooperative form of the FP64 net heating (on the
// host its table summed in order).
extern "C" void hr_root_mixed_coop(long n, const double* ctx, const double* t_warm,
                                   const double* delta, int* node, float* margin, double tol,
                                   double* t_out, int* n64, int* status) {
  for (long i = 0; i < n; ++i) {
    ThermalCtx c = make_ctx(ctx + 10 * i);
    int nd = node[i], st = 0, ev = 0;
    float mg = margin[i];
    t_out[i] = root_mixed<true>(c, g_lf, g_co, g_theta2, g_l32, g_co32, g_mid, g_node, tol, 80,
                                t_warm[i], delta[i], &nd, &mg, &st, &ev, g_coop);
    node[i] = nd;
    margin[i] = mg;
    n64[i] = ev;
    status[i] = st;
  }
}

// The mixed root's form of the FP64 net heating (power laws as products).
extern "C" void hr_net64_mixed(long n, const double* ctx, const double* t, double* out) {
  for (long i = 0; i < n; ++i) {
    ThermalCtx c = make_ctx(ctx + 10 * i);
    out[i] = net_heating_mixed64_body(t[i], c, g_lf, g_co, g_theta2);
  }
}

extern "C" void hr_net64_coop(long n, const double* ctx, const double* t, double* out) {
  for (long i = 0; i < n; ++i) {
    ThermalCtx c = make_ctx(ctx + 10 * i);
    out[i] = net_heating_coop64(t[i], c, g_coop, g_co, g_theta2);
  }
}

extern "C" void hr_root_plain(long n, const double* ctx, double tol, double* t_out, int* n64,
                              int* status) {
  for (long i = 0; i < n; ++i) {
    ThermalCtx c = make_ctx(ctx + 10 * i);
    int st = 0, ev = 0;
    t_out[i] = root_plain(c, g_lf, g_co, g_theta2, tol, 80, &st, &ev);
    n64[i] = ev;
    status[i] = st;
  }
}

extern "C" void hr_net64(long n, const double* ctx, const double* t, double* out) {
  for (long i = 0; i < n; ++i) {
    ThermalCtx c = make_ctx(ctx + 10 * i);
    out[i] = net_heating_fast64_body(t[i], c, g_lf, g_co, g_theta2);
  }
}

// Diagnostics Gamma and Lambda at t (heating_cooling64).
extern "C" void hr_heating_cooling(long n, const double* ctx, const double* t, double* gamma,
                                   double* lambda) {
  for (long i = 0; i < n; ++i) {
    ThermalCtx c = make_ctx(ctx + 10 * i);
    heating_cooling64(t[i], c, g_lp, g_co, gamma + i, lambda + i);
  }
}
