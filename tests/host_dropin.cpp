// Host build of the drop-in kernels' cell functions for the CPU tests: the
// reference's 10 + 3 thermal root and its net heating (prism3d_gb300/csrc/
// p3d_thermal.cuh, rust/src/thermal.rs) and the explicit-Euler chemistry
// (p3d_chem.cuh, rust/src/chemistry.rs), the same source compiled by g++
// and checked against the reference's own values.  Only the CUDA
// qualifiers are mapped to host forms.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#undef __device__
#define __device__
#undef __forceinline__
#define __forceinline__ inline
#include "../prism3d_gb300/csrc/p3d_chem.cuh"
#include "../prism3d_gb300/csrc/p3d_thermal.cuh"

using namespace p3d;

namespace {
CoLevel g_co[40];
LineParams g_lp;

ThermalCtx make_ctx(const double* const* ctx, long i) {
  ThermalCtx c;
  c.gamma_fixed = ctx[0][i];
  c.gg_coeff = ctx[1][i];
  c.t_dust = ctx[2][i];
  c.n_e = ctx[3][i];
  c.n_hi = ctx[4][i];
  c.n_h2 = ctx[5][i];
  c.n_co = ctx[6][i];
  c.n_cp_nh = ctx[7][i];
  c.n_o_nh = ctx[8][i];
  c.n_c_nh = ctx[9][i];
  return c;
}
}  // namespace

// Line parameters [freq, A, T_ul, g_u, g_l] (ci: 609 then 370 um); co5: the
// (40, 5) CO ladder rows (T_u, A, g_u/g_l, 1 + 0.1 J, A h nu).
extern "C" void hd_init(const double* cii, const double* oi63, const double* oi145,
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
}

// ctx: 10 pointers to the context arrays (solve_thermal_vec order).
extern "C" void hd_thermal13(long n, const double* const* ctx, int n_bisect, int n_newton,
                             double* t_out) {
  for (long i = 0; i < n; ++i)
    t_out[i] = thermal13_cell(make_ctx(ctx, i), g_lp, g_co, n_bisect, n_newton);
}

extern "C" void hd_net64(long n, const double* const* ctx, double t, double* out) {
  for (long i = 0; i < n; ++i) out[i] = net_heating64(t, make_ctx(ctx, i), g_lp, g_co);
}

// rates: 7 pointers (n_h, k_pd_base, k_ci, alpha_cp, k_co_total,
// r_h2_half_nh, r_cr_base); y: n x 5 in-out (x_hi, x_h2, x_cp, x_c, x_co).
extern "C" void hd_chem_euler(long n, const double* const* r, double x_c_total, double* y,
                              const double* hcop, int n_substeps, double conv_tol) {
  for (long i = 0; i < n; ++i)
    chem_euler_cell(r[0][i], r[1][i], r[2][i], r[3][i], r[4][i], r[5][i], r[6][i], x_c_total,
                    y + 5 * i, hcop[i], n_substeps, conv_tol);
}
