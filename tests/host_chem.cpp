// Host build of the steady driver's per-cell chemistry (prism3d_gb300/csrc/
// p3d_newton.cuh: pseudo-transient Newton on the 5x5 reduced network, FP64
// or FP32 factorisation with FP64 residuals) for the CPU tests: the same
// source compiled by g++, checked against the oracle's FP64 restatement on
// the inputs of the oracle's outer iterations.  Only the CUDA qualifiers are
// mapped to host forms.
#include <cuda_runtime.h>

#include <cmath>

#undef __device__
#define __device__
#undef __forceinline__
#define __forceinline__ inline
#include "../prism3d_gb300/csrc/p3d_newton.cuh"

using namespace p3d;

// Per-cell inputs as the steady driver's chemistry kernel assembles them
// (rates of solver_3d.py:549-557, shielding columns of the selected ray at
// the start of the iteration); y: n x 5 (x_HI, x_H2, x_C+, x_C, x_CO),
// floored at 1e-30 and solved in place.
extern "C" void hc_chem_steady(long n, const double* n_h, const double* kpd0,
                               const double* kci, const double* acp, const double* kco0,
                               const double* rh2_half_nh, const double* rcr, double x_c_total,
                               double x_hcop, const double* kco_cr, const double* u_h2,
                               const double* u_co, double b_dop, int mixed, int max_iter,
                               double rtol, double* y, double* fh2, int* iters, int* status) {
  for (long i = 0; i < n; ++i) {
    ChemCell cc;
    cc.n_h = n_h[i];
    cc.kci = kci[i];
    cc.acp = acp[i];
    cc.rh2 = rh2_half_nh[i];
    cc.rcr = rcr[i];
    cc.xc = x_c_total;
    cc.hcop = x_hcop;
    cc.kpd0 = kpd0[i];
    cc.kco0 = kco0[i];
    cc.kco_cr = kco_cr[i];
    cc.u_h2 = u_h2[i];
    cc.u_co = u_co[i];
    cc.ds = 0.0;
    cc.b_dop = b_dop;
    // the mixed kernel prepares the shielding in its own forms (FAST)
    if (mixed)
      chem_prepare<true>(cc);
    else
      chem_prepare<false>(cc);
    double* yi = y + 5 * i;
    for (int c = 0; c < 5; ++c) yi[c] = fmax(yi[c], 1e-30);
    int it = 0;
    status[i] = mixed ? chem_steady_cell<true>(cc, yi, max_iter, rtol, 4.0, fh2 + i, &it)
                      : chem_steady_cell<false>(cc, yi, max_iter, rtol, 4.0, fh2 + i, &it);
    iters[i] = it;
  }
}

// Residual f (5) and analytic Jacobian J (5 x 5, row-major) of the reduced
// chemistry at one state (chem5_eval, the rows the adjoint's per-cell
// Jacobian takes), with the shielding fixed by the columns (ds = 0, as in the
// adjoint) or with the cell's own H2 half layer inside (ds > 0).
extern "C" void hc_chem5_eval(double n_h, double kpd0, double kci, double acp, double kco0,
                              double rh2_half_nh, double rcr, double x_c_total, double x_hcop,
                              double kco_cr, double koh_s, double u_h2, double u_co,
                              double ds, double b_dop, const double* y, double* f, double* J) {
  ChemCell cc;
  cc.n_h = n_h;
  cc.kci = kci;
  cc.acp = acp;
  cc.rh2 = rh2_half_nh;
  cc.rcr = rcr;
  cc.xc = x_c_total;
  cc.hcop = x_hcop;
  cc.kpd0 = kpd0;
  cc.kco0 = kco0;
  cc.kco_cr = kco_cr;
  cc.koh_s = koh_s;
  cc.u_h2 = u_h2;
  cc.u_co = u_co;
  cc.ds = ds;
  cc.b_dop = b_dop;
  chem_prepare(cc);
  double Jm[5][5], sc[5], fh2;
  chem5_eval(cc, y, f, Jm, sc, &fh2);
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) J[5 * r + c] = Jm[r][c];
}

// H2 self-shielding factor and the slope the steady driver's worklist keeps
// (|d ln f_H2 / d ln b|), for the CPU tests.
extern "C" void hc_fsh_h2(long n, const double* nh2, const double* b, double* f,
                          double* dlnb) {
  for (long i = 0; i < n; ++i) {
    double dfdn;
    f[i] = fsh_h2(nh2[i], b[i], &dfdn);
    dlnb[i] = fsh_h2_dlnb(nh2[i], b[i], f[i]);
  }
}
