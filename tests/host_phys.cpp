// Host build of the steady driver's per-cell physics (prism3d_gb300/csrc/
// p3d_phys.cuh: H2 and CO self-shielding, cosmic-ray attenuation, dust
// temperature, H2 formation; p3d_pe.cuh: PE heating on the condensed
// tables) for the CPU tests, checked against the reference's own values.
// Only the CUDA qualifiers and __ldg are mapped to host forms.
#include <cuda_runtime.h>

#include <cmath>

#undef __device__
#define __device__
#undef __forceinline__
#define __forceinline__ inline
#define __ldg(p) (*(p))
#include "../prism3d_gb300/csrc/p3d_pe.cuh"
#include "../prism3d_gb300/csrc/p3d_phys.cuh"

using namespace p3d;

// fast != 0: the mixed path's forms (template argument FAST)
extern "C" void hp_fsh_h2(long n, const double* nh2, double b, double* out, double* dfdn,
                          int fast) {
  for (long i = 0; i < n; ++i)
    out[i] = fast ? fsh_h2<true>(nh2[i], b, dfdn + i) : fsh_h2<false>(nh2[i], b, dfdn + i);
}

extern "C" void hp_fsh_co(long n, const double* nco, const double* nh2, double* out,
                          double* d_h2, int fast) {
  for (long i = 0; i < n; ++i)
    out[i] = fast ? fsh_co<true>(nco[i], nh2[i], d_h2 + i) : fsh_co<false>(nco[i], nh2[i], d_h2 + i);
}

extern "C" void hp_cr_rate(long n, const double* nh, double zeta0, double* out) {
  for (long i = 0; i < n; ++i) out[i] = cr_rate(nh[i], zeta0);
}

extern "C" void hp_tdust(long n, const double* g0, const double* av, const double* nh,
                         const double* tg, double* out) {
  for (long i = 0; i < n; ++i) out[i] = tdust(tdust_rad(g0[i], av[i]), nh[i], tg[i]);
}

extern "C" void hp_h2_form(long n, const double* tg, const double* td, const double* fnano,
                           double s_nano, double s_lc, double s_sil, double* out, int fast) {
  for (long i = 0; i < n; ++i)
    out[i] = fast ? h2_form<true>(tg[i], td[i], fnano[i], s_nano, s_lc, s_sil)
                  : h2_form<false>(tg[i], td[i], fnano[i], s_nano, s_lc, s_sil);
}

// PE heating per cell from the condensed tables a_nano, a_rest (n_psi x
// n_eg, the per-bin sums pe_condense_kernel forms).
extern "C" void hp_pe(long n, double log_psi_min, double log_psi_step, int n_psi, double eg_min,
                      double eg_step, int n_eg, const double* a_nano, const double* a_rest,
                      const double* g0, const double* tg, const double* xe, const double* nh,
                      const double* fn, const double* eg, double* out) {
  PeGrid g{log_psi_min, log_psi_step, eg_min, eg_step, n_psi, n_eg};
  for (long i = 0; i < n; ++i)
    out[i] = pe_cell(g, a_nano, a_rest, g0[i], tg[i], xe[i], nh[i], fn[i], eg[i]);
}

extern "C" void hp_interp_idx_weight(double x, double gmin, double gstep, int n, int* idx,
                                     double* w) {
  interp_idx_weight(x, gmin, gstep, n, *idx, *w);
}
