// p3d_pe.cuh -- device PE heating cell function (rust/src/pe_table.rs:22-141).
#pragma once

#include "p3d_common.cuh"

namespace p3d {

struct PeGrid {
  double log_psi_min, log_psi_step, eg_min, eg_step;
  int n_psi, n_eg;
};

// rust/src/pe_table.rs:22-28: floor index clamped to [0, n-2], weight
// clamped to [0, 1].  NaN maps to index 0 like Rust's saturating cast.
__device__ __forceinline__ void interp_idx_weight(double x, double gmin, double gstep, int n,
                                                  int& idx, double& w) {
  double tf = floor((x - gmin) / gstep);
  idx = (tf >= (double)(n - 2)) ? n - 2 : (tf > 0.0 ? (int)tf : 0);
  w = fmin(fmax((x - (gmin + (double)idx * gstep)) / gstep, 0.0), 1.0);
}

__device__ __forceinline__ double bilinear(const double* __restrict__ a, int n_eg, int pi,
                                           int ei, double pw, double ew) {
  const double* r0 = a + (int64_t)pi * n_eg + ei;
  const double* r1 = r0 + n_eg;
  double v00 = __ldg(r0), v01 = __ldg(r0 + 1), v10 = __ldg(r1), v11 = __ldg(r1 + 1);
  return v00 * (1.0 - pw) * (1.0 - ew) + v10 * pw * (1.0 - ew) + v01 * (1.0 - pw) * ew +
         v11 * pw * ew;
}

__device__ __forceinline__ double pe_cell(const PeGrid& g, const double* __restrict__ a_nano,
                                          const double* __restrict__ a_rest, double g0,
                                          double tg, double xe, double nh, double fn,
                                          double eg) {
  double n_e = fmax(xe * nh, 1e-10 * nh);
  double psi = g0 * sqrt(tg) / n_e;
  double log_psi = log10(fmax(psi, 0.1));
  double phi_uv = kFHabing * g0 / kEFUVMean;
  int pi, ei;
  double pw, ew;
  interp_idx_weight(log_psi, g.log_psi_min, g.log_psi_step, g.n_psi, pi, pw);
  interp_idx_weight(eg, g.eg_min, g.eg_step, g.n_eg, ei, ew);
  double yn = bilinear(a_nano, g.n_eg, pi, ei, pw, ew);
  double yr = bilinear(a_rest, g.n_eg, pi, ei, pw, ew);
  return nh * phi_uv * (fn * yn + yr);
}

cudaError_t launch_pe_condense(const double* table, int n_bins, const PeGrid& g,
                               const double* sigma, const double* dnda, const double* is_nano,
                               double* a_nano, double* a_rest, cudaStream_t s);
cudaError_t launch_pe_cells(int64_t n, const PeGrid& g, const double* a_nano,
                            const double* a_rest, const double* const* cells6, double* out,
                            int sms, cudaStream_t s);

}  // namespace p3d
