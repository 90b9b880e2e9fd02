// p3d_pe.cu -- THEMIS photoelectric heating (rust/src/pe_table.rs:43-141).
//
// The reference sums, per cell, a bilinear interpolation of 32 per-bin tables
// PE_b(log psi, E_g) weighted by n_gr,b * sigma_b (and by f_nano for the nano
// bins).  Interpolation is linear in the table values, so the per-bin sum can
// be taken over the table first:
//   Gamma = n_H phi_UV [ f_nano * interp(A_nano) + interp(A_rest) ],
//   A_nano = sum_{nano b} n_gr,b sigma_b PE_b,  A_rest = sum_{other b} ...
// This turns 128 gathered table reads per cell into 8, and the two condensed
// tables (2 x n_psi x n_eg doubles, 64 KB for the THEMIS grid) stay in L1.
// The result equals the reference's up to summation order (a few ulp).
#include "p3d_common.cuh"
#include "p3d_pe.cuh"

namespace p3d {

__global__ void pe_condense_kernel(const double* __restrict__ table, int n_bins, int n_pe,
                                   const double* __restrict__ sigma,
                                   const double* __restrict__ dnda,
                                   const double* __restrict__ is_nano,
                                   double* __restrict__ a_nano, double* __restrict__ a_rest) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_pe) return;
  double sn = 0.0, sr = 0.0;
  for (int b = 0; b < n_bins; ++b) {
    double w = dnda[b] * sigma[b];
    double v = w * table[(int64_t)b * n_pe + idx];
    if (is_nano[b] > 0.5) sn += v; else sr += v;
  }
  a_nano[idx] = sn;
  a_rest[idx] = sr;
}

__global__ void __launch_bounds__(kThreads)
pe_cell_kernel(int64_t n, PeGrid grid, const double* __restrict__ a_nano,
               const double* __restrict__ a_rest, const double* __restrict__ g0,
               const double* __restrict__ tg, const double* __restrict__ xe,
               const double* __restrict__ nh, const double* __restrict__ fn,
               const double* __restrict__ eg, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    out[i] = pe_cell(grid, a_nano, a_rest, g0[i], tg[i], xe[i], nh[i], fn[i], eg[i]);
  }
}

cudaError_t launch_pe_condense(const double* table, int n_bins, const PeGrid& g,
                               const double* sigma, const double* dnda, const double* is_nano,
                               double* a_nano, double* a_rest, cudaStream_t s) {
  int n_pe = g.n_psi * g.n_eg;
  pe_condense_kernel<<<(unsigned)ceil_div(n_pe, 256), 256, 0, s>>>(
      table, n_bins, n_pe, sigma, dnda, is_nano, a_nano, a_rest);
  return cudaGetLastError();
}

cudaError_t launch_pe_cells(int64_t n, const PeGrid& g, const double* a_nano,
                            const double* a_rest, const double* const* cells6, double* out,
                            int sms, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  pe_cell_kernel<<<grid_for(n, sms, 8), kThreads, 0, s>>>(
      n, g, a_nano, a_rest, cells6[0], cells6[1], cells6[2], cells6[3], cells6[4], cells6[5],
      out);
  return cudaGetLastError();
}

}  // namespace p3d
