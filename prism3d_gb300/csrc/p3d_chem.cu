// p3d_chem.cu -- reduced gas-phase chemistry, explicit-Euler drop-in.
//
// One thread per cell runs the reference's rate-limited explicit Euler
// substeps (rust/src/chemistry.rs:13-98): 5 species (H, H2, C+, C, CO), x_e
// and x_OH derived, adaptive dt growing x3 per substep up to 1e16 s and
// limited to 0.1 / max relative rate, H and C renormalised after every
// substep, per-cell early exit checked every 20 substeps.
#include "p3d_common.cuh"
#include "p3d_chem.cuh"

namespace p3d {

__global__ void __launch_bounds__(kThreads)
chem_euler_kernel(int64_t n, const double* __restrict__ n_h, const double* __restrict__ kpd,
                  const double* __restrict__ kci, const double* __restrict__ acp,
                  const double* __restrict__ kco, const double* __restrict__ rh2,
                  const double* __restrict__ rcr, double x_c_total, double* __restrict__ x_hi,
                  double* __restrict__ x_h2, double* __restrict__ x_cp,
                  double* __restrict__ x_c, double* __restrict__ x_co,
                  double* __restrict__ x_o, double* __restrict__ x_e,
                  const double* __restrict__ x_hcop, int n_substeps, double conv_tol) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double y[5] = {x_hi[i], x_h2[i], x_cp[i], x_c[i], x_co[i]};
    const double hcop = x_hcop[i];
    chem_euler_cell(n_h[i], kpd[i], kci[i], acp[i], kco[i], rh2[i], rcr[i], x_c_total, y,
                    hcop, n_substeps, conv_tol);
    x_hi[i] = y[0]; x_h2[i] = y[1]; x_cp[i] = y[2]; x_c[i] = y[3]; x_co[i] = y[4];
    x_o[i] = fmax(kXOTotal - y[4], 1e-30);
    x_e[i] = fmax(y[2] + hcop, 1e-30);
  }
}

cudaError_t launch_chem_euler(int64_t n, const double* const* rates, double x_c_total,
                              double* const* state7, const double* x_hcop, int n_substeps,
                              double conv_tol, int sms, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  chem_euler_kernel<<<grid_for(n, sms, 4), kThreads, 0, s>>>(
      n, rates[0], rates[1], rates[2], rates[3], rates[4], rates[5], rates[6], x_c_total,
      state7[0], state7[1], state7[2], state7[3], state7[4], state7[5], state7[6], x_hcop,
      n_substeps, conv_tol);
  return cudaGetLastError();
}

}  // namespace p3d
