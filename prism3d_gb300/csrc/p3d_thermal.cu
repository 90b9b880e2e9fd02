// p3d_thermal.cu -- per-cell thermal-balance root on sm_103a.
//
// Net heating Gamma - Lambda follows rust/src/thermal.rs:50-184 term by term
// (heating from the precomputed context + gas-grain exchange; cooling by
// [CII] 158, [OI] 63/145, [CI] 609/370, the CO rotational ladder with its
// early break, H2 ro-vibrational (Glover & Abel 2008), Lyman alpha, gas-grain
// and C+ recombination).  Two root drivers use it:
//   * thermal13_kernel: the reference's 10 geometric bisections + 3 clamped
//     finite-difference Newton steps (thermal.rs:189-270), the drop-in for
//     solve_thermal_vec;
//   * the steady-state drivers in p3d_steady.cu.
// heating_cooling_kernel evaluates the diagnostics Gamma and Lambda of the
// same terms at given temperatures.
#include "p3d_common.cuh"
#include "p3d_thermal.cuh"

namespace p3d {

__constant__ CoLevel c_co_levels[40];

__global__ void __launch_bounds__(kThreads)
thermal13_kernel(int64_t n, const double* __restrict__ gf, const double* __restrict__ gg,
                 const double* __restrict__ td, const double* __restrict__ ne,
                 const double* __restrict__ nhi, const double* __restrict__ nh2,
                 const double* __restrict__ nco, const double* __restrict__ ncp,
                 const double* __restrict__ no, const double* __restrict__ nc,
                 LineParams lp, int n_bisect, int n_newton, double* __restrict__ t_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    ThermalCtx c;
    c.gamma_fixed = gf[i]; c.gg_coeff = gg[i]; c.t_dust = td[i]; c.n_e = ne[i];
    c.n_hi = nhi[i]; c.n_h2 = nh2[i]; c.n_co = nco[i]; c.n_cp_nh = ncp[i];
    c.n_o_nh = no[i]; c.n_c_nh = nc[i];
    t_out[i] = thermal13_cell(c, lp, c_co_levels, n_bisect, n_newton);
  }
}

// Diagnostics Gamma and Lambda at t (solver_3d.py:898-1050), per cell.
__global__ void __launch_bounds__(kThreads)
heating_cooling_kernel(int64_t n, const double* __restrict__ gf, const double* __restrict__ gg,
                       const double* __restrict__ td, const double* __restrict__ ne,
                       const double* __restrict__ nhi, const double* __restrict__ nh2,
                       const double* __restrict__ nco, const double* __restrict__ ncp,
                       const double* __restrict__ no, const double* __restrict__ nc,
                       LineParams lp, const double* __restrict__ t, double* __restrict__ gamma,
                       double* __restrict__ lambda) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    ThermalCtx c;
    c.gamma_fixed = gf[i]; c.gg_coeff = gg[i]; c.t_dust = td[i]; c.n_e = ne[i];
    c.n_hi = nhi[i]; c.n_h2 = nh2[i]; c.n_co = nco[i]; c.n_cp_nh = ncp[i];
    c.n_o_nh = no[i]; c.n_c_nh = nc[i];
    double g, l;
    heating_cooling64(t[i], c, lp, c_co_levels, &g, &l);
    gamma[i] = g;
    lambda[i] = l;
  }
}

cudaError_t launch_heating_cooling(int64_t n, const double* const* ctx, const LineParams& lp,
                                   const double* t, double* gamma, double* lambda, int sms,
                                   cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  heating_cooling_kernel<<<grid_for(n, sms, 4), kThreads, 0, s>>>(
      n, ctx[0], ctx[1], ctx[2], ctx[3], ctx[4], ctx[5], ctx[6], ctx[7], ctx[8], ctx[9], lp, t,
      gamma, lambda);
  return cudaGetLastError();
}

cudaError_t upload_co_levels(const CoLevel* host40, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_co_levels, host40, sizeof(CoLevel) * 40, 0,
                                 cudaMemcpyHostToDevice, s);
}

cudaError_t launch_thermal13(int64_t n, const double* const* ctx, const LineParams& lp,
                             int n_bisect, int n_newton, double* t_out, int sms,
                             cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  thermal13_kernel<<<grid_for(n, sms, 4), kThreads, 0, s>>>(
      n, ctx[0], ctx[1], ctx[2], ctx[3], ctx[4], ctx[5], ctx[6], ctx[7], ctx[8], ctx[9], lp,
      n_bisect, n_newton, t_out);
  return cudaGetLastError();
}

}  // namespace p3d
