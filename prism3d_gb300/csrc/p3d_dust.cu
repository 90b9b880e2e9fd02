// p3d_dust.cu -- one THEMIS grain-state step per cell (the reference's
// _evolve_dust_state, prism3d/solver_3d.py:465-507): photo-destruction,
// replenishment and accretion of the nano-grain fraction f_nano, relaxation
// of the band gap E_g towards its equilibrium, over dt = 10 kyr.
#include <cmath>

#include "../../include/prism3d_gb300.h"
#include "p3d_capi_internal.cuh"
#include "p3d_common.cuh"

namespace p3d {

__global__ void dust_evolve_kernel(int64_t n, const double* __restrict__ g0,
                                   const double* __restrict__ nh, double* __restrict__ f_nano,
                                   double* __restrict__ e_g) {
  const double dt = 1e4 * 3.15e7;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double G = g0[i], d = nh[i], fn = f_nano[i], eg = e_g[i];
    const double tau_dest = 1e4 * 3.15e7 / fmax(G / 1e4, 0.01);
    const double f_dest = exp(-dt / tau_dest);
    const double f_rep = fmin(dt / (1e6 * 3.15e7), 0.1);
    const double f_acc = (G < 1.0 && d > 1e4) ? fmin(dt / (1e5 * 3.15e7 * 1e4 / d), 0.1) : 0.0;
    const double f = __dadd_rn(__dadd_rn(__dmul_rn(fn, f_dest), __dmul_rn(1.0 - fn, f_rep)), f_acc);
    f_nano[i] = fmin(fmax(f, 0.01), 2.0);
    const double tau_ar = 1e3 * 3.15e7 / fmax(G, 0.01);
    const double eq = G > 10.0 ? 0.01 : fmin(0.1 + 0.5 * log10(fmax(d, 1.0)), 2.5);
    const double e = __dadd_rn(eg, __dmul_rn(eq - eg, fmin(dt / tau_ar, 1.0)));
    e_g[i] = fmin(fmax(e, 0.01), 2.5);
  }
}

cudaError_t launch_dust_evolve(int64_t n, const double* g0, const double* nh, double* f_nano,
                               double* e_g, int sms, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  dust_evolve_kernel<<<grid_for(n, sms, 8), kThreads, 0, s>>>(n, g0, nh, f_nano, e_g);
  return cudaGetLastError();
}

}  // namespace p3d

using namespace p3d;

extern "C" {

int p3d_evolve_dust_state_dev(int64_t n, const double* g0, const double* n_h, double* f_nano,
                              double* e_g, void* stream) {
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if (n < 0) return set_error(P3D_EINVAL, "n < 0");
  if (n == 0) return P3D_OK;
  if (!g0 || !n_h || !f_nano || !e_g) return set_error(P3D_EINVAL, "null array");
  dust_evolve_kernel<<<grid_for(n, st->sms, 8), kThreads, 0, (cudaStream_t)stream>>>(
      n, g0, n_h, f_nano, e_g);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "dust evolution launch");
}

int p3d_evolve_dust_state(int64_t n, const double* g0, const double* n_h, double* f_nano,
                          double* e_g) {
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if (n < 0) return set_error(P3D_EINVAL, "n < 0");
  if (n == 0) return P3D_OK;
  if (!g0 || !n_h || !f_nano || !e_g) return set_error(P3D_EINVAL, "null array");
  const size_t b = sizeof(double) * (size_t)n;
  double* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, 4 * b);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(P3D_ENOMEM, "dust evolution staging");
  }
  const double* in[4] = {g0, n_h, f_nano, e_g};
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(buf + k * (size_t)n, in[k], b, cudaMemcpyHostToDevice, st->stream);
  if (e == cudaSuccess)
    rc = p3d_evolve_dust_state_dev(n, buf, buf + n, buf + 2 * n, buf + 3 * n, st->stream);
  else
    rc = cuda_fail(e, "dust evolution H2D");
  if (!rc) {
    e = cudaMemcpyAsync(f_nano, buf + 2 * n, b, cudaMemcpyDeviceToHost, st->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(e_g, buf + 3 * n, b, cudaMemcpyDeviceToHost, st->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "dust evolution D2H");
  }
  if (!rc) rc = sync_check(st->stream, "dust evolution");
  cudaStreamSynchronize(st->stream);
  cudaFree(buf);
  return rc;
}

}  // extern "C"
