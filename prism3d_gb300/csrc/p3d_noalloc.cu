// p3d_noalloc.cu -- photoelectric heating without any device allocation.
//
// p3d_pe_heating_vec_dev stages the grain-bin vectors and the two condensed
// PE tables in the library's device workspace, which it grows with
// cudaMalloc on first use.  Some callers cannot let a library allocate: a
// host application that reserves the GPU's memory for its own pool at start
// and hands each library a fixed budget (a later cudaMalloc would fail or
// push the application out of memory), an embedder whose allocator owns
// every device byte and tracks it, and latency-critical callers for which
// the device-wide synchronisation a cudaMalloc / cudaFree can imply stalls
// their other streams.  p3d_pe_heating_vec_noalloc serves them: every
// argument is a device pointer (nothing is copied from the host), and its
// scratch, the two condensed tables, lives in a fixed file-scope device
// array, reserved when the library is loaded and kept by every device that
// loads it until the process exits.
#include <mutex>

#include "../../include/prism3d_gb300.h"
#include "p3d_capi_internal.cuh"
#include "p3d_common.cuh"
#include "p3d_pe.cuh"

namespace p3d {

// Scratch layout (doubles): condensed tables A_nano, A_rest (2 x kNoAllocMaxGrid).
constexpr int kNoAllocMaxGrid = 8192;  // n_psi * n_eg (the THEMIS grid is 200 x 20)
constexpr int kNoAllocDoubles = 2 * kNoAllocMaxGrid;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_na_mu;
double* g_na_ptr[kMaxDevices] = {};  // device address of the scratch, per device
int g_na_sms[kMaxDevices] = {};

// Once per device, with that device current: the host-side symbol is only a
// stand-in, the kernel needs the device address.
int noalloc_setup(double** ptr, int* sms) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(P3D_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) return set_error(P3D_ENODEV, "device index %d", dev);
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    int major = 0, minor = 0, n_sm = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (major != 10 || minor != 3)
      return set_error(P3D_ENODEV, "device %d is sm_%d%d; this library is built for sm_103a",
                       dev, major, minor);
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return set_error(P3D_ECUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    }
    g_na_ptr[dev] = (double*)p;
    g_na_sms[dev] = n_sm > 0 ? n_sm : 1;
  }
  *ptr = g_na_ptr[dev];
  *sms = g_na_sms[dev];
  return P3D_OK;
}
}  // namespace

}  // namespace p3d

using namespace p3d;

extern "C" int p3d_pe_heating_vec_noalloc(
    const double* pe_table, int64_t n_bins, double log_psi_min, double log_psi_step,
    int64_t n_psi, double eg_min, double eg_step, int64_t n_eg, const double* bin_sigma_abs,
    const double* bin_dn_da_da, const double* bin_is_nano, int64_t n_cells, const double* g0,
    const double* t_gas, const double* x_e, const double* n_h, const double* f_nano,
    const double* e_g, double* gamma_pe_out, void* stream) {
  if (n_cells < 0 || n_bins < 0) return set_error(P3D_EINVAL, "negative size");
  if (n_psi < 2 || n_eg < 2) return set_error(P3D_EINVAL, "table grid must be at least 2 x 2");
  if (n_psi * n_eg > kNoAllocMaxGrid)
    return set_error(P3D_EINVAL,
                     "n_psi * n_eg = %lld exceeds the no-allocation limit of %d grid points",
                     (long long)(n_psi * n_eg), kNoAllocMaxGrid);
  if (!(log_psi_step != 0.0) || !(eg_step != 0.0)) return set_error(P3D_EINVAL, "zero grid step");
  double* scratch = nullptr;
  int sms = 1;
  int rc = noalloc_setup(&scratch, &sms);
  if (rc) return rc;
  if (n_cells == 0) return P3D_OK;
  if (!pe_table || !bin_sigma_abs || !bin_dn_da_da || !bin_is_nano || !g0 || !t_gas || !x_e ||
      !n_h || !f_nano || !e_g || !gamma_pe_out)
    return set_error(P3D_EINVAL, "null array");
  cudaStream_t s = (cudaStream_t)stream;
  double* a_nano = scratch;
  double* a_rest = scratch + kNoAllocMaxGrid;
  // The condense kernel rewrites every table entry the cell kernel reads
  // (n_psi * n_eg of each), so the previous call's contents never leak and
  // nothing needs clearing; calls that overlap on the GPU share this
  // scratch and race.
  PeGrid g{log_psi_min, log_psi_step, eg_min, eg_step, (int)n_psi, (int)n_eg};
  cudaError_t e = launch_pe_condense(pe_table, (int)n_bins, g, bin_sigma_abs, bin_dn_da_da,
                                     bin_is_nano, a_nano, a_rest, s);
  if (e != cudaSuccess) return cuda_fail(e, "noalloc condense launch");
  const double* cells[6] = {g0, t_gas, x_e, n_h, f_nano, e_g};
  e = launch_pe_cells(n_cells, g, a_nano, a_rest, cells, gamma_pe_out, sms, s);
  if (e != cudaSuccess) return cuda_fail(e, "noalloc pe launch");
  return P3D_OK;
}
