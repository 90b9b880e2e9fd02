// p3d_capi_internal.cuh -- per-device library state shared by the C-ABI files.
#pragma once

#include <cstdarg>

#include "p3d_common.cuh"
#include "p3d_rt.cuh"

namespace p3d {

// Workspace slots: 0..15 per-call arrays, then named slots.
enum : int {
  kSlotBins = 16,
  kSlotPeCond = 17,
  kSlotPeTable = 18,
  kSlotRay = 19,
  kSlotRtWork = 20,
  kSlots = 24,
};

// One per CUDA device, created on first use with that device current.
struct DeviceState {
  int device = -1;
  int sms = 0;
  cudaStream_t stream = nullptr;
  void* buf[kSlots] = {};
  size_t cap[kSlots] = {};
  RaySet rayset;
  // grow-only device buffer for slot k (never shrinks; freed at exit)
  void* slot(int k, size_t bytes, int* err);
};

int set_error(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* where);
int get_state(DeviceState** out);
int sync_check(cudaStream_t s, const char* where);
void co_ladder_host(CoLevel* out);
// One THEMIS grain step (f_nano, E_g in place) per cell, p3d_dust.cu.
cudaError_t launch_dust_evolve(int64_t n, const double* g0, const double* nh, double* f_nano,
                               double* e_g, int sms, cudaStream_t s);
// FUV field of a point source (p3d_point_source.cu); cols_only = 1 writes
// N_H2 / N_CO only.
cudaError_t launch_point_source(int64_t nx, int64_t ny, int64_t nz, const double* dens,
                                const double* xh2, const double* xco, const double* star_pos,
                                double lum, double cell, int cols_only, double* g0, double* av,
                                double* nh, double* nh2, double* nco, int sms, cudaStream_t s);
int build_rayset(const double* dirs, const double* weights, int64_t n_rays,
                 const double* g0_ext, int64_t n_g0, double cell_size, RaySet* rs);

}  // namespace p3d
