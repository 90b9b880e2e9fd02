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
int build_rayset(const double* dirs, const double* weights, int64_t n_rays,
                 const double* g0_ext, int64_t n_g0, double cell_size, RaySet* rs);

}  // namespace p3d
