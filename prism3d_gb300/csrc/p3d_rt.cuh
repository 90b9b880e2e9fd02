// p3d_rt.cuh -- FUV ray set and launch declarations.
#pragma once

#include "p3d_common.cuh"

namespace p3d {

constexpr int kRayChunk = 12;
constexpr int kMaxRays = 768;  // nside <= 8
constexpr int32_t kNoRay = 0x7fffffff;

// Host-side description of the ray set (fuv_rt_3d.py:272-281, :324-340).
struct RaySet {
  int n;
  int axis[kMaxRays];   // dominant axis (np.argmax(|d|): first maximum)
  int fwd[kMaxRays];    // 1: cumsum in ascending index order (d[dom] < 0)
  double ds[kMaxRays];  // cell_size * (1 / max(|d_dom|, 0.01))
  double g_ext[kMaxRays];
  double w[kMaxRays];   // weight / (4 pi)
};

// Up to kRayChunk rays of one family, passed by value to the kernel.
struct RayChunk {
  int n;
  int id[kRayChunk];
  double ds[kRayChunk];
  double g_ext[kRayChunk];
  double w[kRayChunk];
};

// Device workspace launch_fuv_full needs for n cells (per-family partial
// results: 36 bytes per cell and family).
size_t rt_work_bytes(int64_t n);
// Kernel launches of one launch_fuv_full call for this ray set.
int rt_launch_count(const RaySet& rs);

cudaError_t launch_fuv_full(int64_t nx, int64_t ny, int64_t nz, const double* dens,
                            const double* xh2, const double* xco, const RaySet& rs,
                            void* work, double* g0, double* av, double* nh, double* nh2,
                            double* nco, int32_t* ray, int sms, cudaStream_t s);

}  // namespace p3d
