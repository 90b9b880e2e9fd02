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

cudaError_t launch_fuv_full(int64_t nx, int64_t ny, int64_t nz, const double* dens,
                            const double* xh2, const double* xco, const RaySet& rs,
                            double* g0, double* av, double* nh, double* nh2, double* nco,
                            int32_t* ray, int sms, cudaStream_t s);

}  // namespace p3d
