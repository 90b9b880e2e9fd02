// p3d_rt.cu -- multi-ray FUV transfer on sm_103a.
//
// The reference (prism3d/radiative_transfer/fuv_rt_3d.py:215-392) traces each
// of the 12*nside^2 Fibonacci-spiral rays as a prefix sum along the ray's
// dominant grid axis, with per-cell layers n_H ds, 2 n_H x_H2 ds, n_H x_CO ds
// (ds = cell / max(|d_dom|, 0.01)), a midpoint correction of half the cell's
// own layer, clamping at 0, A_V = N_H * 5.34e-22, and then
//   G0 = sum_r G0_ext,r exp(-1.8 A_V,r) w_r / 4pi,
//   (A_V, N_H, N_H2, N_CO) taken from the ray with the smallest A_V
//   (strict '<' in ray order: the earliest ray wins ties).
//
// GB300 mapping: rays sharing a dominant axis and direction form one of six
// families; a thread owns one pencil of the grid along that axis and walks
// it once per family, carrying one running N_H sum per ray of the family in
// registers (chunks of kRayChunk rays) plus the family's unscaled H2 and CO
// sums.  Consecutive threads own pencils that are adjacent in memory, so
// every step of the walk is a coalesced load for the x and y axes; for the z
// axis each thread's pencil is contiguous and the strided warp loads are
// served from L1 lines fetched by the first step.
//
// Bit-exactness: A_V decides the selected ray, so its N_H is summed exactly
// as numpy does it (layer = n * ds rounded, sequential cumsum in the ray's
// direction, minus 0.5 * layer) with explicit _rn intrinsics, which nvcc
// never contracts into FMAs.  N_H2 and N_CO use the family sums scaled by the
// ray's ds (equal to numpy up to summation rounding).
#include "p3d_common.cuh"
#include "p3d_rt.cuh"

namespace p3d {

__device__ __forceinline__ void pencil_geometry(int axis, int64_t p, int64_t nx, int64_t ny,
                                                int64_t nz, int64_t& base, int64_t& stride,
                                                int64_t& len) {
  if (axis == 0) {  // pencil (j, k) along i
    base = p;  // j*nz + k
    stride = ny * nz;
    len = nx;
  } else if (axis == 1) {  // pencil (i, k) along j
    int64_t i = p / nz, k = p - i * nz;
    base = i * ny * nz + k;
    stride = nz;
    len = ny;
  } else {  // pencil (i, j) along k
    base = p * nz;
    stride = 1;
    len = nz;
  }
}

// One family chunk over all pencils of `axis`.  rays[0..nr) are ray slots of
// the chunk in ascending ray order.
__global__ void __launch_bounds__(128)
rt_family_kernel(int axis, int fwd, int64_t nx, int64_t ny, int64_t nz, int64_t n_pencils,
                 const double* __restrict__ dens, const double* __restrict__ xh2,
                 const double* __restrict__ xco, RayChunk chunk,
                 double* __restrict__ g0_acc, double* __restrict__ av_acc,
                 double* __restrict__ nh_acc, double* __restrict__ nh2_acc,
                 double* __restrict__ nco_acc, int32_t* __restrict__ ray_acc) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n_pencils) return;
  int64_t base, stride, len;
  pencil_geometry(axis, p, nx, ny, nz, base, stride, len);
  double cs[kRayChunk];
#pragma unroll
  for (int r = 0; r < kRayChunk; ++r) cs[r] = 0.0;
  double s2 = 0.0, s3 = 0.0;
  for (int64_t t = 0; t < len; ++t) {
    int64_t step = fwd ? t : (len - 1 - t);
    int64_t c = base + step * stride;
    double n = dens[c];
    double l2 = xh2 ? __dmul_rn(__dmul_rn(n, xh2[c]), 2.0) : 0.0;
    double l3 = xco ? n * xco[c] : 0.0;
    s2 += l2;
    s3 += l3;
    double h2 = s2 - 0.5 * l2;
    double co = s3 - 0.5 * l3;
    double best_av = av_acc[c];
    int best_ray = ray_acc[c];
    double best_nh = 0.0, best_ds = 0.0;
    bool took = false;
    double g0_sum = 0.0;
#pragma unroll
    for (int r = 0; r < kRayChunk; ++r) {
      if (r < chunk.n) {
        double ds = chunk.ds[r];
        double layer = __dmul_rn(n, ds);
        cs[r] = __dadd_rn(cs[r], layer);
        double nh = fmax(__dsub_rn(cs[r], 0.5 * layer), 0.0);
        double av = __dmul_rn(nh, kAVperNH);
        if (chunk.g_ext[r] != 0.0) g0_sum += chunk.g_ext[r] * exp(-1.8 * av) * chunk.w[r];
        int id = chunk.id[r];
        if (av < best_av || (av == best_av && best_ray != kNoRay && id < best_ray)) {
          best_av = av;
          best_ray = id;
          best_nh = nh;
          best_ds = ds;
          took = true;
        }
      }
    }
    g0_acc[c] += g0_sum;
    if (took) {
      av_acc[c] = best_av;
      ray_acc[c] = best_ray;
      nh_acc[c] = best_nh;
      nh2_acc[c] = fmax(best_ds * h2, 0.0);
      nco_acc[c] = fmax(best_ds * co, 0.0);
    }
  }
}

__global__ void rt_init_kernel(int64_t n, double* g0, double* av, double* nh, double* nh2,
                               double* nco, int32_t* ray) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    g0[i] = 0.0;
    av[i] = 1e10;
    nh[i] = 0.0;
    nh2[i] = 0.0;
    nco[i] = 0.0;
    ray[i] = kNoRay;
  }
}

__global__ void rt_fix_unset_kernel(int64_t n, int32_t* ray) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (ray[i] == kNoRay) ray[i] = -1;
  }
}

cudaError_t launch_fuv_full(int64_t nx, int64_t ny, int64_t nz, const double* dens,
                            const double* xh2, const double* xco, const RaySet& rs,
                            double* g0, double* av, double* nh, double* nh2, double* nco,
                            int32_t* ray, int sms, cudaStream_t s) {
  int64_t n = nx * ny * nz;
  if (n <= 0) return cudaSuccess;
  rt_init_kernel<<<grid_for(n, sms, 8), kThreads, 0, s>>>(n, g0, av, nh, nh2, nco, ray);
  for (int fam = 0; fam < 6; ++fam) {
    int axis = fam >> 1, fwd = fam & 1;
    int64_t dims[3] = {nx, ny, nz};
    int64_t n_pencils = n / dims[axis];
    // rays of this family in ascending order, in chunks
    RayChunk ch;
    ch.n = 0;
    for (int r = 0; r <= rs.n; ++r) {
      bool flush = (r == rs.n) || ch.n == kRayChunk;
      if (flush && ch.n > 0) {
        rt_family_kernel<<<(unsigned)ceil_div(n_pencils, 128), 128, 0, s>>>(
            axis, fwd, nx, ny, nz, n_pencils, dens, xh2, xco, ch, g0, av, nh, nh2, nco, ray);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        ch.n = 0;
      }
      if (r == rs.n) break;
      if (rs.axis[r] == axis && rs.fwd[r] == fwd) {
        ch.id[ch.n] = r;
        ch.ds[ch.n] = rs.ds[r];
        ch.g_ext[ch.n] = rs.g_ext[r];
        ch.w[ch.n] = rs.w[r];
        ++ch.n;
      }
    }
  }
  rt_fix_unset_kernel<<<grid_for(n, sms, 8), kThreads, 0, s>>>(n, ray);
  return cudaGetLastError();
}

}  // namespace p3d
