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
// GB300 mapping.  Rays sharing a dominant axis and direction form one of six
// families.  One launch walks every family: a thread owns one (family,
// pencil), walks the pencil once in the family's direction and carries in
// registers a running N_H per ray of the family (chunks of kRayChunk rays)
// plus the family's unscaled H2 and CO sums.  Two facts cut the FP64 work,
// which bounds this kernel on GB300 (FP64 runs at 1/64 of the FP32 rate):
//  * only rays with an external field contribute to G0, so a ray with
//    G0_ext = 0 matters only if it can be its family's smallest A_V; within
//    a family every layer is n ds_r, so the ray with the smallest ds has the
//    smallest A_V at every cell (rays whose ds lies within 1e-9 of the
//    smallest are all kept as candidates and compared exactly, so rounding
//    cannot move the minimum), and the other unlit rays are not marched;
//  * the per-cell clamp at 0 never fires (the running sum already includes
//    the cell's whole layer) and the argmin compares non-negative doubles.
// Each family writes its partial result per cell (G0 share, its candidate's
// N_H and ray, the N_H2 / N_CO of that ray) to its own slice of a workspace,
// so the six families never write the same word; a second kernel merges
// the six slices per cell in the reference's tie order and writes each
// output once.  Consecutive threads own pencils that are adjacent in memory,
// so the x and y walks load coalesced rows; a z pencil is contiguous and its
// walk is served from the L1 lines of the first loads.
//
// Bit-exactness: A_V decides the selected ray, so N_H is summed exactly as
// numpy does it (layer = n * ds rounded, sequential cumsum in the ray's
// direction, minus 0.5 * layer) with explicit _rn intrinsics, which nvcc
// never contracts into FMAs.  N_H2 and N_CO use the family sums scaled by
// the ray's ds (equal to numpy up to summation rounding); G0 uses the
// table-driven exp64 (<= 1 ulp) and sums in family order (1e-15 of numpy's).
#include "p3d_common.cuh"
#include "p3d_fastexp.cuh"
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

// Per-family partial results, one slice of n cells per family.
struct RtPartial {
  double* g0;    // 6 n: the family's share of G0
  double* nh;    // 6 n: N_H of the family's best candidate ray
  double* nh2;   // 6 n: N_H2 of that ray
  double* nco;   // 6 n: N_CO of that ray
  int32_t* id;   // 6 n: that ray (kNoRay: none below A_V = 1e10; -1: no ray marched)
};

constexpr uint8_t kRtLit = 1, kRtCand = 2;

// One chunk (<= kRayChunk rays) of every family's marched rays.
struct RtLaunch {
  int n[6];
  int id[6][kRayChunk];
  double ds[6][kRayChunk];
  double gw[6][kRayChunk];  // G0_ext w / 4 pi
  uint8_t flags[6][kRayChunk];
  int64_t start[7];  // first thread of each family (pencils are per family)
};

__global__ void __launch_bounds__(128)
rt_walk_kernel(int64_t nx, int64_t ny, int64_t nz, const double* __restrict__ dens,
               const double* __restrict__ xh2, const double* __restrict__ xco, RtLaunch L,
               RtPartial P, int first) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= L.start[6]) return;
  int f = 0;
  while (f < 5 && q >= L.start[f + 1]) ++f;
  const int nr = L.n[f];
  if (nr == 0) return;
  const int axis = f >> 1, fwd = f & 1;
  const int64_t p = q - L.start[f];
  int64_t base, stride, len;
  pencil_geometry(axis, p, nx, ny, nz, base, stride, len);
  const int64_t n = nx * ny * nz;
  const int64_t off = (int64_t)f * n;
  double cs[kRayChunk];
#pragma unroll
  for (int r = 0; r < kRayChunk; ++r) cs[r] = 0.0;
  double s2 = 0.0, s3 = 0.0;
  int64_t c = base + (fwd ? 0 : (len - 1)) * stride;
  const int64_t step = fwd ? stride : -stride;
  double n_next = len > 0 ? dens[c] : 0.0;
  for (int64_t t = 0; t < len; ++t, c += step) {
    const double nv = n_next;
    if (t + 1 < len) n_next = dens[c + step];  // load one cell ahead
    double h2 = 0.0, co = 0.0;
    if (first) {
      const double l2 = xh2 ? __dmul_rn(__dmul_rn(nv, xh2[c]), 2.0) : 0.0;
      const double l3 = xco ? __dmul_rn(nv, xco[c]) : 0.0;
      s2 += l2;
      s3 += l3;
      h2 = s2 - 0.5 * l2;
      co = s3 - 0.5 * l3;
    }
    double g0 = 0.0, best_nh = 0.0, best_ds = 0.0;
    double best_av = 1e10;
    int best_id = kNoRay;
#pragma unroll
    for (int r = 0; r < kRayChunk; ++r) {
      if (r < nr) {
        const double dsr = L.ds[f][r];
        const uint8_t fl = L.flags[f][r];
        const double layer = __dmul_rn(nv, dsr);
        cs[r] = __dadd_rn(cs[r], layer);
        const double nh = __dsub_rn(cs[r], 0.5 * layer);
        const double av = __dmul_rn(nh, kAVperNH);
        if (fl & kRtLit) g0 = fma(L.gw[f][r], exp64(-1.8 * av), g0);
        if (fl & kRtCand) {
          const int id = L.id[f][r];
          if (av < best_av || (av == best_av && id < best_id)) {
            best_av = av;
            best_id = id;
            best_nh = nh;
            best_ds = dsr;
          }
        }
      }
    }
    const int64_t o = off + c;
    if (first) {
      P.g0[o] = g0;
      P.id[o] = best_id;
      P.nh[o] = best_nh;
      P.nh2[o] = best_ds * h2;
      P.nco[o] = best_ds * co;
    } else {
      // later chunks hold lit rays only (every candidate is in the first)
      P.g0[o] += g0;
    }
  }
}

// Per cell: G0 = sum of the family shares, the smallest (A_V, ray) over the
// families' candidates, and that ray's columns.
__global__ void __launch_bounds__(kThreads)
rt_merge_kernel(int64_t n, RtPartial P, double* __restrict__ g0_out,
                double* __restrict__ av_out, double* __restrict__ nh_out,
                double* __restrict__ nh2_out, double* __restrict__ nco_out,
                int32_t* __restrict__ ray_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double g0 = 0.0, best_av = 1e10, nh = 0.0, nh2 = 0.0, nco = 0.0;
    int best = kNoRay;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const int64_t o = (int64_t)f * n + i;
      g0 += P.g0[o];
      const int id = P.id[o];
      if ((unsigned)id < (unsigned)kNoRay) {  // a candidate below A_V = 1e10
        const double nhf = P.nh[o];
        const double av = __dmul_rn(nhf, kAVperNH);
        if (av < best_av || (av == best_av && id < best)) {
          best_av = av;
          best = id;
          nh = nhf;
          nh2 = P.nh2[o];
          nco = P.nco[o];
        }
      }
    }
    g0_out[i] = g0;
    av_out[i] = best_av;
    nh_out[i] = nh;
    nh2_out[i] = nh2;
    nco_out[i] = nco;
    ray_out[i] = best == kNoRay ? -1 : best;
  }
}

size_t rt_work_bytes(int64_t n) { return (size_t)n * 6 * (4 * sizeof(double) + sizeof(int32_t)); }

// Per family: the rays to march (lit, or an argmin candidate); the argmin
// candidates first (they all land in the first chunk, which also forms the
// family's H2 / CO sums), then the other lit rays, each group by ascending id.
struct RtFamilies {
  int rays[6][kMaxRays];
  uint8_t flags[6][kMaxRays];
  int n[6];
  int chunks;
};

static void rt_families(const RaySet& rs, RtFamilies* F) {
  F->chunks = 1;
  for (int f = 0; f < 6; ++f) {
    F->n[f] = 0;
    double ds_min = INFINITY;
    for (int r = 0; r < rs.n; ++r)
      if (rs.axis[r] * 2 + rs.fwd[r] == f) ds_min = fmin(ds_min, rs.ds[r]);
    for (int pass = 0; pass < 2; ++pass)
      for (int r = 0; r < rs.n; ++r) {
        if (rs.axis[r] * 2 + rs.fwd[r] != f) continue;
        const bool cand = rs.ds[r] <= ds_min * (1.0 + 1e-9);
        if (pass == 0 ? !cand : (cand || rs.g_ext[r] == 0.0)) continue;
        uint8_t fl = cand ? kRtCand : 0;
        if (rs.g_ext[r] != 0.0) fl |= kRtLit;
        F->rays[f][F->n[f]] = r;
        F->flags[f][F->n[f]++] = fl;
      }
    const int ch = (int)ceil_div(F->n[f], kRayChunk);
    if (ch > F->chunks) F->chunks = ch;
  }
}

int rt_launch_count(const RaySet& rs) {
  static thread_local RtFamilies F;
  rt_families(rs, &F);
  return F.chunks + 1;
}

cudaError_t launch_fuv_full(int64_t nx, int64_t ny, int64_t nz, const double* dens,
                            const double* xh2, const double* xco, const RaySet& rs,
                            void* work, double* g0, double* av, double* nh, double* nh2,
                            double* nco, int32_t* ray, int sms, cudaStream_t s) {
  const int64_t n = nx * ny * nz;
  if (n <= 0) return cudaSuccess;
  RtPartial P;
  P.g0 = (double*)work;
  P.nh = P.g0 + 6 * n;
  P.nh2 = P.nh + 6 * n;
  P.nco = P.nh2 + 6 * n;
  P.id = (int32_t*)(P.nco + 6 * n);
  static thread_local RtFamilies F;  // ~23 KB: kept off the stack
  rt_families(rs, &F);
  RtLaunch L;
  const int64_t dims[3] = {nx, ny, nz};
  L.start[0] = 0;
  for (int f = 0; f < 6; ++f) L.start[f + 1] = L.start[f] + n / dims[f >> 1];
  for (int ch = 0; ch < F.chunks; ++ch) {
    for (int f = 0; f < 6; ++f) {
      const int k0 = ch * kRayChunk;
      const int rest = F.n[f] - k0;
      const int cnt = rest < 0 ? 0 : (rest > kRayChunk ? kRayChunk : rest);
      L.n[f] = cnt;
      for (int r = 0; r < cnt; ++r) {
        const int id = F.rays[f][k0 + r];
        L.id[f][r] = id;
        L.ds[f][r] = rs.ds[id];
        L.gw[f][r] = rs.g_ext[id] * rs.w[id];
        L.flags[f][r] = F.flags[f][k0 + r];
      }
      if (ch == 0 && cnt == 0) {
        // a family without marched rays still has a slice: no share, no ray
        cudaError_t e = cudaMemsetAsync(P.g0 + f * n, 0, sizeof(double) * n, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(P.id + f * n, 0xff, sizeof(int32_t) * n, s);
        if (e != cudaSuccess) return e;
      }
    }
    rt_walk_kernel<<<(unsigned)ceil_div(L.start[6], 128), 128, 0, s>>>(nx, ny, nz, dens, xh2,
                                                                         xco, L, P, ch == 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  rt_merge_kernel<<<grid_for(n, sms, 8), kThreads, 0, s>>>(n, P, g0, av, nh, nh2, nco, ray);
  return cudaGetLastError();
}

}  // namespace p3d
