// p3d_maps.cu -- column-density maps of a grid (the observation pipeline's
// column_density_maps / integrate_column, prism3d/observations/
// jwst_pipeline.py:109-180) with the optional inclination shear
// (jwst_pipeline.py:472-520): LOS slice t shifted by tan(i) (t - n_los / 2)
// pixels along the first non-LOS axis, linear interpolation, 0 where the
// source position falls outside the grid.
//
// One thread per map pixel sums its line of sight in order (deterministic);
// threads of a warp take adjacent pixels of the last map axis, so for LOS
// axes 0 and 1 a warp reads contiguous z-runs.
#include <cmath>

#include "../../include/prism3d_gb300.h"
#include "p3d_capi_internal.cuh"
#include "p3d_common.cuh"

namespace p3d {

// Map axes: a (the sheared one) and b, each a grid axis other than los.
struct MapGeom {
  int64_t nx, ny, nz, n_los, na, nb, s_los, s_a, s_b;
};

static MapGeom map_geom(int los, int64_t nx, int64_t ny, int64_t nz) {
  MapGeom g{nx, ny, nz, 0, 0, 0, 0, 0, 0};
  const int64_t sx = ny * nz, sy = nz, sz = 1;
  if (los == 0) { g.n_los = nx; g.s_los = sx; g.na = ny; g.s_a = sy; g.nb = nz; g.s_b = sz; }
  else if (los == 1) { g.n_los = ny; g.s_los = sy; g.na = nx; g.s_a = sx; g.nb = nz; g.s_b = sz; }
  else { g.n_los = nz; g.s_los = sz; g.na = nx; g.s_a = sx; g.nb = ny; g.s_b = sy; }
  return g;
}

// Value of field k (0 n, 1 2 n x_H2, 2 n x_CO, 3 n x_C+, 4 n x_e) at cell c.
__device__ __forceinline__ double map_field(int k, int64_t c, const double* __restrict__ n,
                                            const double* __restrict__ xh2,
                                            const double* __restrict__ xco,
                                            const double* __restrict__ xcp,
                                            const double* __restrict__ xe) {
  const double d = n[c];
  switch (k) {
    case 0: return d;
    case 1: return d * xh2[c] * 2.0;
    case 2: return d * xco[c];
    case 3: return d * xcp[c];
    default: return d * xe[c];
  }
}

// nf fields (nf = 1: integrate `n` itself; nf = 5: the five column maps).
__global__ void column_maps_kernel(MapGeom g, int nf, double tan_inc, int sheared, double ds,
                                   const double* __restrict__ n, const double* __restrict__ xh2,
                                   const double* __restrict__ xco,
                                   const double* __restrict__ xcp,
                                   const double* __restrict__ xe, double* __restrict__ out) {
  const int64_t npix = g.na * g.nb;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < npix;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = q / g.nb, b = q - a * g.nb;
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int64_t t = 0; t < g.n_los; ++t) {
      const int64_t base = t * g.s_los + b * g.s_b;
      if (!sheared) {
        const int64_t c = base + a * g.s_a;
        for (int k = 0; k < nf; ++k) acc[k] += map_field(nf == 1 ? 0 : k, c, n, xh2, xco, xcp, xe);
      } else {
        const double dx = tan_inc * ((double)t - (double)g.n_los / 2.0);
        const double src = (double)a - dx;
        if (!(src >= 0.0 && src <= (double)(g.na - 1))) continue;
        const double fl = floor(src);
        const int64_t i0 = (int64_t)fl;
        const int64_t i1 = i0 + 1 < g.na ? i0 + 1 : g.na - 1;
        const double w = src - fl;
        for (int k = 0; k < nf; ++k) {
          const int kk = nf == 1 ? 0 : k;
          acc[k] += (1.0 - w) * map_field(kk, base + i0 * g.s_a, n, xh2, xco, xcp, xe) +
                    w * map_field(kk, base + i1 * g.s_a, n, xh2, xco, xcp, xe);
        }
      }
    }
    for (int k = 0; k < nf; ++k) out[k * npix + q] = acc[k] * ds;
    if (nf == 5) out[5 * npix + q] = acc[0] * ds * kAVperNH;
  }
}

}  // namespace p3d

using namespace p3d;

static int check_map_args(int64_t nx, int64_t ny, int64_t nz, int los, double cell_size,
                          double inc) {
  if (nx < 1 || ny < 1 || nz < 1) return set_error(P3D_EINVAL, "grid dimensions must be >= 1");
  if (los < 0 || los > 2) return set_error(P3D_EINVAL, "los_axis must be 0, 1 or 2");
  if (!(cell_size > 0.0)) return set_error(P3D_EINVAL, "cell_size must be > 0");
  if (!std::isfinite(inc) || fabs(inc) >= 90.0)
    return set_error(P3D_EINVAL, "inclination must be finite and below 90 degrees");
  return P3D_OK;
}

static void launch_maps(int los, int64_t nx, int64_t ny, int64_t nz, int nf, double cell_size,
                        double inc, const double* n, const double* xh2, const double* xco,
                        const double* xcp, const double* xe, double* out, cudaStream_t s,
                        int sms) {
  const MapGeom g = map_geom(los, nx, ny, nz);
  const bool sheared = fabs(inc) >= 0.01;
  const double t = sheared ? tan(inc * 3.14159265358979323846 / 180.0) : 0.0;
  column_maps_kernel<<<grid_for(g.na * g.nb, sms, 8), kThreads, 0, s>>>(
      g, nf, t, sheared ? 1 : 0, cell_size, n, xh2, xco, xcp, xe, out);
}

extern "C" {

int p3d_column_maps_dev(int64_t nx, int64_t ny, int64_t nz, const double* density,
                        const double* x_h2, const double* x_co, const double* x_cp,
                        const double* x_e, double cell_size, int32_t los_axis,
                        double inclination_deg, double* maps, void* stream) {
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if ((rc = check_map_args(nx, ny, nz, los_axis, cell_size, inclination_deg))) return rc;
  if (!density || !x_h2 || !x_co || !x_cp || !x_e || !maps)
    return set_error(P3D_EINVAL, "null array");
  launch_maps(los_axis, nx, ny, nz, 5, cell_size, inclination_deg, density, x_h2, x_co, x_cp,
              x_e, maps, (cudaStream_t)stream, st->sms);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "column maps launch");
}

int p3d_column_maps(int64_t nx, int64_t ny, int64_t nz, const double* density, const double* x_h2,
                    const double* x_co, const double* x_cp, const double* x_e, double cell_size,
                    int32_t los_axis, double inclination_deg, double* maps) {
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if ((rc = check_map_args(nx, ny, nz, los_axis, cell_size, inclination_deg))) return rc;
  if (!density || !x_h2 || !x_co || !x_cp || !x_e || !maps)
    return set_error(P3D_EINVAL, "null array");
  const size_t n = (size_t)(nx * ny * nz);
  const MapGeom g = map_geom(los_axis, nx, ny, nz);
  const size_t npix = (size_t)(g.na * g.nb);
  double* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, sizeof(double) * (5 * n + 6 * npix));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(P3D_ENOMEM, "column maps staging");
  }
  const double* src[5] = {density, x_h2, x_co, x_cp, x_e};
  for (int k = 0; k < 5 && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(buf + k * n, src[k], sizeof(double) * n, cudaMemcpyHostToDevice,
                        st->stream);
  if (e == cudaSuccess) {
    launch_maps(los_axis, nx, ny, nz, 5, cell_size, inclination_deg, buf, buf + n, buf + 2 * n,
                buf + 3 * n, buf + 4 * n, buf + 5 * n, st->stream, st->sms);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(maps, buf + 5 * n, sizeof(double) * 6 * npix, cudaMemcpyDeviceToHost,
                        st->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st->stream);
  cudaFree(buf);
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "column maps");
}

int p3d_integrate_column(int64_t nx, int64_t ny, int64_t nz, const double* field,
                         double cell_size, int32_t los_axis, double* out) {
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if ((rc = check_map_args(nx, ny, nz, los_axis, cell_size, 0.0))) return rc;
  if (!field || !out) return set_error(P3D_EINVAL, "null array");
  const size_t n = (size_t)(nx * ny * nz);
  const MapGeom g = map_geom(los_axis, nx, ny, nz);
  const size_t npix = (size_t)(g.na * g.nb);
  double* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, sizeof(double) * (n + npix));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(P3D_ENOMEM, "integrate column staging");
  }
  e = cudaMemcpyAsync(buf, field, sizeof(double) * n, cudaMemcpyHostToDevice, st->stream);
  if (e == cudaSuccess) {
    launch_maps(los_axis, nx, ny, nz, 1, cell_size, 0.0, buf, buf, buf, buf, buf, buf + n,
                st->stream, st->sms);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, buf + n, sizeof(double) * npix, cudaMemcpyDeviceToHost, st->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st->stream);
  cudaFree(buf);
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "integrate column");
}

}  // extern "C"
