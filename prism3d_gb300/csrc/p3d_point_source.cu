// p3d_point_source.cu -- FUV field of an embedded point source
// (prism3d/radiative_transfer/fuv_rt_3d.py:74-212).
//
// Per axis the column from the star's plane outward: cells above the plane
// sum the layers star .. i-1, cells below i+1 .. star (the star cell's layer
// included, the cell's own excluded), cells in the plane 0.  Each cell takes
// the column of its dominant displacement axis (ties: x before y before z),
// scaled by min(r / max(|d_dom|, cell / 2), 3), minus half its own layer
// (midpoint), clamped at 0; A_V = 5.34e-22 N_H and
// G0 = L / (4 pi r^2 F_Habing) exp(-1.8 A_V) with r >= cell / 2.
//
// One launch per axis, one thread per pencil along that axis: it runs both
// half-line sums in order (the reference's cumsum order) and writes the
// cells whose dominant axis it is, so every cell is written once.  Products
// and sums use explicit round-to-nearest operations (no contraction), so the
// columns are bit-identical to the reference; G0 differs by the rounding of
// exp.
#include <cmath>

#include "../../include/prism3d_gb300.h"
#include "p3d_capi_internal.cuh"
#include "p3d_common.cuh"

namespace p3d {

constexpr double kG0ToFlux = 1.6e-3;  // prism3d/utils/constants.py:45

struct PsGeom {
  int64_t n[3];
  int64_t star[3];
  double spos[3];
  double cell, lum;
  int cols_only;  // 1: write N_H2 / N_CO only (the steady driver's per-iteration columns)
};

__device__ __forceinline__ void ps_cell(const PsGeom& g, int axis, int64_t c, const int64_t* idx,
                                        double col_h, double col_h2, double col_co,
                                        double lay_h, double lay_h2, double lay_co,
                                        double* __restrict__ g0, double* __restrict__ av,
                                        double* __restrict__ nh, double* __restrict__ nh2,
                                        double* __restrict__ nco) {
  double d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = __dsub_rn(__dmul_rn((double)idx[k] + 0.5, g.cell), g.spos[k]);
  const double ax = fabs(d[0]), ay = fabs(d[1]), az = fabs(d[2]);
  const int dom = (ax >= ay && ax >= az) ? 0 : ((ay > ax && ay >= az) ? 1 : 2);
  if (dom != axis) return;
  double r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])),
                            __dmul_rn(d[2], d[2])));
  r = fmax(r, 0.5 * g.cell);
  const double dd = fmax(dom == 0 ? ax : (dom == 1 ? ay : az), 0.5 * g.cell);
  const double pc = fmin(r / dd, 3.0);
  const double th = fmax(__dsub_rn(__dmul_rn(col_h, pc), __dmul_rn(__dmul_rn(0.5, lay_h), pc)), 0.0);
  const double th2 =
      fmax(__dsub_rn(__dmul_rn(col_h2, pc), __dmul_rn(__dmul_rn(0.5, lay_h2), pc)), 0.0);
  const double tco =
      fmax(__dsub_rn(__dmul_rn(col_co, pc), __dmul_rn(__dmul_rn(0.5, lay_co), pc)), 0.0);
  nh2[c] = th2;
  nco[c] = tco;
  if (g.cols_only) return;
  const double a = __dmul_rn(th, kAVperNH);
  const double four_pi = 4.0 * 3.14159265358979323846;
  const double unatt = g.lum / __dmul_rn(__dmul_rn(four_pi, __dmul_rn(r, r)), kG0ToFlux);
  g0[c] = unatt * exp(-1.8 * a);
  av[c] = a;
  nh[c] = th;
}

__global__ void point_source_kernel(int axis, PsGeom g, const double* __restrict__ dens,
                                    const double* __restrict__ xh2, const double* __restrict__ xco,
                                    double* __restrict__ g0, double* __restrict__ av,
                                    double* __restrict__ nh, double* __restrict__ nh2,
                                    double* __restrict__ nco) {
  const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
  const int64_t np = g.n[a1] * g.n[a2];
  const int64_t sz[3] = {g.n[1] * g.n[2], g.n[2], 1};
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t idx[3];
    idx[a1] = p / g.n[a2];
    idx[a2] = p - idx[a1] * g.n[a2];
    const int64_t base = idx[a1] * sz[a1] + idx[a2] * sz[a2], st = sz[axis];
    const int64_t na = g.n[axis], s = g.star[axis];
    auto layers = [&](int64_t k, double* lh, double* lh2, double* lco) {
      const int64_t c = base + k * st;
      const double n = dens[c];
      *lh = __dmul_rn(n, g.cell);
      *lh2 = xh2 ? __dmul_rn(__dmul_rn(__dmul_rn(n, xh2[c]), 2.0), g.cell) : 0.0;
      *lco = xco ? __dmul_rn(__dmul_rn(n, xco[c]), g.cell) : 0.0;
    };
    double lh, lh2, lco;
    // the star's plane
    layers(s, &lh, &lh2, &lco);
    idx[axis] = s;
    ps_cell(g, axis, base + s * st, idx, 0.0, 0.0, 0.0, lh, lh2, lco, g0, av, nh, nh2, nco);
    // above
    double ch = 0.0, ch2 = 0.0, cco = 0.0;
    for (int64_t k = s; k < na - 1; ++k) {
      layers(k, &lh, &lh2, &lco);
      ch = __dadd_rn(ch, lh);
      ch2 = __dadd_rn(ch2, lh2);
      cco = __dadd_rn(cco, lco);
      double oh, oh2, oco;
      layers(k + 1, &oh, &oh2, &oco);
      idx[axis] = k + 1;
      ps_cell(g, axis, base + (k + 1) * st, idx, ch, ch2, cco, oh, oh2, oco, g0, av, nh, nh2, nco);
    }
    // below
    ch = ch2 = cco = 0.0;
    for (int64_t k = s; k >= 1; --k) {
      layers(k, &lh, &lh2, &lco);
      ch = __dadd_rn(ch, lh);
      ch2 = __dadd_rn(ch2, lh2);
      cco = __dadd_rn(cco, lco);
      double oh, oh2, oco;
      layers(k - 1, &oh, &oh2, &oco);
      idx[axis] = k - 1;
      ps_cell(g, axis, base + (k - 1) * st, idx, ch, ch2, cco, oh, oh2, oco, g0, av, nh, nh2, nco);
    }
  }
}

static int64_t star_index(double pos, double cell, int64_t n) {
  double v = pos / cell;
  v = v < 0.0 ? 0.0 : (v > (double)(n - 1) ? (double)(n - 1) : v);
  return (int64_t)v;  // truncation, as int() of the clipped value
}

cudaError_t launch_point_source(int64_t nx, int64_t ny, int64_t nz, const double* dens,
                                const double* xh2, const double* xco, const double* star_pos,
                                double lum, double cell, int cols_only, double* g0, double* av,
                                double* nh, double* nh2, double* nco, int sms, cudaStream_t s) {
  PsGeom g;
  g.n[0] = nx; g.n[1] = ny; g.n[2] = nz;
  g.cell = cell;
  g.lum = lum;
  g.cols_only = cols_only;
  for (int k = 0; k < 3; ++k) {
    g.spos[k] = star_pos[k];
    g.star[k] = star_index(star_pos[k], cell, g.n[k]);
  }
  for (int axis = 0; axis < 3; ++axis) {
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    point_source_kernel<<<grid_for(g.n[a1] * g.n[a2], sms, 8), kThreads, 0, s>>>(
        axis, g, dens, xh2, xco, g0, av, nh, nh2, nco);
  }
  return cudaGetLastError();
}

}  // namespace p3d

using namespace p3d;

extern "C" {

int p3d_fuv_point_source_dev(int64_t nx, int64_t ny, int64_t nz, const double* density,
                             const double* x_h2, const double* x_co, const double* star_pos,
                             double L_fuv, double cell_size, double* g0, double* a_v,
                             double* n_h, double* n_h2, double* n_co, void* stream) {
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if (nx < 1 || ny < 1 || nz < 1) return set_error(P3D_EINVAL, "grid dimensions must be >= 1");
  if (!(cell_size > 0.0)) return set_error(P3D_EINVAL, "cell_size must be > 0");
  if (!density || !star_pos || !g0 || !a_v || !n_h || !n_h2 || !n_co)
    return set_error(P3D_EINVAL, "null array");
  cudaError_t e = launch_point_source(nx, ny, nz, density, x_h2, x_co, star_pos, L_fuv,
                                      cell_size, 0, g0, a_v, n_h, n_h2, n_co, st->sms,
                                      (cudaStream_t)stream);
  return e == cudaSuccess ? P3D_OK : cuda_fail(e, "point source launch");
}

int p3d_fuv_point_source(int64_t nx, int64_t ny, int64_t nz, const double* density,
                         const double* x_h2, const double* x_co, const double* star_pos,
                         double L_fuv, double cell_size, double* g0, double* a_v, double* n_h,
                         double* n_h2, double* n_co) {
  DeviceState* st;
  int rc = get_state(&st);
  if (rc) return rc;
  if (nx < 1 || ny < 1 || nz < 1) return set_error(P3D_EINVAL, "grid dimensions must be >= 1");
  if (!density || !star_pos || !g0 || !a_v || !n_h || !n_h2 || !n_co)
    return set_error(P3D_EINVAL, "null array");
  const size_t n = (size_t)(nx * ny * nz), b = sizeof(double) * n;
  double* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, 8 * b);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(P3D_ENOMEM, "point source staging");
  }
  double *dd = buf, *dh2 = x_h2 ? buf + n : nullptr, *dco = x_co ? buf + 2 * n : nullptr;
  e = cudaMemcpyAsync(dd, density, b, cudaMemcpyHostToDevice, st->stream);
  if (e == cudaSuccess && dh2) e = cudaMemcpyAsync(dh2, x_h2, b, cudaMemcpyHostToDevice, st->stream);
  if (e == cudaSuccess && dco) e = cudaMemcpyAsync(dco, x_co, b, cudaMemcpyHostToDevice, st->stream);
  if (e != cudaSuccess) {
    cudaFree(buf);
    return cuda_fail(e, "point source H2D");
  }
  double* o = buf + 3 * n;
  rc = p3d_fuv_point_source_dev(nx, ny, nz, dd, dh2, dco, star_pos, L_fuv, cell_size, o, o + n,
                                o + 2 * n, o + 3 * n, o + 4 * n, st->stream);
  double* outs[5] = {g0, a_v, n_h, n_h2, n_co};
  for (int k = 0; k < 5 && !rc; ++k) {
    e = cudaMemcpyAsync(outs[k], o + k * n, b, cudaMemcpyDeviceToHost, st->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "point source D2H");
  }
  if (!rc) rc = sync_check(st->stream, "point source");
  cudaStreamSynchronize(st->stream);
  cudaFree(buf);
  return rc;
}

}  // extern "C"
