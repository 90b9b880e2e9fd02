// p3d_chem.cuh -- device chemistry cell functions.
#pragma once

#include "p3d_common.cuh"

namespace p3d {

// rust/src/chemistry.rs:13-98.  y = (x_hi, x_h2, x_cp, x_c, x_co), in-out.
__device__ __forceinline__ void chem_euler_cell(double n_h, double kpd, double kci,
                                                double acp, double kco, double rh2,
                                                double rcr, double x_c_total, double* y,
                                                double hcop, int n_substeps, double conv_tol) {
  double x_hi = y[0], x_h2 = y[1], x_cp = y[2], x_c = y[3], x_co = y[4];
  double dt = 1e10;
  for (int step = 0; step < n_substeps; ++step) {
    double xe = fmax(x_cp + hcop, 1e-30);
    double dx_h2 = rh2 * x_hi - kpd * x_h2 - rcr * x_h2;
    double dx_h = -2.0 * dx_h2;
    double alpha_ne = acp * xe * n_h;
    double x_oh = 1e-9 + 9e-8 * fmin(fmax(x_h2 * 10.0, 0.0), 1.0);
    double form_co = 1e-10 * x_c * x_oh * n_h;
    double dx_cp = kci * x_c - alpha_ne * x_cp + kco * x_co;
    double dx_co = form_co - kco * x_co;
    double dx_c = -kci * x_c + alpha_ne * x_cp - form_co;
    double max_rate = fmax(fabs(dx_h2) / fmax(x_h2, 1e-20),
                           fmax(fabs(dx_cp) / fmax(x_cp, 1e-20), fabs(dx_co) / fmax(x_co, 1e-20)));
    double dt_eff = (max_rate * dt > 0.1) ? 0.1 / fmax(max_rate, 1e-30) : dt;
    x_hi = fmax(x_hi + dx_h * dt_eff, 1e-30);
    x_h2 = fmax(x_h2 + dx_h2 * dt_eff, 1e-30);
    x_cp = fmax(x_cp + dx_cp * dt_eff, 1e-30);
    x_c = fmax(x_c + dx_c * dt_eff, 1e-30);
    x_co = fmax(x_co + dx_co * dt_eff, 1e-30);
    double h_sum = x_hi + 2.0 * x_h2;
    x_hi /= h_sum;
    x_h2 /= h_sum;
    double c_sum = x_cp + x_c + x_co;
    if (c_sum > 0.0) {
      double scale = x_c_total / c_sum;
      x_cp *= scale;
      x_c *= scale;
      x_co *= scale;
    }
    if (step > 0 && step % 20 == 0 && dt >= 1e15 && max_rate * dt < conv_tol) break;
    dt = fmin(dt * 3.0, 1e16);
  }
  y[0] = x_hi; y[1] = x_h2; y[2] = x_cp; y[3] = x_c; y[4] = x_co;
}

cudaError_t launch_chem_euler(int64_t n, const double* const* rates, double x_c_total,
                              double* const* state7, const double* x_hcop, int n_substeps,
                              double conv_tol, int sms, cudaStream_t s);

}  // namespace p3d
