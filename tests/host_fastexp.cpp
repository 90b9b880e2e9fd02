// Host build of the table-driven exponential (prism3d_gb300/csrc/
// p3d_fastexp.cuh) for the CPU tests: the same source compiled by g++.
#include "../prism3d_gb300/csrc/p3d_fastexp.cuh"

extern "C" void fe_exp64(long n, const double* x, double* out) {
  for (long i = 0; i < n; ++i) out[i] = p3d::exp64(x[i]);
}
