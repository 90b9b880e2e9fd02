// p3d_fastexp.cuh -- table-driven FP64 exponential for the kernels that are
// bound by the FP64 pipe (thermal balance, ray march).
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so every FP64
// instruction of an exponential counts.  This follows the method of
// P. T. P. Tang, "Table-driven implementation of the exponential function in
// IEEE floating-point arithmetic", ACM TOMS 15 (1989) 144-157:
//   x = (64 m + j) ln2 / 64 + r,  |r| <= ln2 / 128,
//   exp(x) = 2^m * 2^(j/64) * e^r,
// with 2^(j/64) from a 64-entry table (each entry the double nearest to the
// exact value, computed offline in 60-digit decimal arithmetic), ln2 / 64
// split into a head and a tail so that r is exact to ~1e-32, and e^r - 1 by
// its Taylor polynomial of degree 5 (truncation < 4e-17).  The integer m
// enters through the exponent bits.  Cost: six FMAs, one multiply, one add,
// one table load and integer operations; error <= ~1 ulp for |x| <= 700
// (checked against the C library in tests/test_fastexp_host.py).  Outside
// that range (never reached by the thermal terms; deep rays of the ray
// march) exp() is called.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

// Device functions under nvcc; plain inline functions for the host build the
// CPU tests compile with g++.
#ifdef __CUDACC__
#define P3D_FE_FN __device__ __forceinline__
#define P3D_FE_TAB __device__ static const
#else
#define P3D_FE_FN inline
#define P3D_FE_TAB static const
#endif

namespace p3d {

// 2^(j/64), j = 0..63, nearest doubles.
P3D_FE_TAB double kExp2J64[64] = {
    0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, 0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0,
    0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, 0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0,
    0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, 0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0,
    0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, 0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0,
    0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, 0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0,
    0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, 0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0,
    0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, 0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0,
    0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, 0x1.6247eb03a5585p+0, 0x1.6623882552225p+0,
    0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, 0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0,
    0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, 0x1.82589994cce13p+0, 0x1.868d99b4492edp+0,
    0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, 0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0,
    0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, 0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0,
    0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, 0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0,
    0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, 0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0,
    0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, 0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0,
    0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, 0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0,
};

P3D_FE_FN int64_t fe_bits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  int64_t b;
  memcpy(&b, &x, 8);
  return b;
#endif
}

P3D_FE_FN double fe_double(int64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}

P3D_FE_FN double fe_table(int j) {
#ifdef __CUDA_ARCH__
  return __ldg(kExp2J64 + j);
#else
  return kExp2J64[j];
#endif
}

P3D_FE_FN double exp64(double x) {
  // |x| > 700 (or NaN): library exponential
  if ((int)((fe_bits(x) >> 32) & 0x7fffffff) > 0x4085e000) return std::exp(x);
  const double kInvL = 0x1.71547652b82fep+6;   // 64 / ln 2
  const double kLhi = 0x1.62e42fefa39efp-7;    // ln 2 / 64, head
  const double kLlo = 0x1.abc9e3b39803fp-62;   // ln 2 / 64, tail
  const double kShift = 0x1.8p52;              // rounds to an integer in the low bits
  const double t = fma(x, kInvL, kShift);
  const int k = (int)(fe_bits(t) & 0xffffffff);  // nearest integer of 64 x / ln 2
  const double kd = t - kShift;
  double r = fma(-kd, kLhi, x);
  r = fma(-kd, kLlo, r);
  double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  q = fma(q, r, 1.0);
  const double p = q * r;  // e^r - 1
  const double tj = fe_table(k & 63);
  const double v = fma(tj, p, tj);  // 2^(j/64) e^r, in [1, 2)
  return fe_double(fe_bits(v) + ((int64_t)(k >> 6) << 52));
}

}  // namespace p3d
