// mh_exp.h -- single-precision exp from basic IEEE operations only.
//
// The PSDF update and the inlier prediction evaluate exp() per voxel and per
// vertex (the Gaussian of UpdateBlocksBayesianKernel and the distance and
// disk weights of PredictOutlierRatioKernel, mapping/update_bayesian.cu).
// Library exponentials are not correctly rounded, and CUDA's and the host C
// library's differ in the last bits, so a CPU restatement of the update could
// only match the GPU to a few ulp.  This function uses nothing but IEEE
// single-precision +, -, *, round-to-nearest-even and exact power-of-two
// scaling, with no fused multiply-add, so the GPU and any CPU compiled without
// FMA contraction compute the same bits.
//
// Method (Cody & Waite, "Software Manual for the Elementary Functions", 1980):
//   k = rint(x / ln 2),  r = (x - k * L1) - k * L2,  L1 + L2 = ln 2,
// where L1 = 0.693359375 has 9 significant bits, so k * L1 is exact for the
// |k| <= 150 that occur, and |r| <= ln2 / 2 (plus rounding).  exp(r) is the
// Taylor series to degree 7, evaluated by Horner's rule: the truncation error
// |r|^8 / 8! is below 6e-9, a tenth of an ulp.  The result is scaled by 2^k
// in two power-of-two steps, each factor a normal number, so only the last
// product can round (into the subnormal range).  Measured against the
// double-precision exp rounded to single, on every 97th float in
// [-103.9, 88.7]: at most 1 ulp apart.
#pragma once

#include <cstdint>
#include <cstring>
#include <cmath>

#if defined(__CUDACC__)
#define MH_HD __host__ __device__ __forceinline__
#else
#define MH_HD inline
#endif

// 2^j as a float, -126 <= j <= 127
MH_HD float mh_pow2i(int j) {
#if defined(__CUDA_ARCH__)
  return __int_as_float((j + 127) << 23);
#else
  const uint32_t u = (uint32_t)(j + 127) << 23;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

// round to the nearest integer, ties to even
MH_HD float mh_rint(float v) {
#if defined(__CUDA_ARCH__)
  return rintf(v);
#else
  return std::nearbyint(v);
#endif
}

// products and sums that no compiler flag may fuse: the device forms are the
// round-to-nearest intrinsics; host code including this header is compiled
// with -ffp-contract=off
MH_HD float mh_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
MH_HD float mh_add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}

MH_HD float mh_expf(float x) {
  if (!(x == x)) return x;                        // NaN
  if (x > 88.7228394f) return HUGE_VALF;          // above ln(FLT_MAX)
  if (x < -103.972084f) return 0.0f;              // below half the smallest subnormal
  const float k = mh_rint(mh_mul(x, 1.44269504f));
  const float r = mh_add(mh_add(x, -mh_mul(k, 0.693359375f)), -mh_mul(k, -2.12194440e-4f));
  float q = 1.98412701e-4f;                       // 1/7!
  q = mh_add(mh_mul(q, r), 1.38888892e-3f);       // 1/6!
  q = mh_add(mh_mul(q, r), 8.33333377e-3f);       // 1/5!
  q = mh_add(mh_mul(q, r), 4.16666679e-2f);       // 1/4!
  q = mh_add(mh_mul(q, r), 1.66666672e-1f);       // 1/3!
  q = mh_add(mh_mul(q, r), 0.5f);
  q = mh_add(mh_mul(q, r), 1.0f);
  q = mh_add(mh_mul(q, r), 1.0f);
  const int ki = (int)k;
  const int k1 = ki / 2, k2 = ki - k1;
  return mh_mul(mh_mul(q, mh_pow2i(k1)), mh_pow2i(k2));
}
