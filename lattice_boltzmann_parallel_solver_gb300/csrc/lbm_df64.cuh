// lbm_df64.cuh -- float-float ("double-float") arithmetic for the quadratic
// term of the fixed-point collision (lbm_fx.cuh).  A value is hi + lo, two
// binary32 numbers with |lo| <= ulp(hi)/2 after normalisation, about 48
// significant bits.  GB300 runs float32 FMAs at 64x its float64 rate.
//
// The error-free transformations are the published ones:
//   fast_two_sum  Dekker 1971 (s = a + b and its exact error, |a| >= |b|)
//   two_prod      with a fused multiply-add (p = a * b, e = fma(a, b, -p))
// and the products built from them follow Dekker's double-length arithmetic
// as used in the QD library (Hida, Li, Bailey 2001).  The same code compiles
// for the host (tests and emulation of the arithmetic) with IEEE binary32
// operations and no contraction.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace lbm {
namespace df {

#if defined(__CUDA_ARCH__)
DF_HD float add_(float a, float b) { return __fadd_rn(a, b); }
DF_HD float sub_(float a, float b) { return __fsub_rn(a, b); }
DF_HD float mul_(float a, float b) { return __fmul_rn(a, b); }
DF_HD float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
// host build must use -ffp-contract=off
DF_HD float add_(float a, float b) { return a + b; }
DF_HD float sub_(float a, float b) { return a - b; }
DF_HD float mul_(float a, float b) { return a * b; }
DF_HD float fma_(float a, float b, float c) { return fmaf(a, b, c); }
#endif

struct F2 {
  float hi, lo;
};

DF_HD F2 fast_two_sum(float a, float b) {
  const float s = add_(a, b);
  return {s, sub_(b, sub_(s, a))};
}
DF_HD F2 two_prod(float a, float b) {
  const float p = mul_(a, b);
  return {p, fma_(a, b, -p)};
}
DF_HD F2 mul(F2 a, F2 b) {
  F2 p = two_prod(a.hi, b.hi);
  p.lo = fma_(a.hi, b.lo, fma_(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}
// a * c for a float constant c
DF_HD F2 mulf(F2 a, float c) {
  F2 p = two_prod(a.hi, c);
  p.lo = fma_(a.lo, c, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
DF_HD uint64_t bits64(double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
}
DF_HD double from_bits64(uint64_t u) {
  double d;
  memcpy(&d, &u, 8);
  return d;
}
DF_HD float from_bits32(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
DF_HD uint32_t bits32(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

// float64 -> float-float without float64 arithmetic (the relaxation constant
// omega/2): hi is d truncated to 24 significant bits, lo the remaining 29 bits
// rounded to 24.  Magnitudes below 2^-74 keep only hi (and below 2^-126 become
// 0); omega/2 lies in (0, 1).
DF_HD F2 split(double d) {
  const uint64_t b = bits64(d);
  const uint32_t bh = (uint32_t)(b >> 32), bl = (uint32_t)b;
  const uint32_t e = (bh >> 20) & 0x7FFu;
  const uint32_t sign = bh & 0x80000000u;
  float hi;
  if (e >= 897u && e <= 1150u) {
    // binary32 with exponent e - 896 and the top 23 explicit mantissa bits
    hi = from_bits32(sign | ((e - 896u) << 23) | ((bh & 0xFFFFFu) << 3) | (bl >> 29));
  } else {
    hi = 0.0f;
  }
  const uint32_t low = bl & 0x1FFFFFFFu;
  const uint32_t sbits = (e >= 949u && e <= 1150u) ? (sign | ((e - 948u) << 23)) : 0u;
  const float lo = mul_((float)low, from_bits32(sbits));
  return {hi, lo};
}

}  // namespace df
}  // namespace lbm
