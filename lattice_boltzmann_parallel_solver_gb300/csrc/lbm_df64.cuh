// lbm_df64.cuh -- float-float ("double-float") arithmetic for the float64-storage
// fused step.  A value is hi + lo, two binary32 numbers with |lo| <= ulp(hi)/2
// after normalisation, about 48 significant bits.  GB300 runs float32 FMAs at
// 64x the float64 rate, so the BGK collision in float-float costs fewer cycles
// than in float64 while keeping the populations in float64 memory.
//
// The error-free transformations are the published ones:
//   two_sum       Knuth, TAOCP vol. 2, 4.2.2 (s = a + b, exact error)
//   fast_two_sum  Dekker 1971 (|a| >= |b|)
//   two_prod      with a fused multiply-add (p = a * b, e = fma(a, b, -p))
// and the add/multiply built from them follow Dekker's double-length
// arithmetic as used in the QD library (Hida, Li, Bailey 2001).
// The same code compiles for the host (tests of the arithmetic) with IEEE
// binary32 operations and no contraction.
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

DF_HD F2 two_sum(float a, float b) {
  const float s = add_(a, b);
  const float bb = sub_(s, a);
  const float e = add_(sub_(a, sub_(s, bb)), sub_(b, bb));
  return {s, e};
}
DF_HD F2 fast_two_sum(float a, float b) {
  const float s = add_(a, b);
  return {s, sub_(b, sub_(s, a))};
}
DF_HD F2 two_prod(float a, float b) {
  const float p = mul_(a, b);
  return {p, fma_(a, b, -p)};
}
// a + b (error bounded relative to |a| + |b|)
DF_HD F2 add(F2 a, F2 b) {
  F2 s = two_sum(a.hi, b.hi);
  s.lo = add_(s.lo, add_(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}
DF_HD F2 neg(F2 a) { return {-a.hi, -a.lo}; }
DF_HD F2 sub(F2 a, F2 b) { return add(a, neg(b)); }
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
DF_HD F2 from_float(float a) { return {a, 0.0f}; }
DF_HD int round_to_int(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(x);
#else
  return (int)lrintf(x);
#endif
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

// float64 -> float-float without float64 arithmetic: hi is d truncated to 24
// significant bits, lo the remaining 29 bits rounded to 24.  Magnitudes below
// 2^-74 keep only hi (and below 2^-126 become 0): populations never get there.
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

// float-float -> float64, rounded to nearest (ties to even up to a carry into
// the next binade): the low word is rounded onto hi's float64 grid as an
// integer and added to hi's mantissa.
DF_HD double to_double(F2 a) {
  a = fast_two_sum(a.hi, a.lo);
  const uint32_t hb = bits32(a.hi);
  const uint32_t eh = (hb >> 23) & 0xFFu;
  if (eh == 0u || eh == 0xFFu) return (double)a.hi + (double)a.lo;  // zero, subnormal, inf, nan
  const uint64_t sign = (uint64_t)(hb & 0x80000000u) << 32;
  // lo in units of hi's float64 ulp, 2^(E - 52) with E = eh - 127
  const int k = 52 - ((int)eh - 127);  // scale 2^k
  const float lo_units = mul_(a.lo, from_bits32((uint32_t)(k + 127) << 23));
  const float signed_units = (hb & 0x80000000u) ? -lo_units : lo_units;
  const int64_t L = (int64_t)round_to_int(signed_units);
  int64_t M = ((int64_t)((hb & 0x7FFFFFu) | 0x800000u) << 29) + L;
  int64_t E = (int64_t)eh - 127 + 1023;
  if (M >= ((int64_t)1 << 53)) {
    M = (M + 1) >> 1;
    E += 1;
  } else if (M < ((int64_t)1 << 52)) {
    M <<= 1;
    E -= 1;
  }
  return from_bits64(sign | ((uint64_t)E << 52) | ((uint64_t)M & 0xFFFFFFFFFFFFFull));
}

// float-float constants of one relaxation: omega, 1 - omega and the weights
struct Consts {
  F2 om, om1, w0, w1, w5;
};

// BGK collision of one node in float-float, in place: moments in the
// reference's summation order, one Newton step on a float reciprocal for
// 1/rho, then fpre_i = (1 - omega) f_i + omega w_i rho (B + 4.5 cu^2 +- 3 cu)
// with B = 1 - 1.5 |u|^2, opposite directions sharing the even part.
DF_HD void collide(F2 f[9], const Consts& c) {
  const F2 rho = add(add(add(add(f[0], f[1]), add(f[2], f[3])), add(add(f[4], f[5]), add(f[6], f[7]))), f[8]);
  const F2 jx = sub(add(add(f[1], f[5]), f[8]), add(add(f[3], f[6]), f[7]));
  const F2 jy = sub(add(add(f[2], f[5]), f[6]), add(add(f[4], f[7]), f[8]));
#if defined(__CUDA_ARCH__)
  const float r0 = __frcp_rn(rho.hi);
#else
  const float r0 = 1.0f / rho.hi;
#endif
  const F2 e = sub(from_float(1.0f), mulf(rho, r0));
  const F2 inv = add(from_float(r0), mulf(e, r0));
  const F2 ux = mul(jx, inv), uy = mul(jy, inv);
  const F2 B = sub(from_float(1.0f), mulf(add(mul(ux, ux), mul(uy, uy)), 1.5f));
  const F2 orho = mul(c.om, rho);
  const F2 W0 = mul(orho, c.w0), W1 = mul(orho, c.w1), W5 = mul(orho, c.w5);
  const F2 V1 = mulf(W1, 3.0f), V5 = mulf(W5, 3.0f);
  f[0] = add(mul(c.om1, f[0]), mul(W0, B));
  const F2 d58 = add(ux, uy), d67 = sub(uy, ux);
#define LBM_DF_PAIR(I, J, V, W, VV)                   \
  {                                                  \
    const F2 t = add(mulf(mul(V, V), 4.5f), B);      \
    const F2 s = mul(W, t);                          \
    const F2 m = mul(VV, V);                         \
    f[I] = add(mul(c.om1, f[I]), add(s, m));         \
    f[J] = add(mul(c.om1, f[J]), sub(s, m));         \
  }
  LBM_DF_PAIR(1, 3, ux, W1, V1)
  LBM_DF_PAIR(2, 4, uy, W1, V1)
  LBM_DF_PAIR(5, 7, d58, W5, V5)
  LBM_DF_PAIR(6, 8, d67, W5, V5)
#undef LBM_DF_PAIR
}

}  // namespace df
}  // namespace lbm
