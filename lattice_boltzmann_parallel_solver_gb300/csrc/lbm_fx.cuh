// lbm_fx.cuh -- 64-bit fixed-point populations and their BGK collision.
//
// The fixed-point storage ("fx64") keeps each population as its deviation from
// the lattice weight in 64-bit fixed point, d_i = round((f_i - w_i) 2^56):
// 72 B per node like float64, a resolution of 2^-56 (1.4e-17, finer than
// float64's spacing for f_i > 1/8), and the streaming and bounce-back moves
// stay exact.  GB300 runs float64 instructions, and conversions between 64-bit
// integers and floats, at about 1.6 per clock per SM -- a float64 BGK collision
// (~66 such instructions per node) is bound there at a sixth of the HBM
// roofline.  The collision below uses 32-bit integer and float32 instructions:
//
//   * with f_i = w_i + d_i, rho = 1 + D (D = sum d_i) and j = sum c_i d_i are
//     exact integer sums (sum w_i = 1 and sum c_i w_i = 0 cancel exactly);
//   * the linear part of BGK, omega (w_i rho + 3 w_i c_i.j - f_i), is
//     omega/36 times the exact integer L_i = 36 w_i D + 108 w_i c_i.j - 36 d_i
//     (36 w_i = 16, 4, 1), multiplied by M = omega/36 2^64 in five 32-bit
//     multiply-adds and rounded to nearest (mulq);
//   * the quadratic part omega w_i (4.5 (c_i.j)^2 - 1.5 |j|^2) / rho is a sum of
//     A = (omega/2) jx^2/rho, B = (omega/2) jy^2/rho and P = (omega/2) jx jy/rho,
//     formed in float-float (about 48 bits; the terms are small against f_i) and
//     converted to fixed point once each, with 32-bit conversions;
//   * d_i' = d_i + T_i + N_i is one exact integer addition.
//
// Nodes whose populations, density or velocity leave the range where every
// intermediate fits (|f_i - w_i| < 1/4, 0 < rho < 2, |ux| + |uy| <= 0.35) are
// collided in float64 by the caller instead.
#pragma once
#include <stdint.h>

#include "lbm_df64.cuh"

namespace lbm {
namespace fx {

constexpr int kQ = 53;  // scale of the exact moment sums of float64 inputs (lbm_reduce.cu)
constexpr int kS = 56;  // scale of the stored deviations
// stored value of a population that is not finite or too far from its weight
constexpr int64_t kNaN = (int64_t)0x8000000000000000ull;

#if defined(__CUDA_ARCH__)
DF_HD int clz64(uint64_t a) { return __clzll((long long)a); }
DF_HD uint32_t umulhi(uint32_t a, uint32_t b) { return __umulhi(a, b); }
DF_HD float fadd_rd(float a, float b) { return __fadd_rd(a, b); }
DF_HD uint32_t f2u_rn(float f) { return __float2uint_rn(f); }
DF_HD int32_t f2i_rn(float f) { return __float2int_rn(f); }
DF_HD float rcp(float a) { return __frcp_rn(a); }
DF_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
DF_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
#else
DF_HD int clz64(uint64_t a) { return a ? __builtin_clzll(a) : 64; }
DF_HD uint32_t umulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
DF_HD float fadd_rd(float a, float b) {
  // a + b rounded down: the round-to-nearest sum, stepped down when it is above
  const float s = a + b;
  const double e = (double)a + (double)b;  // exact for the operands used here
  return (double)s > e ? nextafterf(s, -INFINITY) : s;
}
DF_HD uint32_t f2u_rn(float f) { return (uint32_t)llrintf(f); }
DF_HD int32_t f2i_rn(float f) { return (int32_t)lrintf(f); }
DF_HD float rcp(float a) { return 1.0f / a; }
DF_HD double dsub(double a, double b) { return a - b; }
DF_HD double dadd(double a, double b) { return a + b; }
#endif

DF_HD uint32_t lo32(int64_t v) { return (uint32_t)(uint64_t)v; }
DF_HD int32_t hi32(int64_t v) { return (int32_t)(uint32_t)((uint64_t)v >> 32); }

// round(x 2^S) (ties away from zero) from the bits of x; kNaN when x is not
// finite or |x 2^S| >= 2^63
DF_HD int64_t round_scaled(double x, int S) {
  const uint64_t b = df::bits64(x);
  const int e = (int)((b >> 52) & 0x7FFu);
  if (e == 0x7FF) return kNaN;
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | ((uint64_t)(e != 0) << 52);
  // x 2^S = m 2^sh
  const int sh = (e == 0 ? 1 : e) - 1075 + S;
  uint64_t v;
  if (sh >= 0) {
    if (sh > 10) return kNaN;  // m < 2^53: m 2^sh < 2^63 needs sh <= 10
    v = m << sh;
  } else {
    const int r = -sh;
    v = r > 63 ? 0 : (m + (((uint64_t)1 << (r & 63)) >> 1)) >> (r & 63);
  }
  return (b >> 63) ? -(int64_t)v : (int64_t)v;
}

// f -> round(f 2^53); false when |f| >= 2 or f is not finite
DF_HD bool to_fixed(double f, int64_t& out) {
  out = round_scaled(f, kQ);
  return out != kNaN && out < ((int64_t)1 << 54) && out > -((int64_t)1 << 54);
}

// v 2^-S -> float64, round to nearest even (exact when |v| <= 2^53)
DF_HD double from_scaled(int64_t v, int S) {
  if (v == 0) return 0.0;
  const uint64_t sign = v < 0 ? 0x8000000000000000ull : 0ull;
  uint64_t a = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
  const int lz = clz64(a);
  int e = 63 - lz;  // a in [2^e, 2^(e+1))
  uint64_t m;
  if (e <= 52) {
    m = a << (52 - e);
  } else {
    const int s = e - 52;
    const uint64_t half = (uint64_t)1 << (s - 1);
    const uint64_t rem = a & (((uint64_t)1 << s) - 1);
    m = a >> s;
    if (rem > half || (rem == half && (m & 1))) ++m;
    if (m >> 53) {
      m >>= 1;
      ++e;
    }
  }
  return df::from_bits64(sign | ((uint64_t)(e - S + 1023) << 52) | (m & 0xFFFFFFFFFFFFFull));
}

// stored deviation of a population with float64 weight w: round((f - w) 2^56)
DF_HD int64_t to_fx(double f, double w) { return round_scaled(dsub(f, w), kS); }

// population from its stored deviation (NaN for kNaN)
DF_HD double from_fx(int64_t v, double w) {
  return v == kNaN ? df::from_bits64(0x7FF8000000000000ull) : dadd(w, from_scaled(v, kS));
}

// ---- the collision ------------------------------------------------------------

// round(Lu M 2^-64) for 0 <= Lu < 2^63 and M = mh 2^32 + ml < 2^63 with
// Lu_hi ml + Lu_lo mh + 2^32 < 2^64, in five 32-bit multiply-adds; round half up
DF_HD uint64_t mulq(uint64_t lu, uint32_t mh, uint32_t ml) {
  const uint32_t ll = (uint32_t)lu, lh = (uint32_t)(lu >> 32);
  uint64_t mid = (uint64_t)ll * mh + umulhi(ll, ml);
  mid += (uint64_t)lh * ml;
  const uint32_t c = (uint32_t)(mid >> 32) + ((uint32_t)mid >> 31);
  return (uint64_t)lh * mh + c;
}

// fixed-point integer (|v| < 2^56) -> float-float v 2^-56, from three exact
// 32-bit conversions (high word, 24 + 8 low bits); about 48 significant bits
DF_HD df::F2 q_to_f2(int64_t v) {
  const uint32_t l = lo32(v);
  const float h = df::mul_((float)hi32(v), 5.9604644775390625e-08f);        // 2^-24
  const float m = df::mul_((float)(l >> 8), 3.552713678800501e-15f);        // 2^-48
  const float b = df::mul_((float)(l & 0xFFu), 1.3877787807814457e-17f);   // 2^-56
  df::F2 s = df::fast_two_sum(h, m);  // exact: |h| >= 2^-24 > |m| or h = 0
  return df::fast_two_sum(s.hi, df::add_(s.lo, b));
}

// float-float x (|x.hi| < 1/4) -> round(x 2^56) with 32-bit conversions: the
// high part's magnitude a = |x.hi| 2^24 splits into floor(a) (a rounded-down
// magic-number addition) and a - floor(a) in [0, 1) (exact), which gives the low
// word; the sign is applied to both, and the low part adds round(x.lo 2^56)
DF_HD int64_t f2_to_q(df::F2 x) {
  const float magic = 12582912.0f;                    // 1.5 2^23
  const float a = df::mul_(fabsf(x.hi), 16777216.0f);  // |x.hi| 2^24 < 2^22
  const float t = fadd_rd(a, magic);                  // floor(a) + magic, exact
  const uint32_t fl = df::bits32(t) - df::bits32(magic);
  const float rem = df::sub_(a, df::sub_(t, magic));  // exact
  const uint32_t r1 = f2u_rn(df::mul_(rem, 4294967296.0f));
  const int64_t s = (int64_t)((int32_t)df::bits32(x.hi) >> 31);  // 0 or -1
  const int64_t v = (int64_t)(((uint64_t)fl << 32) | r1);
  const int32_t r2 = f2i_rn(df::mul_(x.lo, 72057594037927936.0f));  // 2^56
  return ((v ^ s) - s) + r2;
}

// omega-dependent constants of one relaxation
struct QConsts {
  uint32_t mh, ml;  // M = 4 round(omega/36 2^62) = mh 2^32 + ml
  int64_t m4;       // M / 4
  df::F2 om2;       // omega / 2
};

// M / 4 = round(omega / 36 * 2^62) from the bits of omega (host side)
inline QConsts q_consts(double omega) {
  const uint64_t b = df::bits64(omega);
  const int ex = (int)((b >> 52) & 0x7FFu);
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | ((uint64_t)(ex != 0) << 52);
  // omega = m 2^(ex - 1075): omega 2^62 / 36 = m 2^sh / 36, sh <= 10 for omega < 2
  const int sh = (ex == 0 ? 1 : ex) - 1075 + 62;
  const unsigned __int128 num = sh >= 0 ? (unsigned __int128)m << sh : (unsigned __int128)(sh > -64 ? m >> -sh : 0);
  const uint64_t m4 = (uint64_t)((num + 18) / 36);
  const uint64_t M = m4 << 2;
  QConsts c;
  c.mh = (uint32_t)(M >> 32);
  c.ml = (uint32_t)M;
  c.m4 = (int64_t)m4;
  c.om2 = df::split(omega * 0.5);
  return c;
}

// One node in place: d_i = round((f_i - w_i) 2^56).  Returns false (d
// untouched) outside the range above.
DF_HD bool collide_q(int64_t d[9], const QConsts& c) {
  uint32_t big = 0;  // |d_i| < 2^54: (hi32 + 2^22) < 2^23 for all i
#pragma unroll
  for (int i = 0; i < 9; ++i) big |= (uint32_t)hi32(d[i]) + (1u << 22);
  const int64_t pa = d[1] + d[5] + d[8], pb = d[3] + d[6] + d[7];
  const int64_t pc = d[2] + d[5] + d[6], pe = d[4] + d[7] + d[8];
  const int64_t D = (d[0] + d[2] + d[4]) + (pa + pb);
  const int64_t jx = pa - pb, jy = pc - pe;
  // |rho - 1| < 1
  if ((big >> 23) != 0u || (uint32_t)hi32(D) + (1u << 24) >= (1u << 25)) return false;
  const df::F2 Dq = q_to_f2(D), X = q_to_f2(jx), Y = q_to_f2(jy);
  const df::F2 r1 = df::fast_two_sum(1.0f, Dq.hi);
  const df::F2 R = df::fast_two_sum(r1.hi, df::add_(r1.lo, Dq.lo));  // rho
  if (!(R.hi > 9.5367431640625e-07f && fabsf(X.hi) + fabsf(Y.hi) <= 0.35f * R.hi)) return false;

  // linear part: T_i = round(omega/36 L_i), computed as mulq(L_i + 2^62) - M/4
  const int64_t off = (int64_t)1 << 62;
  const int64_t r4 = (D << 2) + off, ro = D + off;
  const int64_t X12 = jx * 12, Y12 = jy * 12;
  const int64_t d58 = (jx + jy) * 3, d67 = (jy - jx) * 3;
  int64_t Lu[9];
  Lu[0] = (D << 4) + off - d[0] * 36;
  Lu[1] = r4 + X12 - d[1] * 36;
  Lu[3] = r4 - X12 - d[3] * 36;
  Lu[2] = r4 + Y12 - d[2] * 36;
  Lu[4] = r4 - Y12 - d[4] * 36;
  Lu[5] = ro + d58 - d[5] * 36;
  Lu[7] = ro - d58 - d[7] * 36;
  Lu[6] = ro + d67 - d[6] * 36;
  Lu[8] = ro - d67 - d[8] * 36;

  // quadratic part: U = (omega/2) / rho with one Newton step on a float reciprocal
  const float q0 = rcp(R.hi);
  const float u0 = df::mul_(c.om2.hi, q0);
  const df::F2 p = df::mulf(R, u0);
  const float eh = df::add_(df::sub_(c.om2.hi, p.hi), df::sub_(c.om2.lo, p.lo));
  const df::F2 U = df::fast_two_sum(u0, df::mul_(eh, q0));
  const df::F2 UX = df::mul(X, U), UY = df::mul(Y, U);
  const int64_t A = f2_to_q(df::mul(X, UX));   // (omega/2) jx^2 / rho
  const int64_t B = f2_to_q(df::mul(Y, UY));   // (omega/2) jy^2 / rho
  const int64_t P2 = f2_to_q(df::mul(X, UY));  // (omega/2) jx jy / rho
  // Q6 = (A + B) / 3 = omega |j|^2 / (6 rho)
  const int64_t Q6 = (int64_t)mulq((uint64_t)(A + B), 0x55555555u, 0x55555555u);
  const int64_t N5 = (Q6 + P2) >> 1;
  // N_i (omega w_i (4.5 (c_i.j)^2 - 1.5 |j|^2) / rho) less the M/4 offset of T_i;
  // N5 + N6 = Q6 exactly, so the halving moves no mass
  const int64_t N0 = -(Q6 << 2) - c.m4;
  const int64_t N1 = A - Q6 - c.m4;
  const int64_t N2 = B - Q6 - c.m4;
  const int64_t N6 = Q6 - N5 - c.m4;
  const int64_t N5o = N5 - c.m4;
  const int64_t N[9] = {N0, N1, N2, N1, N2, N5o, N6, N5o, N6};
#pragma unroll
  for (int i = 0; i < 9; ++i) d[i] += (int64_t)mulq((uint64_t)Lu[i], c.mh, c.ml) + N[i];
  return true;
}

}  // namespace fx
}  // namespace lbm
