// lbm_core.cuh -- device building blocks of the D2Q9 BGK hot path (sm_103a).
//
// The arithmetic follows src/lattice_boltzmann_method.py of the reference:
//   rho  = sum_i f_i                                    (:93-105)
//   u    = (sum_i c_i f_i) / rho, 0 where rho == 0      (:108-137)
//   feq  = w rho (1 + 3 c.u + 9/2 (c.u)^2 - 3/2 |u|^2)  (:162-188)
//   fpre = f + (feq - f) omega                          (:215)
// in two forms: "exact" reproduces NumPy's float64 operation order with no
// FMA contraction (pairwise 9-term sum, |u|^2 = sqrt(ux^2+uy^2)^2, IEEE
// division), "fast" regroups the same formula around FMAs and one reciprocal.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lbm_gb300.h"
#include "lbm_fx.cuh"

namespace lbm {

// D2Q9 velocity set, opposite map and weights (lattice_boltzmann_method.py:14-52).
__host__ __device__ constexpr int cx(int i) { return (i == 1 || i == 5 || i == 8) ? 1 : ((i == 3 || i == 6 || i == 7) ? -1 : 0); }
__host__ __device__ constexpr int cy(int i) { return (i == 2 || i == 5 || i == 6) ? 1 : ((i == 4 || i == 7 || i == 8) ? -1 : 0); }
__host__ __device__ constexpr int opp(int i) { return i == 0 ? 0 : (i <= 4 ? ((i + 1) % 4) + 1 : ((i - 3) % 4) + 5); }
__host__ __device__ constexpr double wd(int i) { return i == 0 ? 4.0 / 9.0 : (i <= 4 ? 1.0 / 9.0 : 1.0 / 36.0); }
__host__ __device__ constexpr float wf(int i) { return i == 0 ? 4.0f / 9.0f : (i <= 4 ? 1.0f / 9.0f : 1.0f / 36.0f); }
static_assert(opp(1) == 3 && opp(2) == 4 && opp(3) == 1 && opp(4) == 2, "opp");
static_assert(opp(5) == 7 && opp(6) == 8 && opp(7) == 5 && opp(8) == 6, "opp");

// outlet directions (boundary_conditions.py:265) and their slot in aux[3][ny]
__host__ __device__ constexpr int outlet_slot(int i) { return i == 3 ? 0 : (i == 6 ? 1 : (i == 7 ? 2 : -1)); }

// ---------------------------------------------------------------------------
// storage of the resident populations
// ---------------------------------------------------------------------------
template <int S> struct Store;
template <> struct Store<LBM_STORE_F64> {
  using T = double;
  using R = double;
  __device__ static R ld(const T* p, int) { return __ldg(p); }
  __device__ static void st(T* p, R v, int) { *p = v; }
  __device__ static R to_r(T t, int) { return t; }
  __device__ static T from_r(R v, int) { return v; }
  using A = R;  // outlet memory: full populations in the working type
  __device__ static A to_aux(R v, int) { return v; }
  __device__ static R from_aux(A a, int) { return a; }
  static constexpr bool kShifted = false;
};
template <> struct Store<LBM_STORE_F32> {
  using T = float;
  using R = float;
  __device__ static R ld(const T* p, int) { return __ldg(p); }
  __device__ static void st(T* p, R v, int) { *p = v; }
  __device__ static R to_r(T t, int) { return t; }
  __device__ static T from_r(R v, int) { return v; }
  using A = R;  // outlet memory: full populations in the working type
  __device__ static A to_aux(R v, int) { return v; }
  __device__ static R from_aux(A a, int) { return a; }
  static constexpr bool kShifted = false;
};
// fixed-point storage: round((f_i - w_i) 2^56) in 64 bits (lbm_fx.cuh); the
// generic kernels work on its float64 value, the vectorised one on the integers.
// Its outlet memory keeps the stored integers too (the copy stays exact).
template <> struct Store<LBM_STORE_FX64> {
  using T = long long;
  using R = double;
  using A = long long;
  __device__ static R ld(const T* p, int i) { return fx::from_fx(__ldg(p), wd(i)); }
  __device__ static void st(T* p, R v, int i) { *p = fx::to_fx(v, wd(i)); }
  __device__ static R to_r(T t, int i) { return fx::from_fx(t, wd(i)); }
  __device__ static T from_r(R v, int i) { return fx::to_fx(v, wd(i)); }
  __device__ static A to_aux(R v, int i) { return fx::to_fx(v, wd(i)); }
  __device__ static R from_aux(A a, int i) { return fx::from_fx(a, wd(i)); }
  static constexpr bool kShifted = false;
};
// shifted storage: the deviation f_i - w_i is kept in 16 bits.  binary16 keeps
// 1024 (f_i - w_i): deviations down to 6e-8 then stay in the normal range,
// where stochastic rounding is adding random bits below the kept 10 mantissa
// bits of the float32 value and truncating.
template <> struct Store<LBM_STORE_F16S> {
  using T = __half;
  using R = float;
  static constexpr float kScale = 1024.0f, kInv = 1.0f / 1024.0f;
  __device__ static R ld(const T* p, int i) { return fmaf(__half2float(__ldg(p)), kInv, wf(i)); }
  __device__ static void st(T* p, R v, int i) { *p = __float2half_rn((v - wf(i)) * kScale); }
  __device__ static R to_r(T t, int i) { return fmaf(__half2float(t), kInv, wf(i)); }
  __device__ static T from_r(R v, int i) { return __float2half_rn((v - wf(i)) * kScale); }
  using A = R;  // outlet memory: full populations in the working type
  __device__ static A to_aux(R v, int) { return v; }
  __device__ static R from_aux(A a, int) { return a; }
  static constexpr bool kShifted = true;
  // the vectorised kernel works on the stored, scaled deviation D = 1024 (f_i - w_i)
  static constexpr float kDev = kScale;
  __device__ static R dev(T t) { return __half2float(t); }
  __device__ static R ld_dev(const T* p) { return __half2float(__ldg(p)); }
  __device__ static T dev_rn(R d) { return __float2half_rn(d); }
  // stochastic rounding: the top 13 bits of r, added below the 10 mantissa bits
  // binary16 keeps, then truncation
  __device__ static T dev_sr(R d, uint32_t r) {
    return __float2half_rz(__uint_as_float(__float_as_uint(d) + (r >> 19)));
  }
};
template <> struct Store<LBM_STORE_BF16S> {
  using T = __nv_bfloat16;
  using R = float;
  __device__ static R ld(const T* p, int i) { return wf(i) + __bfloat162float(__ldg(p)); }
  __device__ static void st(T* p, R v, int i) { *p = __float2bfloat16_rn(v - wf(i)); }
  __device__ static R to_r(T t, int i) { return wf(i) + __bfloat162float(t); }
  __device__ static T from_r(R v, int i) { return __float2bfloat16_rn(v - wf(i)); }
  using A = R;  // outlet memory: full populations in the working type
  __device__ static A to_aux(R v, int) { return v; }
  __device__ static R from_aux(A a, int) { return a; }
  static constexpr bool kShifted = true;
  static constexpr float kDev = 1.0f;  // working deviation: f_i - w_i
  __device__ static R dev(T t) { return __bfloat162float(t); }
  __device__ static R ld_dev(const T* p) { return __bfloat162float(__ldg(p)); }
  __device__ static T dev_rn(R d) { return __float2bfloat16_rn(d); }
  // stochastic rounding: the top 16 bits of r, added below the 16 bits bfloat16
  // keeps, then truncation
  __device__ static T dev_sr(R d, uint32_t r) {
    const uint32_t u = __float_as_uint(d) + (r >> 16);
    return __ushort_as_bfloat16((unsigned short)(u >> 16));
  }
};

// 32-bit integer hash (C. Wellons' "lowbias32" constants) for the random bits
// of the stochastic rounding
__host__ __device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x21f0aaadu;
  x ^= x >> 15;
  x *= 0x735a2d97u;
  x ^= x >> 15;
  return x;
}

// short integer mixer (xor-shift, multiply, xor-shift) for the per-node seed of
// the stochastic rounding; a multiply-add step per direction follows it
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  return x;
}

// N contiguous elements, N * sizeof(T) bytes aligned to that size (up to 16)
template <typename T, int N>
__device__ __forceinline__ void ld_vec(const T* p, T out[N]) {
  constexpr int B = N * (int)sizeof(T);
  if constexpr (B % 16 == 0) {
#pragma unroll
    for (int j = 0; j < B / 16; ++j) {
      const uint4 t = __ldg(reinterpret_cast<const uint4*>(p) + j);
      memcpy(&out[j * (16 / sizeof(T))], &t, 16);
    }
  } else if constexpr (B == 8) {
    const uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
    memcpy(out, &t, 8);
  } else if constexpr (B == 4) {
    const unsigned t = __ldg(reinterpret_cast<const unsigned*>(p));
    memcpy(out, &t, 4);
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) out[j] = p[j];
  }
}
template <typename T, int N>
__device__ __forceinline__ void st_vec(T* p, const T in[N]) {
  constexpr int B = N * (int)sizeof(T);
  if constexpr (B % 16 == 0) {
#pragma unroll
    for (int j = 0; j < B / 16; ++j) {
      uint4 t;
      memcpy(&t, &in[j * (16 / sizeof(T))], 16);
      reinterpret_cast<uint4*>(p)[j] = t;
    }
  } else if constexpr (B == 8) {
    uint2 t;
    memcpy(&t, in, 8);
    *reinterpret_cast<uint2*>(p) = t;
  } else if constexpr (B == 4) {
    unsigned t;
    memcpy(&t, in, 4);
    *reinterpret_cast<unsigned*>(p) = t;
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) p[j] = in[j];
  }
}

// ---------------------------------------------------------------------------
// moments
// ---------------------------------------------------------------------------
// NumPy's float64 reduction of 9 contiguous terms is pairwise:
// ((f0+f1)+(f2+f3)) + ((f4+f5)+(f6+f7)), then + f8.
template <typename R>
__device__ __forceinline__ R density9(const R f[9]) {
  return (((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7]))) + f[8];
}
// sum f_i and j = sum c_i f_i with shared partial sums (14 additions instead of 18)
template <typename R>
__device__ __forceinline__ void moments9(const R f[9], R& sum, R& jx, R& jy) {
  const R a = (f[1] + f[5]) + f[8], b = (f[3] + f[6]) + f[7];
  const R c = (f[2] + f[5]) + f[6], e = (f[4] + f[7]) + f[8];
  jx = a - b;
  jy = c - e;
  sum = ((f[0] + f[2]) + (a + b)) + f[4];
}
__device__ __forceinline__ double density9_exact(const double f[9]) {
  double a = __dadd_rn(__dadd_rn(f[0], f[1]), __dadd_rn(f[2], f[3]));
  double b = __dadd_rn(__dadd_rn(f[4], f[5]), __dadd_rn(f[6], f[7]));
  return __dadd_rn(__dadd_rn(a, b), f[8]);
}

__device__ __forceinline__ void velocity_exact(const double f[9], double rho, double& ux, double& uy) {
  double jx = __dsub_rn(__dadd_rn(__dadd_rn(f[1], f[5]), f[8]), __dadd_rn(__dadd_rn(f[3], f[6]), f[7]));
  double jy = __dsub_rn(__dadd_rn(__dadd_rn(f[2], f[5]), f[6]), __dadd_rn(__dadd_rn(f[4], f[7]), f[8]));
  ux = rho != 0.0 ? __ddiv_rn(jx, rho) : 0.0;
  uy = rho != 0.0 ? __ddiv_rn(jy, rho) : 0.0;
}

// Reciprocal by Newton-Raphson iteration r <- r + r (1 - a r) from a
// single-precision seed; two iterations take the 2^-23 seed error below the
// float64 rounding error.  Arguments outside the float range fall back to
// the IEEE division.
__device__ __forceinline__ double rcp_nr(double a) {
  float af = __double2float_rn(a);
  if (!(fabsf(af) > 1e-30f && fabsf(af) < 1e30f)) return 1.0 / a;
  double r = (double)__frcp_rn(af);
  double e = fma(-a, r, 1.0);
  r = fma(r, e, r);
  e = fma(-a, r, 1.0);
  return fma(r, e, r);
}
__device__ __forceinline__ float rcp_nr(float a) { return __frcp_rn(a); }

template <typename R>
__device__ __forceinline__ void velocity_fast(const R f[9], R rho, R& ux, R& uy) {
  R jx = ((f[1] + f[5]) + f[8]) - ((f[3] + f[6]) + f[7]);
  R jy = ((f[2] + f[5]) + f[6]) - ((f[4] + f[7]) + f[8]);
  R inv = rho != R(0) ? rcp_nr(rho) : R(0);
  ux = jx * inv;
  uy = jy * inv;
}

// ---------------------------------------------------------------------------
// equilibrium and collision
// ---------------------------------------------------------------------------
// c_i.u exactly as the matmul u @ c.T rounds it (one rounding for diagonals)
__device__ __forceinline__ void cu9_exact(double ux, double uy, double cu[9]) {
  cu[0] = 0.0;
  cu[1] = ux;
  cu[2] = uy;
  cu[3] = -ux;
  cu[4] = -uy;
  cu[5] = __dadd_rn(ux, uy);
  cu[6] = __dadd_rn(-ux, uy);
  cu[7] = -cu[5];
  cu[8] = __dadd_rn(ux, -uy);
}

// bracket(i) = ((1 + 3 cu) + 4.5 cu^2) - 1.5 |u|^2, |u|^2 = sqrt(ux^2 + uy^2)^2
__device__ __forceinline__ void bracket9_exact(double ux, double uy, double br[9]) {
  double nrm = __dsqrt_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)));
  double usq15 = __dmul_rn(1.5, __dmul_rn(nrm, nrm));
  double cu[9];
  cu9_exact(ux, uy, cu);
  br[0] = __dsub_rn(1.0, usq15);
#pragma unroll
  for (int i = 1; i < 9; ++i)
    br[i] = __dsub_rn(__dadd_rn(__dadd_rn(1.0, __dmul_rn(3.0, cu[i])), __dmul_rn(4.5, __dmul_rn(cu[i], cu[i]))), usq15);
}

__device__ __forceinline__ void collide_exact(double f[9], double rho, double ux, double uy, double omega,
                                              double feq[9], double br[9]) {
  bracket9_exact(ux, uy, br);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    feq[i] = __dmul_rn(__dmul_rn(wd(i), rho), br[i]);
    f[i] = __dadd_rn(f[i], __dmul_rn(__dsub_rn(feq[i], f[i]), omega));
  }
}

template <typename R> __device__ constexpr R wr(int i);
template <> __device__ constexpr double wr<double>(int i) { return wd(i); }
template <> __device__ constexpr float wr<float>(int i) { return wf(i); }

// Fast form: fpre_i = (1-omega) f_i + omega w_i rho (B + 4.5 cu^2 + 3 cu),
// B = 1 - 1.5 |u|^2; opposite directions share the even part.
template <typename R>
__device__ __forceinline__ void collide_fast(R f[9], R rho, R ux, R uy, R omega) {
  const R om1 = R(1) - omega;
  const R usq = fma(ux, ux, uy * uy);
  const R B = fma(R(-1.5), usq, R(1));
  const R orho = omega * rho;
  const R W0 = orho * wr<R>(0), W1 = orho * wr<R>(1), W5 = orho * wr<R>(5);
  const R V1 = R(3) * W1, V5 = R(3) * W5;
  f[0] = fma(om1, f[0], W0 * B);
  const R d58 = ux + uy, d67 = uy - ux;
#define LBM_PAIR(I, J, V, W, VV)                       \
  {                                                   \
    const R t = fma(R(4.5) * (V), (V), B);            \
    const R s = (W) * t;                              \
    const R m = (VV) * (V);                           \
    f[I] = fma(om1, f[I], s + m);                     \
    f[J] = fma(om1, f[J], s - m);                     \
  }
  LBM_PAIR(1, 3, ux, W1, V1)
  LBM_PAIR(2, 4, uy, W1, V1)
  LBM_PAIR(5, 7, d58, W5, V5)
  LBM_PAIR(6, 8, d67, W5, V5)
#undef LBM_PAIR
}

// The same collision on scaled deviations d_i = s (f_i - w_i) (float32): with
// sd = s (rho - 1) = sum d_i and srho = s rho = s + sd,
// d_i' = (1 - omega) d_i + omega w_i (sd + srho (4.5 cu^2 +- 3 cu - 1.5 |u|^2)).
__device__ __forceinline__ void collide_dev(float d[9], float drho, float rho, float ux, float uy, float omega) {
  const float om1 = 1.0f - omega;
  const float Bd = -1.5f * fmaf(ux, ux, uy * uy);
  const float orho = omega * rho, odr = omega * drho;
  const float W0 = orho * wf(0), W1 = orho * wf(1), W5 = orho * wf(5);
  const float D0 = odr * wf(0), D1 = odr * wf(1), D5 = odr * wf(5);
  const float V1 = 3.0f * W1, V5 = 3.0f * W5;
  d[0] = fmaf(om1, d[0], fmaf(W0, Bd, D0));
  const float d58 = ux + uy, d67 = uy - ux;
#define LBM_DPAIR(I, J, V, W, D, VV)                 \
  {                                                 \
    const float t = fmaf(4.5f * (V), (V), Bd);      \
    const float s = fmaf((W), t, (D));              \
    const float m = (VV) * (V);                     \
    d[I] = fmaf(om1, d[I], s + m);                  \
    d[J] = fmaf(om1, d[J], s - m);                  \
  }
  LBM_DPAIR(1, 3, ux, W1, D1, V1)
  LBM_DPAIR(2, 4, uy, W1, D1, V1)
  LBM_DPAIR(5, 7, d58, W5, D5, V5)
  LBM_DPAIR(6, 8, d67, W5, D5, V5)
#undef LBM_DPAIR
}

// ---- two nodes per instruction: packed float32 pairs (sm_100 family) --------
__device__ __forceinline__ float2 f2c(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2c(-1.0f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ void moments9x2(const float2 f[9], float2& sum, float2& jx, float2& jy) {
  const float2 a = add2(add2(f[1], f[5]), f[8]), b = add2(add2(f[3], f[6]), f[7]);
  const float2 c = add2(add2(f[2], f[5]), f[6]), e = add2(add2(f[4], f[7]), f[8]);
  jx = sub2(a, b);
  jy = sub2(c, e);
  sum = add2(add2(add2(f[0], f[2]), add2(a, b)), f[4]);
}

// collide_dev on two nodes at once
__device__ __forceinline__ void collide_dev2(float2 d[9], float2 drho, float2 rho, float2 ux, float2 uy, float omega) {
  const float2 om1 = f2c(1.0f - omega), om = f2c(omega);
  const float2 Bd = mul2(f2c(-1.5f), fma2(ux, ux, mul2(uy, uy)));
  const float2 orho = mul2(om, rho), odr = mul2(om, drho);
  const float2 W0 = mul2(orho, f2c(wf(0))), W1 = mul2(orho, f2c(wf(1))), W5 = mul2(orho, f2c(wf(5)));
  const float2 D0 = mul2(odr, f2c(wf(0))), D1 = mul2(odr, f2c(wf(1))), D5 = mul2(odr, f2c(wf(5)));
  const float2 V1 = mul2(f2c(3.0f), W1), V5 = mul2(f2c(3.0f), W5);
  d[0] = fma2(om1, d[0], fma2(W0, Bd, D0));
  const float2 d58 = add2(ux, uy), d67 = sub2(uy, ux);
#define LBM_DPAIR2(I, J, V, W, D, VV)                  \
  {                                                   \
    const float2 t = fma2(mul2(f2c(4.5f), (V)), (V), Bd); \
    const float2 s = fma2((W), t, (D));               \
    const float2 m = mul2((VV), (V));                 \
    d[I] = fma2(om1, d[I], add2(s, m));               \
    d[J] = fma2(om1, d[J], sub2(s, m));               \
  }
  LBM_DPAIR2(1, 3, ux, W1, D1, V1)
  LBM_DPAIR2(2, 4, uy, W1, D1, V1)
  LBM_DPAIR2(5, 7, d58, W5, D5, V5)
  LBM_DPAIR2(6, 8, d67, W5, D5, V5)
#undef LBM_DPAIR2
}

// Constants of the reference-shifted 16-bit storages in the working units
// (scale s): stored numbers D_i = d_i - sig_i, sig_i = s (c_i - w_i) with c_i
// the equilibrium at the reference velocity.  The collision works on D
// directly: D_i' = (1 - omega) D_i + omega (E_i - sig_i), E the deviation
// equilibrium of the moments of d = D + sig.  -omega sig_i is split per
// direction pair (1,3), (2,4), (5,7), (6,8) into an even part qe and an odd
// part qo (-omega sig of the first direction = qe + qo, of the second
// qe - qo), q0 for direction 0; sig holds the values these constants imply,
// S = sum_i sig_i, oS = omega S, (sx, sy) = sum_i c_i sig_i.
struct ShiftK {
  float sig[9];
  float q0, qe[4], qo[4];
  float S, oS, sx, sy;
};

// collide_dev2 on stored numbers of a reference-shifted storage: sum, jx, jy
// are the moments of D with (sx, sy) already added to jx, jy; the mass
// offset S enters through oS
__device__ __forceinline__ void collide_dev2_ref(float2 d[9], float2 drho, float2 rho, float2 ux, float2 uy,
                                                 float omega, const ShiftK& h) {
  const float2 om1 = f2c(1.0f - omega), om = f2c(omega);
  const float2 Bd = mul2(f2c(-1.5f), fma2(ux, ux, mul2(uy, uy)));
  const float2 orho = mul2(om, rho), odr = fma2(om, drho, f2c(h.oS));
  const float2 W0 = mul2(orho, f2c(wf(0))), W1 = mul2(orho, f2c(wf(1))), W5 = mul2(orho, f2c(wf(5)));
  const float2 V1 = mul2(f2c(3.0f), W1), V5 = mul2(f2c(3.0f), W5);
  d[0] = fma2(om1, d[0], fma2(W0, Bd, fma2(odr, f2c(wf(0)), f2c(h.q0))));
  const float2 d58 = add2(ux, uy), d67 = sub2(uy, ux);
#define LBM_RPAIR2(I, J, V, W, WI, VV, P)                             \
  {                                                                   \
    const float2 t = fma2(mul2(f2c(4.5f), (V)), (V), Bd);             \
    const float2 s = fma2((W), t, fma2(odr, f2c(wf(WI)), f2c(h.qe[P]))); \
    const float2 m = fma2((VV), (V), f2c(h.qo[P]));                   \
    d[I] = fma2(om1, d[I], add2(s, m));                               \
    d[J] = fma2(om1, d[J], sub2(s, m));                               \
  }
  LBM_RPAIR2(1, 3, ux, W1, 1, V1, 0)
  LBM_RPAIR2(2, 4, uy, W1, 1, V1, 1)
  LBM_RPAIR2(5, 7, d58, W5, 5, V5, 2)
  LBM_RPAIR2(6, 8, d67, W5, 5, V5, 3)
#undef LBM_RPAIR2
}

// equilibrium with FMAs (used where the fast path needs feq itself)
template <typename R>
__device__ __forceinline__ void bracket9_fast(R ux, R uy, R br[9]) {
  const R B = fma(R(-1.5), fma(ux, ux, uy * uy), R(1));
  const R cu[9] = {R(0), ux, uy, -ux, -uy, ux + uy, uy - ux, -(ux + uy), ux - uy};
#pragma unroll
  for (int i = 0; i < 9; ++i) br[i] = fma(cu[i], fma(R(4.5), cu[i], R(3)), B);
}

}  // namespace lbm
