// lbm_ops.cu -- the reference's component functions as standalone kernels on
// the reference layout f[nx][ny][9] (float64, NumPy operation order), used by
// the drop-in functions and by the unfused step that runs arbitrary Python
// boundary or halo callables between kernels.
#include <cstring>

#include "lbm_core.cuh"
#include "lbm_host.h"

namespace lbm {

constexpr int kThreads = 256;

static inline unsigned blocks_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

__global__ void density_kernel(const double* __restrict__ f, double* __restrict__ rho, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double v[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] = f[k * 9 + i];
  rho[k] = density9_exact(v);
}

__global__ void velocity_kernel(const double* __restrict__ rho, const double* __restrict__ f,
                                double* __restrict__ u, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double v[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] = f[k * 9 + i];
  double ux, uy;
  velocity_exact(v, rho[k], ux, uy);
  u[2 * k] = ux;
  u[2 * k + 1] = uy;
}

__global__ void equilibrium_kernel(const double* __restrict__ rho, const double* __restrict__ u,
                                   double* __restrict__ feq, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double br[9];
  bracket9_exact(u[2 * k], u[2 * k + 1], br);
  const double r = rho[k];
#pragma unroll
  for (int i = 0; i < 9; ++i) feq[k * 9 + i] = __dmul_rn(__dmul_rn(wd(i), r), br[i]);
}

__global__ void streaming_kernel(const double* __restrict__ f, double* __restrict__ out, int nx, int ny) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)nx * ny) return;
  const int x = (int)(k / ny), y = (int)(k % ny);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    int xs = x - cx(i), ys = y - cy(i);
    xs = xs < 0 ? xs + nx : (xs >= nx ? xs - nx : xs);
    ys = ys < 0 ? ys + ny : (ys >= ny ? ys - ny : ys);
    out[k * 9 + i] = f[((int64_t)xs * ny + ys) * 9 + i];
  }
}

template <bool EXACT>
__global__ void collide_kernel(const double* __restrict__ f, const double* __restrict__ rho,
                               const double* __restrict__ u, double omega, double* __restrict__ out, int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double v[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] = f[k * 9 + i];
  if (EXACT) {
    double feq[9], br[9];
    collide_exact(v, rho[k], u[2 * k], u[2 * k + 1], omega, feq, br);
  } else {
    collide_fast(v, rho[k], u[2 * k], u[2 * k + 1], omega);
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) out[k * 9 + i] = v[i];
}

struct BcTables {
  double kconst[LBM_MAX_SETS][9];
  double cconst[LBM_MAX_SETS][9];
};

__global__ void apply_boundary_kernel(const uint32_t* __restrict__ bcmask, const uint32_t* __restrict__ desc,
                                      int nx, int ny, const __grid_constant__ BcTables t,
                                      const double* __restrict__ f_pre, const double* __restrict__ f_prev,
                                      double* __restrict__ f_post) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= nx || y >= ny) return;
  const int words = (nx + 31) / 32;
  if (!((bcmask[(int64_t)y * words + (x >> 5)] >> (x & 31)) & 1u)) return;
  const uint32_t d = desc[(int64_t)y * nx + x];
  const int ks = (d >> LBM_DESC_KSET_SHIFT) & 15, cs = (d >> LBM_DESC_CSET_SHIFT) & 15;
  const int64_t node = ((int64_t)x * ny + y) * 9;
  const int64_t left = ((int64_t)(x == 0 ? nx - 1 : x - 1) * ny + y) * 9;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const uint32_t s = (d >> (2 * i)) & 3u;
    if (s == LBM_SRC_BOUNCE)
      f_post[node + i] = __dsub_rn(f_pre[node + opp(i)], t.kconst[ks][i]);
    else if (s == LBM_SRC_CONST)
      f_post[node + i] = t.cconst[cs][i];
    else if (s == LBM_SRC_OUTLET && f_prev != nullptr)
      f_post[node + i] = f_prev[left + i];
  }
}

// periodic_with_pressure_variations' closure (boundary_conditions.py:320-346)
__global__ void pressure_kernel(double* __restrict__ f_pre, const double* __restrict__ rho,
                                const double* __restrict__ u, int nx, int ny, uint32_t pin, uint32_t pout,
                                double rho_in, double rho_out) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  const int64_t a = (int64_t)(nx - 2) * ny + y, b = (int64_t)1 * ny + y;
  double fa[9], fb[9], bra[9], brb[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    fa[i] = f_pre[a * 9 + i];
    fb[i] = f_pre[b * 9 + i];
  }
  bracket9_exact(u[2 * a], u[2 * a + 1], bra);
  bracket9_exact(u[2 * b], u[2 * b + 1], brb);
  const int64_t c0 = (int64_t)y * 9, c1 = ((int64_t)(nx - 1) * ny + y) * 9;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    if ((pin >> i) & 1u) {
      const double feq = __dmul_rn(__dmul_rn(wd(i), rho[a]), bra[i]);
      f_pre[c0 + i] = __dadd_rn(__dmul_rn(__dmul_rn(wd(i), rho_in), bra[i]), __dsub_rn(fa[i], feq));
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    if ((pout >> i) & 1u) {
      const double feq = __dmul_rn(__dmul_rn(wd(i), rho[b]), brb[i]);
      f_pre[c1 + i] = __dadd_rn(__dmul_rn(__dmul_rn(wd(i), rho_out), brb[i]), __dsub_rn(fb[i], feq));
    }
  }
}

// single-rank periodic ghost exchange: ghost (x, y) <- (mx(x), my(y)) with
// mx(0) = nx-2, mx(nx-1) = 1 (x exchange first, then rows including the ghost columns)
__global__ void halo_kernel(double* __restrict__ f, int nx, int ny) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)nx * ny) return;
  const int x = (int)(k / ny), y = (int)(k % ny);
  const bool gx = x == 0 || x == nx - 1, gy = y == 0 || y == ny - 1;
  if (!gx && !gy) return;
  const int sx = x == 0 ? nx - 2 : (x == nx - 1 ? 1 : x);
  const int sy = y == 0 ? ny - 2 : (y == ny - 1 ? 1 : y);
  const int64_t s = ((int64_t)sx * ny + sy) * 9;
#pragma unroll
  for (int i = 0; i < 9; ++i) f[k * 9 + i] = f[s + i];
}

static int done(const char* what) {
  count_launch();
  return check_launch(what);
}

}  // namespace lbm

using namespace lbm;

extern "C" {

int lbm_density_f64(const double* f, double* rho, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (f == nullptr || rho == nullptr))) return set_error(LBM_ERR_ARG, "bad density arguments");
  if (n == 0) return LBM_OK;
  density_kernel<<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(f, rho, n);
  return done("density_kernel");
}

int lbm_velocity_f64(const double* rho, const double* f, double* u, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (f == nullptr || rho == nullptr || u == nullptr)))
    return set_error(LBM_ERR_ARG, "bad velocity arguments");
  if (n == 0) return LBM_OK;
  velocity_kernel<<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(rho, f, u, n);
  return done("velocity_kernel");
}

int lbm_equilibrium_f64(const double* rho, const double* u, double* feq, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (feq == nullptr || rho == nullptr || u == nullptr)))
    return set_error(LBM_ERR_ARG, "bad equilibrium arguments");
  if (n == 0) return LBM_OK;
  equilibrium_kernel<<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(rho, u, feq, n);
  return done("equilibrium_kernel");
}

int lbm_streaming_f64(const double* f, double* out, int32_t nx, int32_t ny, void* stream) {
  if (nx < 1 || ny < 1 || f == nullptr || out == nullptr || f == out)
    return set_error(LBM_ERR_ARG, "bad streaming arguments (out of place, nx, ny >= 1)");
  const int64_t n = (int64_t)nx * ny;
  streaming_kernel<<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(f, out, nx, ny);
  return done("streaming_kernel");
}

int lbm_collide_f64(const double* f, const double* rho, const double* u, double omega, double* out, int64_t n,
                    int32_t flags, void* stream) {
  if (!(omega > 0.0 && omega < 2.0)) return set_error(LBM_ERR_OMEGA, "omega must lie in (0, 2)");
  if (n < 0 || (n > 0 && (f == nullptr || rho == nullptr || u == nullptr || out == nullptr)))
    return set_error(LBM_ERR_ARG, "bad collide arguments");
  if (n == 0) return LBM_OK;
  if (flags & LBM_FLAG_EXACT)
    collide_kernel<true><<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(f, rho, u, omega, out, n);
  else
    collide_kernel<false><<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(f, rho, u, omega, out, n);
  return done("collide_kernel");
}

int lbm_apply_boundary_f64(const lbm_geometry* g, const double* f_pre, const double* f_prev, double* f_post,
                           void* stream) {
  if (g == nullptr || g->nx < 1 || g->ny < 1 || f_pre == nullptr || f_post == nullptr)
    return set_error(LBM_ERR_ARG, "bad boundary arguments");
  if (g->bcmask == nullptr) return LBM_OK;
  if (g->desc == nullptr) return set_error(LBM_ERR_ARG, "bcmask given without desc");
  if (g->outlet && (f_prev == nullptr || g->nx < 2)) return set_error(LBM_ERR_ARG, "the outlet needs f_prev and nx >= 2");
  BcTables t;
  std::memcpy(t.kconst, g->kconst, sizeof(t.kconst));
  std::memcpy(t.cconst, g->cconst, sizeof(t.cconst));
  dim3 grid((g->nx + 127) / 128, g->ny);
  apply_boundary_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(g->bcmask, g->desc, g->nx, g->ny, t, f_pre, f_prev, f_post);
  return done("apply_boundary_kernel");
}

int lbm_pressure_prestream_f64(const lbm_geometry* g, double* f_pre, const double* rho, const double* u,
                               void* stream) {
  if (g == nullptr || g->nx < 2 || g->ny < 1 || f_pre == nullptr || rho == nullptr || u == nullptr)
    return set_error(LBM_ERR_ARG, "bad pressure arguments (nx >= 2)");
  if (!g->pressure) return LBM_OK;
  pressure_kernel<<<blocks_for(g->ny), kThreads, 0, (cudaStream_t)stream>>>(
      f_pre, rho, u, g->nx, g->ny, g->pressure_in_dirs & 0x1FFu, g->pressure_out_dirs & 0x1FFu, g->rho_in, g->rho_out);
  return done("pressure_kernel");
}

int lbm_halo_fill_f64(double* f, int32_t nx, int32_t ny, void* stream) {
  if (f == nullptr || nx < 3 || ny < 3) return set_error(LBM_ERR_ARG, "bad halo arguments (padded sizes >= 3)");
  const int64_t n = (int64_t)nx * ny;
  halo_kernel<<<blocks_for(n), kThreads, 0, (cudaStream_t)stream>>>(f, nx, ny);
  return done("halo_kernel");
}

}  // extern "C"
