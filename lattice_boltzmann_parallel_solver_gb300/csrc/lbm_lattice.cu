// lbm_lattice.cu -- fused pull-scheme stream + boundary + collide kernel and
// the C ABI of the drop-in step and of the resident lattice.
//
// State convention.  The reference's step (lattice_boltzmann_method.py:191-228)
// maps the post-streaming state f_n to f_{n+1} = BC(stream(collide(f_n))).
// The resident state kept here is S_n = collide(f_n) with the pre-streaming
// pressure rewrite already applied (boundary_conditions.py:320-346), so one
// kernel per step reads S_{n-1} once (pull: node x takes S(x - c_i, i)),
// applies the boundary sources, forms the moments of f_n, collides and
// writes S_n once: 72 B read + 72 B written per node in float64.
//   MODE_INIT  : S_0 = collide(f_0) from a reference-layout f_0 (rho,u passed in or recomputed)
//   MODE_FUSED : S_n from S_{n-1}
//   MODE_READ  : f_n = BC(stream(S_{n-1})) and its moments, in the reference layout
// The outlet (boundary_conditions.py:279-280) needs f_{n-1} at column nx-2;
// each kernel stores those three populations in aux[3][ny] for the next one.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lbm_fused.cuh"

namespace lbm {

template <int STORE, bool EXACT, int MODE>
__global__ void __launch_bounds__(256) lattice_kernel(const __grid_constant__ KParams P) {
  using St = Store<STORE>;
  using T = typename St::T;
  using R = typename St::R;
  const int nx = P.g.nx, ny = P.g.ny;
  const int x = P.xb + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= (P.xe > 0 ? P.xe : nx) || y >= ny) return;
  const int64_t r0 = (int64_t)y * P.pitch;
  using A = typename St::A;
  const A* aux_in = static_cast<const A*>(P.aux_in);
  // reference-shifted 16-bit storages: the stored deviation is taken from
  // c_i = w_i + sig_i instead of w_i
  const bool shift = St::kShifted && P.dev_shift;
  auto ld = [&](const T* p, int i) -> R {
    const R v = St::ld(p, i);
    if constexpr (St::kShifted) return shift ? v + (R)P.shf[1].sig[i] : v;
    else return v;
  };
  auto st = [&](T* p, R v, int i) {
    if constexpr (St::kShifted) St::st(p, shift ? v - (R)P.shf[1].sig[i] : v, i);
    else St::st(p, v, i);
  };

  R f[9];
  if (MODE == MODE_INIT) {
    const double* src = P.f_in.p + x * P.f_in.sx + y * P.f_in.sy;
#pragma unroll
    for (int i = 0; i < 9; ++i) f[i] = (R)src[i * P.f_in.sc];
  } else {
    // pull: direction i arrives from node (x - cx_i, y - cy_i), periodic
    const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const int64_t rm = (int64_t)ym * P.pitch, rp = (int64_t)yp * P.pitch;
    const T* pin = static_cast<const T*>(P.pop_in);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const int xs = cx(i) == 1 ? xm : (cx(i) == -1 ? xp : x);
      const int64_t rs = cy(i) == 1 ? rm : (cy(i) == -1 ? rp : r0);
      f[i] = ld(pin + i * P.plane + rs + xs, i);
    }
    if (P.g.bcmask != nullptr) {
      const uint32_t word = __ldg(P.g.bcmask + (int64_t)y * P.g.words + (x >> 5));
      if ((word >> (x & 31)) & 1u) {
        const uint32_t d = __ldg(P.g.desc + (int64_t)y * nx + x);
        const int ks = (d >> LBM_DESC_KSET_SHIFT) & 15, cs = (d >> LBM_DESC_CSET_SHIFT) & 15;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          const uint32_t s = (d >> (2 * i)) & 3u;
          if (s == LBM_SRC_BOUNCE) {
            const R v = ld(pin + opp(i) * P.plane + r0 + x, opp(i));
            if (EXACT)
              f[i] = (R)__dsub_rn((double)v, P.g.kconst[ks][i]);
            else
              f[i] = v - (R)P.g.kconst[ks][i];
          } else if (s == LBM_SRC_CONST) {
            f[i] = (R)P.g.cconst[cs][i];
          } else if (s == LBM_SRC_OUTLET && outlet_slot(i) >= 0 && aux_in != nullptr) {
            f[i] = St::from_aux(aux_in[outlet_slot(i) * ny + y], i);
          }
        }
      }
    }
  }

  // outlet memory: the pre-collision populations 3,6,7 of column nx-2
  if (MODE != MODE_READ && P.aux_out != nullptr && x == nx - 2) {
    A* aux_out = static_cast<A*>(P.aux_out);
    aux_out[0 * ny + y] = St::to_aux(f[3], 3);
    aux_out[1 * ny + y] = St::to_aux(f[6], 6);
    aux_out[2 * ny + y] = St::to_aux(f[7], 7);
  }

  // moments of f_n; the collision of the first step uses the rho,u passed in
  R rho, ux, uy;
  const bool given = MODE == MODE_INIT && P.rho_in.p != nullptr;
  if (given) {
    rho = (R)P.rho_in.p[x * P.rho_in.sx + y * P.rho_in.sy];
    const double* up = P.u_in.p + x * P.u_in.sx + y * P.u_in.sy;
    ux = (R)up[0];
    uy = (R)up[P.u_in.sc];
  } else if (EXACT || MODE == MODE_READ) {
    // read-out moments always follow compute_density / compute_velocity_field exactly
    double fd[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) fd[i] = (double)f[i];
    const double r = density9_exact(fd);
    double a, b;
    velocity_exact(fd, r, a, b);
    rho = (R)r;
    ux = (R)a;
    uy = (R)b;
  } else {
    rho = density9(f);
    velocity_fast(f, rho, ux, uy);
  }

  if (MODE == MODE_FUSED) write_probe(P, x, y, ux, uy);
  if (MODE == MODE_READ || (MODE == MODE_FUSED && P.rho_out.p != nullptr)) {
    if (P.rho_out.p != nullptr) P.rho_out.p[x * P.rho_out.sx + y * P.rho_out.sy] = (double)rho;
    if (P.u_out.p != nullptr) {
      double* up = P.u_out.p + x * P.u_out.sx + y * P.u_out.sy;
      up[0] = (double)ux;
      up[P.u_out.sc] = (double)uy;
    }
  }
  if (MODE == MODE_READ) {
    if (P.f_out.p != nullptr) {
      double* dst = P.f_out.p + x * P.f_out.sx + y * P.f_out.sy;
#pragma unroll
      for (int i = 0; i < 9; ++i) dst[i * P.f_out.sc] = (double)f[i];
    }
    return;
  }

  // collision
  const bool pressure_src = P.g.pressure && (x == nx - 2 || x == 1);
  R pin_v[9], pout_v[9];
  if (EXACT) {
    double fd[9], feq[9], br[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) fd[i] = (double)f[i];
    collide_exact(fd, (double)rho, (double)ux, (double)uy, P.omega, feq, br);
    if (pressure_src) {
      // feq(rho_in, u(nx-2)) + (fpre - feq(rho, u))  at column 0, and the outlet analogue
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        const double neq = __dsub_rn(fd[i], feq[i]);
        pin_v[i] = (R)__dadd_rn(__dmul_rn(__dmul_rn(wd(i), P.g.rho_in), br[i]), neq);
        pout_v[i] = (R)__dadd_rn(__dmul_rn(__dmul_rn(wd(i), P.g.rho_out), br[i]), neq);
      }
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) f[i] = (R)fd[i];
  } else {
    collide_fast(f, rho, ux, uy, (R)P.omega);
    if (pressure_src) {
      R br[9];
      bracket9_fast(ux, uy, br);
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        pin_v[i] = fma(wr<R>(i) * br[i], (R)P.g.rho_in - rho, f[i]);
        pout_v[i] = fma(wr<R>(i) * br[i], (R)P.g.rho_out - rho, f[i]);
      }
    }
  }

  // store S_n; columns 0 / nx-1 take the pressure rewrite from columns nx-2 / 1
  T* pout = static_cast<T*>(P.pop_out);
  const uint32_t skip = P.g.pressure ? ((x == 0 ? P.g.pin : 0u) | (x == nx - 1 ? P.g.pout : 0u)) : 0u;
#pragma unroll
  for (int i = 0; i < 9; ++i)
    if (!((skip >> i) & 1u)) st(pout + i * P.plane + r0 + x, f[i], i);
  if (pressure_src) {
    if (x == nx - 2) {
#pragma unroll
      for (int i = 0; i < 9; ++i)
        if ((P.g.pin >> i) & 1u) st(pout + i * P.plane + r0 + 0, pin_v[i], i);
    }
    if (x == 1) {
#pragma unroll
      for (int i = 0; i < 9; ++i)
        if ((P.g.pout >> i) & 1u) st(pout + i * P.plane + r0 + (nx - 1), pout_v[i], i);
    }
  }
}

// the float32 and 16-bit storages: registers capped so that 1024 threads fit
// on an SM; SHIFT: the reference-shifted 16-bit storages
template <int STORE, int NPT, int THREADS, bool SHIFT, bool HAS_BC, bool HAS_PRESSURE>
__global__ void __launch_bounds__(THREADS, (STORE == LBM_STORE_F16S || STORE == LBM_STORE_BF16S ||
                                            (STORE == LBM_STORE_F32 && NPT <= 2))
                                               ? 1024 / THREADS
                                               : 1)
    fused_v2_kernel(const __grid_constant__ KParams P) {
  fused_v2_body<STORE, NPT, HAS_BC, HAS_PRESSURE, false, SHIFT>(P, P.pop_in, P.pop_out, P.aux_in, P.aux_out,
                                                                (blockIdx.x * THREADS + threadIdx.x) * NPT,
                                                                blockIdx.y, launch_seed(P));
}

// one node per thread: registers capped so that 1024 threads fit on an SM
template <int NPT, int THREADS, bool HAS_BC, bool HAS_PRESSURE>
__global__ void __launch_bounds__(THREADS, NPT == 1 ? 1024 / THREADS : 1) fused_fx_kernel(const __grid_constant__ KParams P) {
  fused_fx_body<NPT, HAS_BC, HAS_PRESSURE>(P, P.pop_in, P.pop_out, P.aux_in, P.aux_out,
                                           (blockIdx.x * THREADS + threadIdx.x) * NPT, blockIdx.y);
}

// The boundary-node pass: after a vectorised step ran its boundary-free body
// over every node, one thread per listed boundary node recomputes that node
// with its sources (the same body at one node per thread, so the arithmetic and
// the random bits are those of the in-step path) and overwrites its outputs.
template <int STORE, int THREADS, bool HAS_PRESSURE, bool SHIFT>
__global__ void __launch_bounds__(THREADS) fixup_v2_kernel(const __grid_constant__ KParams P) {
  const int t = blockIdx.x * THREADS + threadIdx.x;
  if (t >= P.g.n_bcnodes) return;
  const int node = __ldg(P.g.bcnodes + t);
  const int y = node / P.g.nx, x = node - y * P.g.nx;
  if constexpr (STORE == LBM_STORE_FX64)
    fused_fx_body<1, true, HAS_PRESSURE>(P, P.pop_in, P.pop_out, P.aux_in, P.aux_out, x, y);
  else
    fused_v2_body<STORE, 1, true, HAS_PRESSURE, false, SHIFT>(P, P.pop_in, P.pop_out, P.aux_in, P.aux_out, x, y,
                                                              launch_seed(P), true);
}

// adds the steps of a lbm_lattice_run_opts call to its device step counter
__global__ void advance_counter_kernel(int32_t* counter, int32_t n) { *counter += n; }

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static void launch_dims(int nx, int ny, dim3& grid, dim3& block) {
  int bx = nx >= 128 ? 128 : ((nx + 31) / 32) * 32;
  int by = std::max(1, 128 / bx);
  block = dim3(bx, by, 1);
  grid = dim3((nx + bx - 1) / bx, (ny + by - 1) / by, 1);
}

template <int STORE, bool EXACT, int MODE>
static int launch(const KParams& P, cudaStream_t s) {
  dim3 grid, block;
  launch_dims((P.xe > 0 ? P.xe : P.g.nx) - P.xb, P.g.ny, grid, block);
  lattice_kernel<STORE, EXACT, MODE><<<grid, block, 0, s>>>(P);
  count_launch();
  return check_launch("lattice_kernel");
}

template <int MODE>
static int dispatch(int storage, bool exact, const KParams& P, cudaStream_t s) {
  if (exact && storage != LBM_STORE_F64)
    return set_error(LBM_ERR_UNSUPPORTED, "exact arithmetic needs float64 storage");
  switch (storage) {
    case LBM_STORE_F64:
      return exact ? launch<LBM_STORE_F64, true, MODE>(P, s) : launch<LBM_STORE_F64, false, MODE>(P, s);
    case LBM_STORE_F32: return launch<LBM_STORE_F32, false, MODE>(P, s);
    case LBM_STORE_F16S: return launch<LBM_STORE_F16S, false, MODE>(P, s);
    case LBM_STORE_BF16S: return launch<LBM_STORE_BF16S, false, MODE>(P, s);
    case LBM_STORE_FX64: return launch<LBM_STORE_FX64, false, MODE>(P, s);
    case LBM_STORE_F16R:
    case LBM_STORE_BF16R: {
      KParams Q = P;
      Q.dev_shift = 1;
      return storage == LBM_STORE_F16R ? launch<LBM_STORE_F16S, false, MODE>(Q, s)
                                       : launch<LBM_STORE_BF16S, false, MODE>(Q, s);
    }
    default: return set_error(LBM_ERR_ARG, "unknown storage type");
  }
}

constexpr int kV2Threads = 128;

// the four boundary specialisations of one vectorised kernel
#define LBM_LAUNCH_SPECIALISED(KERNEL, ...)                                            \
  do {                                                                                 \
    const bool bc = P.g.bcmask != nullptr, pr = P.g.pressure != 0;                     \
    if (bc && pr)                                                                      \
      KERNEL<__VA_ARGS__, true, true><<<grid, kV2Threads, 0, s>>>(P);                  \
    else if (bc)                                                                       \
      KERNEL<__VA_ARGS__, true, false><<<grid, kV2Threads, 0, s>>>(P);                 \
    else if (pr)                                                                       \
      KERNEL<__VA_ARGS__, false, true><<<grid, kV2Threads, 0, s>>>(P);                 \
    else                                                                               \
      KERNEL<__VA_ARGS__, false, false><<<grid, kV2Threads, 0, s>>>(P);                \
  } while (0)

template <int NPT>
static dim3 v2_grid(const KParams& P) {
  const int chunks = (P.g.nx + NPT - 1) / NPT;
  return dim3((unsigned)((chunks + kV2Threads - 1) / kV2Threads), (unsigned)P.g.ny, 1);
}

template <int STORE, int NPT, bool SHIFT = false>
static int launch_v2(const KParams& P, cudaStream_t s) {
  const dim3 grid = v2_grid<NPT>(P);
  LBM_LAUNCH_SPECIALISED(fused_v2_kernel, STORE, NPT, kV2Threads, SHIFT);
  count_launch();
  return check_launch("fused_v2_kernel");
}

template <int NPT>
static int launch_fx(const KParams& P, cudaStream_t s) {
  const dim3 grid = v2_grid<NPT>(P);
  LBM_LAUNCH_SPECIALISED(fused_fx_kernel, NPT, kV2Threads);
  count_launch();
  return check_launch("fused_fx_kernel");
}

// nodes per thread, measured on the 8192^2 cavity: float32 87.7 GLUPS at 4
// against 83.6 at 2; 16-bit 168 at 4 against 160 at 8 (512 threads per SM)
static int default_npt(int storage) {
  switch (storage) {
    case LBM_STORE_F64: return 2;
    case LBM_STORE_FX64: return 1;
    default: return 4;
  }
}

// the reference-shifted 16-bit storages run at 4 nodes per thread only
static bool ref_shifted(int storage) { return storage == LBM_STORE_F16R || storage == LBM_STORE_BF16R; }

// nodes per thread of the vectorised kernel for this lattice, 0 when it does not apply
static int v2_npt(int storage, int flags, const KParams& P) {
  if ((flags & LBM_FLAG_EXACT) || (flags & LBM_FLAG_GENERIC)) return 0;
  int npt = ref_shifted(storage) ? 0 : (flags >> LBM_FLAG_NPT_SHIFT) & 15;
  if (npt == 0) npt = default_npt(storage);
  if (!v2_fits(P, npt)) return 0;
  return npt;
}

constexpr int kFixupThreads = 128;

template <int STORE, bool SHIFT = false>
static int launch_fixup(const KParams& P, cudaStream_t s) {
  const dim3 grid((unsigned)((P.g.n_bcnodes + kFixupThreads - 1) / kFixupThreads));
  if (P.g.pressure)
    fixup_v2_kernel<STORE, kFixupThreads, true, SHIFT><<<grid, kFixupThreads, 0, s>>>(P);
  else
    fixup_v2_kernel<STORE, kFixupThreads, false, SHIFT><<<grid, kFixupThreads, 0, s>>>(P);
  count_launch();
  return check_launch("fixup_v2_kernel");
}

static int launch_fused_step(int storage, int npt, int flags, const KParams& P, cudaStream_t s);

// One step.  On large lattices whose geometry lists its boundary nodes (at most
// an eighth of the lattice), the vectorised kernel runs without boundary work:
// the body's boundary block then stays out of the hot loop (it costs registers
// under the 64-register cap), and the listed nodes are recomputed by the
// boundary-node pass.  Smaller lattices keep one launch per step, whose fixed
// cost would otherwise outweigh the gain.  Measured on the cavity (split against
// inline GLUPS): the 16-bit storages gain from 2896^2 on (132 against 124) and
// lose below 2048^2 (64 against 85 at 1024^2); the other storages gain only at
// 8192^2 (fx64 46.9 against 46.5) and lose or tie up to 4096^2.
static int64_t split_nodes(int storage) {
  return (storage == LBM_STORE_F16S || storage == LBM_STORE_BF16S || ref_shifted(storage)) ? (int64_t)1 << 22
                                                                                              : (int64_t)1 << 25;
}

static int launch_fused(int storage, int flags, const KParams& P, cudaStream_t s) {
  const int npt = v2_npt(storage, flags, P);
  const int64_t nodes = (int64_t)P.g.nx * P.g.ny;
  // a probe keeps the sources inside the step, so its node is recorded once
  const bool split = npt > 0 && !(flags & LBM_FLAG_BC_INLINE) && P.g.bcmask != nullptr && P.g.n_bcnodes > 0 &&
                     P.probe_buf == nullptr &&
                     (nodes >= split_nodes(storage) || (flags & LBM_FLAG_BC_SPLIT)) &&
                     (int64_t)P.g.n_bcnodes * 8 <= nodes;
  if (!split) return launch_fused_step(storage, npt, flags, P, s);
  KParams Q = P;
  Q.g.bcmask = nullptr;
  if (int e = launch_fused_step(storage, npt, flags, Q, s)) return e;
  switch (storage) {
    case LBM_STORE_F64: return launch_fixup<LBM_STORE_F64>(P, s);
    case LBM_STORE_F32: return launch_fixup<LBM_STORE_F32>(P, s);
    case LBM_STORE_F16S: return launch_fixup<LBM_STORE_F16S>(P, s);
    case LBM_STORE_BF16S: return launch_fixup<LBM_STORE_BF16S>(P, s);
    case LBM_STORE_FX64: return launch_fixup<LBM_STORE_FX64>(P, s);
    case LBM_STORE_F16R: return launch_fixup<LBM_STORE_F16S, true>(P, s);
    case LBM_STORE_BF16R: return launch_fixup<LBM_STORE_BF16S, true>(P, s);
    default: return set_error(LBM_ERR_ARG, "unknown storage type");
  }
}

static int launch_fused_step(int storage, int npt, int flags, const KParams& P, cudaStream_t s) {
  switch (storage * 16 + npt) {
    case LBM_STORE_F64 * 16 + 2: return launch_v2<LBM_STORE_F64, 2>(P, s);
    case LBM_STORE_F64 * 16 + 4: return launch_v2<LBM_STORE_F64, 4>(P, s);
    case LBM_STORE_FX64 * 16 + 1: return launch_fx<1>(P, s);
    case LBM_STORE_FX64 * 16 + 2: return launch_fx<2>(P, s);
    case LBM_STORE_FX64 * 16 + 4: return launch_fx<4>(P, s);
    case LBM_STORE_F32 * 16 + 2: return launch_v2<LBM_STORE_F32, 2>(P, s);
    case LBM_STORE_F32 * 16 + 4: return launch_v2<LBM_STORE_F32, 4>(P, s);
    case LBM_STORE_F16S * 16 + 2: return launch_v2<LBM_STORE_F16S, 2>(P, s);
    case LBM_STORE_F16S * 16 + 4: return launch_v2<LBM_STORE_F16S, 4>(P, s);
    case LBM_STORE_F16S * 16 + 8: return launch_v2<LBM_STORE_F16S, 8>(P, s);
    case LBM_STORE_BF16S * 16 + 2: return launch_v2<LBM_STORE_BF16S, 2>(P, s);
    case LBM_STORE_BF16S * 16 + 4: return launch_v2<LBM_STORE_BF16S, 4>(P, s);
    case LBM_STORE_BF16S * 16 + 8: return launch_v2<LBM_STORE_BF16S, 8>(P, s);
    case LBM_STORE_F16R * 16 + 4: return launch_v2<LBM_STORE_F16S, 4, true>(P, s);
    case LBM_STORE_BF16R * 16 + 4: return launch_v2<LBM_STORE_BF16S, 4, true>(P, s);
    default: return dispatch<MODE_FUSED>(storage, flags & LBM_FLAG_EXACT, P, s);
  }
}

static size_t store_bytes(int storage) {
  switch (storage) {
    case LBM_STORE_F64:
    case LBM_STORE_FX64: return 8;
    case LBM_STORE_F32: return 4;
    case LBM_STORE_F16S:
    case LBM_STORE_BF16S:
    case LBM_STORE_F16R:
    case LBM_STORE_BF16R: return 2;
    default: return 0;
  }
}

static View ref_f(const double* p, int ny) { return View{p, 9LL * ny, 9, 1}; }
static View ref_rho(const double* p, int ny) { return View{p, (int64_t)ny, 1, 0}; }
static View ref_u(const double* p, int ny) { return View{p, 2LL * ny, 2, 1}; }
static OutView ref_f_out(double* p, int ny) { return OutView{p, 9LL * ny, 9, 1}; }
static OutView ref_rho_out(double* p, int ny) { return OutView{p, (int64_t)ny, 1, 0}; }
static OutView ref_u_out(double* p, int ny) { return OutView{p, 2LL * ny, 2, 1}; }

}  // namespace lbm

using namespace lbm;

extern "C" {

size_t lbm_lattice_pop_bytes(int32_t nx, int32_t ny, int64_t pitch, int32_t storage) {
  (void)nx;
  return (size_t)9 * (size_t)ny * (size_t)pitch * store_bytes(storage);
}

int lbm_lattice_init(const lbm_geometry* g, int32_t storage, const double* f, const double* rho,
                     const double* u, double omega, void* pop_out, int64_t pitch, void* aux_out,
                     int32_t flags, void* stream) {
  KParams P;
  std::memset(&P, 0, sizeof(P));
  if (!to_geok(g, P.g)) return last_status();
  if (int e = check_omega(omega)) return e;
  if (int e = check_pitch(g->nx, pitch)) return e;
  if (f == nullptr || pop_out == nullptr) return set_error(LBM_ERR_ARG, "f and pop_out are required");
  if ((rho == nullptr) != (u == nullptr)) return set_error(LBM_ERR_ARG, "rho and u must be given together");
  if (g->outlet && aux_out == nullptr) return set_error(LBM_ERR_ARG, "the outlet needs aux_out");
  P.pop_out = pop_out;
  P.pitch = pitch;
  P.plane = pitch * g->ny;
  P.aux_out = aux_out;
  P.f_in = ref_f(f, g->ny);
  if (rho) {
    P.rho_in = ref_rho(rho, g->ny);
    P.u_in = ref_u(u, g->ny);
  }
  P.omega = omega;
  set_shift(P);
  return dispatch<MODE_INIT>(storage, flags & LBM_FLAG_EXACT, P, (cudaStream_t)stream);
}

int lbm_lattice_run(const lbm_geometry* g, int32_t storage, void* pop_a, void* pop_b, int64_t pitch,
                    void* aux_a, void* aux_b, double omega, int32_t nsteps, double* rho_out,
                    double* u_out, int32_t flags, uint32_t seed, void* stream) {
  return lbm_lattice_run_opts(g, storage, pop_a, pop_b, pitch, aux_a, aux_b, omega, nsteps, rho_out, u_out, flags,
                              seed, nullptr, stream);
}

int lbm_lattice_run_opts(const lbm_geometry* g, int32_t storage, void* pop_a, void* pop_b, int64_t pitch,
                         void* aux_a, void* aux_b, double omega, int32_t nsteps, double* rho_out,
                         double* u_out, int32_t flags, uint32_t seed, const lbm_run_options* opt,
                         void* stream) {
  KParams P;
  std::memset(&P, 0, sizeof(P));
  if (!to_geok(g, P.g)) return last_status();
  if (int e = check_omega(omega)) return e;
  if (int e = check_pitch(g->nx, pitch)) return e;
  if (pop_a == nullptr || pop_b == nullptr || pop_a == pop_b)
    return set_error(LBM_ERR_ARG, "two distinct population buffers are required");
  if (g->outlet && (aux_a == nullptr || aux_b == nullptr || aux_a == aux_b))
    return set_error(LBM_ERR_ARG, "the outlet needs two distinct aux buffers");
  if (nsteps < 0) return set_error(LBM_ERR_ARG, "nsteps must be >= 0");
  P.probe_x = P.probe_y = -1;
  if (opt != nullptr && opt->probe_buf != nullptr) {
    if (opt->probe_count == nullptr || opt->probe_cap < 0)
      return set_error(LBM_ERR_ARG, "a probe needs probe_count and probe_cap >= 0");
    if (opt->probe_x < 0 || opt->probe_x >= g->nx || opt->probe_y < 0 || opt->probe_y >= g->ny)
      return set_error(LBM_ERR_ARG, "the probe node lies outside the lattice");
    P.probe_x = opt->probe_x;
    P.probe_y = opt->probe_y;
    P.probe_cap = opt->probe_cap;
    P.probe_buf = opt->probe_buf;
    P.probe_count = opt->probe_count;
  }
  const int32_t* counter = opt != nullptr ? opt->step_counter : nullptr;
  P.pitch = pitch;
  P.plane = pitch * g->ny;
  P.omega = omega;
  set_shift(P);
  P.sr = (flags & LBM_FLAG_STOCHASTIC) != 0;
  P.qc = fx::q_consts(omega);
  P.step_dev = counter;
  for (int s = 0; s < nsteps; ++s) {
    // with a device counter the kernels hash (seed + s + *counter) themselves
    P.seed = counter != nullptr ? seed + (uint32_t)s : hash32(seed + (uint32_t)s);
    const bool even = (s % 2) == 0;
    P.pop_in = even ? pop_a : pop_b;
    P.pop_out = even ? pop_b : pop_a;
    P.aux_in = even ? aux_a : aux_b;
    P.aux_out = even ? aux_b : aux_a;
    const bool last = s == nsteps - 1;
    P.rho_out = OutView{last ? rho_out : nullptr, 1, pitch, 0};
    P.u_out = OutView{last ? u_out : nullptr, 1, pitch, pitch * g->ny};
    if (int e = launch_fused(storage, flags, P, (cudaStream_t)stream)) return e;
  }
  if (counter != nullptr && nsteps > 0) {
    advance_counter_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(opt->step_counter, nsteps);
    count_launch();
    if (int e = check_launch("advance_counter_kernel")) return e;
  }
  return LBM_OK;
}

int lbm_lattice_read(const lbm_geometry* g, int32_t storage, const void* pop, int64_t pitch, const void* aux,
                     double* f_out, double* rho_out, double* u_out, void* stream) {
  KParams P;
  std::memset(&P, 0, sizeof(P));
  if (!to_geok(g, P.g)) return last_status();
  if (int e = check_pitch(g->nx, pitch)) return e;
  if (pop == nullptr) return set_error(LBM_ERR_ARG, "pop is required");
  if (g->outlet && aux == nullptr) return set_error(LBM_ERR_ARG, "the outlet needs aux");
  P.pop_in = pop;
  P.aux_in = aux;
  P.pitch = pitch;
  P.plane = pitch * g->ny;
  P.f_out = ref_f_out(f_out, g->ny);
  P.rho_out = ref_rho_out(rho_out, g->ny);
  P.u_out = ref_u_out(u_out, g->ny);
  set_shift(P);  // omega 1: the read converts, it does not collide
  return dispatch<MODE_READ>(storage, false, P, (cudaStream_t)stream);
}

size_t lbm_step_scratch_bytes(int32_t nx, int32_t ny) {
  const int64_t pitch = ((int64_t)nx + 31) / 32 * 32;
  return (size_t)(9 * pitch * ny + 3 * (int64_t)ny) * sizeof(double) + 256;
}

int lbm_step_f64(const lbm_geometry* g, const double* f, const double* rho, const double* u, double omega,
                 double* f_out, double* rho_out, double* u_out, void* scratch, int32_t flags, void* stream) {
  if (g == nullptr) return set_error(LBM_ERR_ARG, "geometry is NULL");
  if (f == nullptr || rho == nullptr || u == nullptr || f_out == nullptr || rho_out == nullptr ||
      u_out == nullptr || scratch == nullptr)
    return set_error(LBM_ERR_ARG, "f, rho, u, f_out, rho_out, u_out and scratch are required");
  const int64_t pitch = ((int64_t)g->nx + 31) / 32 * 32;
  uintptr_t base = ((uintptr_t)scratch + 255) & ~(uintptr_t)255;
  double* pop = reinterpret_cast<double*>(base);
  double* aux = pop + 9 * pitch * g->ny;
  if (int e = lbm_lattice_init(g, LBM_STORE_F64, f, rho, u, omega, pop, pitch, aux, flags, stream)) return e;
  // the read-out kernel recomputes the moments the same way in both forms
  KParams P;
  std::memset(&P, 0, sizeof(P));
  if (!to_geok(g, P.g)) return last_status();
  P.pop_in = pop;
  P.aux_in = aux;
  P.pitch = pitch;
  P.plane = pitch * g->ny;
  P.f_out = ref_f_out(f_out, g->ny);
  P.rho_out = ref_rho_out(rho_out, g->ny);
  P.u_out = ref_u_out(u_out, g->ny);
  return (flags & LBM_FLAG_EXACT) ? launch<LBM_STORE_F64, true, MODE_READ>(P, (cudaStream_t)stream)
                                  : launch<LBM_STORE_F64, false, MODE_READ>(P, (cudaStream_t)stream);
}

// ---- the drop-in step on host buffers, with copies and kernels overlapped ----
size_t lbm_step_host_scratch_bytes(int32_t nx, int32_t ny) {
  const int64_t pitch = ((int64_t)nx + 31) / 32 * 32, n = (int64_t)nx * ny;
  return (size_t)(24 * n + 9 * pitch * ny + 3 * (int64_t)ny) * sizeof(double) + 4 * 256;
}

int lbm_step_f64_host(const lbm_geometry* g, const double* f, const double* rho, const double* u, double omega,
                      double* f_out, double* rho_out, double* u_out, void* scratch, size_t scratch_bytes,
                      int32_t flags, int32_t slabs, void* stream) {
  if (g == nullptr) return set_error(LBM_ERR_ARG, "geometry is NULL");
  if (f == nullptr || rho == nullptr || u == nullptr || f_out == nullptr || rho_out == nullptr ||
      u_out == nullptr || scratch == nullptr)
    return set_error(LBM_ERR_ARG, "f, rho, u, f_out, rho_out, u_out and scratch are required");
  KParams G;
  std::memset(&G, 0, sizeof(G));
  if (!to_geok(g, G.g)) return last_status();
  if (int e = check_omega(omega)) return e;
  const int nx = g->nx, ny = g->ny;
  if (scratch_bytes < lbm_step_host_scratch_bytes(nx, ny)) return set_error(LBM_ERR_ARG, "scratch too small");
  const int64_t n = (int64_t)nx * ny, pitch = ((int64_t)nx + 31) / 32 * 32;
  const bool exact = (flags & LBM_FLAG_EXACT) != 0;
  // device layout: inputs f, rho, u | outputs f, rho, u | populations | outlet memory
  double* base = reinterpret_cast<double*>(((uintptr_t)scratch + 255) & ~(uintptr_t)255);
  double* fin = base;
  double* rin = fin + 9 * n;
  double* uin = rin + n;
  double* fo = uin + 2 * n;
  double* ro = fo + 9 * n;
  double* uo = ro + n;
  double* pop = reinterpret_cast<double*>(((uintptr_t)(uo + 2 * n) + 255) & ~(uintptr_t)255);
  double* aux = pop + 9 * pitch * ny;
  // default depth: one slab per 2^18 nodes, at most 32 (the copies then run
  // within a few percent of the link's two-way rate on large lattices)
  const int64_t auto_k = std::max<int64_t>(1, std::min<int64_t>(32, n >> 18));
  const int K = (int)std::max<int64_t>(1, std::min<int64_t>(slabs > 0 ? slabs : auto_k, nx));
  auto xs = [&](int k) { return (int)((int64_t)k * nx / K); };
  cudaStream_t caller = (cudaStream_t)stream, sh = nullptr, sc = nullptr, sd = nullptr;
  std::vector<cudaEvent_t> ev;
  int st = LBM_OK;
  auto cuda_ok = [&](cudaError_t e) {
    if (e != cudaSuccess && st == LBM_OK) st = set_error(LBM_ERR_CUDA, cudaGetErrorString(e));
    return st == LBM_OK;
  };
  auto event = [&]() {
    cudaEvent_t e = nullptr;
    cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ev.push_back(e);
    return e;
  };
  cuda_ok(cudaStreamCreateWithFlags(&sh, cudaStreamNonBlocking));
  cuda_ok(cudaStreamCreateWithFlags(&sc, cudaStreamNonBlocking));
  cuda_ok(cudaStreamCreateWithFlags(&sd, cudaStreamNonBlocking));
  cudaEvent_t start = event();
  cuda_ok(cudaEventRecord(start, caller));
  cuda_ok(cudaStreamWaitEvent(sh, start, 0));
  cuda_ok(cudaStreamWaitEvent(sc, start, 0));
  cuda_ok(cudaStreamWaitEvent(sd, start, 0));
  std::vector<cudaEvent_t> in_ready(K), out_ready(K);
  auto upload = [&](int k) {
    if (st != LBM_OK) return;
    const int64_t a = xs(k), w = xs(k + 1) - xs(k);
    cuda_ok(cudaMemcpyAsync(fin + 9 * a * ny, f + 9 * a * ny, 9 * w * ny * sizeof(double), cudaMemcpyHostToDevice, sh));
    cuda_ok(cudaMemcpyAsync(rin + a * ny, rho + a * ny, w * ny * sizeof(double), cudaMemcpyHostToDevice, sh));
    cuda_ok(cudaMemcpyAsync(uin + 2 * a * ny, u + 2 * a * ny, 2 * w * ny * sizeof(double), cudaMemcpyHostToDevice, sh));
    in_ready[k] = event();
    cuda_ok(cudaEventRecord(in_ready[k], sh));
  };
  auto init = [&](int k) {
    if (st != LBM_OK) return;
    KParams P = G;
    P.xb = xs(k);
    P.xe = xs(k + 1);
    P.pop_out = pop;
    P.pitch = pitch;
    P.plane = pitch * ny;
    P.aux_out = aux;
    P.f_in = ref_f(fin, ny);
    P.rho_in = ref_rho(rin, ny);
    P.u_in = ref_u(uin, ny);
    P.omega = omega;
    if (!cuda_ok(cudaStreamWaitEvent(sc, in_ready[k], 0))) return;
    const int e = exact ? launch<LBM_STORE_F64, true, MODE_INIT>(P, sc) : launch<LBM_STORE_F64, false, MODE_INIT>(P, sc);
    if (e != LBM_OK && st == LBM_OK) st = e;
  };
  auto read = [&](int k) {
    if (st != LBM_OK) return;
    KParams P = G;
    P.xb = xs(k);
    P.xe = xs(k + 1);
    P.pop_in = pop;
    P.aux_in = aux;
    P.pitch = pitch;
    P.plane = pitch * ny;
    P.f_out = ref_f_out(fo, ny);
    P.rho_out = ref_rho_out(ro, ny);
    P.u_out = ref_u_out(uo, ny);
    const int e = exact ? launch<LBM_STORE_F64, true, MODE_READ>(P, sc) : launch<LBM_STORE_F64, false, MODE_READ>(P, sc);
    if (e != LBM_OK && st == LBM_OK) st = e;
    out_ready[k] = event();
    cuda_ok(cudaEventRecord(out_ready[k], sc));
  };
  auto download = [&](int k) {
    if (st != LBM_OK) return;
    const int64_t a = xs(k), w = xs(k + 1) - xs(k);
    cuda_ok(cudaStreamWaitEvent(sd, out_ready[k], 0));
    cuda_ok(cudaMemcpyAsync(f_out + 9 * a * ny, fo + 9 * a * ny, 9 * w * ny * sizeof(double), cudaMemcpyDeviceToHost, sd));
    cuda_ok(cudaMemcpyAsync(rho_out + a * ny, ro + a * ny, w * ny * sizeof(double), cudaMemcpyDeviceToHost, sd));
    cuda_ok(cudaMemcpyAsync(u_out + 2 * a * ny, uo + 2 * a * ny, 2 * w * ny * sizeof(double), cudaMemcpyDeviceToHost, sd));
  };
  // Read-out of slab k pulls from columns of slabs k-1 and k+1 (periodic in x),
  // so it follows their collisions.  The pressure rewrite writes columns 0 and
  // nx-1 from columns nx-2 and 1: with it, every collision runs first.  The
  // calls are issued interleaved (upload k, collide k, read out and download
  // k-1), which also keeps the host issuing work while copies from pageable
  // memory block it.
  if (g->pressure || K < 3) {
    for (int k = 0; k < K; ++k) {
      upload(k);
      init(k);
    }
    for (int k = 0; k < K; ++k) {
      read(k);
      download(k);
    }
  } else {
    upload(0);
    init(0);
    upload(1);
    init(1);
    for (int k = 2; k < K; ++k) {
      upload(k);
      init(k);
      read(k - 1);
      download(k - 1);
    }
    read(K - 1);
    download(K - 1);
    read(0);
    download(0);
  }
  // the caller's stream continues once every copy has landed
  cudaEvent_t done_h = event(), done_c = event(), done_d = event();
  cuda_ok(cudaEventRecord(done_h, sh));
  cuda_ok(cudaEventRecord(done_c, sc));
  cuda_ok(cudaEventRecord(done_d, sd));
  cuda_ok(cudaStreamWaitEvent(caller, done_h, 0));
  cuda_ok(cudaStreamWaitEvent(caller, done_c, 0));
  cuda_ok(cudaStreamWaitEvent(caller, done_d, 0));
  // streams and events are released once their work completes
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  if (sh) cudaStreamDestroy(sh);
  if (sc) cudaStreamDestroy(sc);
  if (sd) cudaStreamDestroy(sd);
  return st;
}

}  // extern "C"
