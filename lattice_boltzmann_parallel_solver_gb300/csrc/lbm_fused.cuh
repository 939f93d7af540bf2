// lbm_fused.cuh -- parameters and the vectorised fused-step body shared by the
// single-lattice kernels (lbm_lattice.cu) and the batched kernels (lbm_batch.cu).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>

#include "lbm_core.cuh"
#include "lbm_fx.cuh"
#include "lbm_host.h"

namespace lbm {

enum { MODE_INIT = 0, MODE_FUSED = 1, MODE_READ = 2 };

struct GeoK {
  int nx, ny, words;
  const uint32_t* bcmask;
  const uint32_t* desc;
  int pressure;
  uint32_t pin, pout;
  double rho_in, rho_out;
  int outlet;
  double kconst[LBM_MAX_SETS][9];
  double cconst[LBM_MAX_SETS][9];
  const int32_t* bcnodes;
  int n_bcnodes;
  // plain inlet / outlet columns (lbm_geometry), and the inlet's populations
  uint32_t edge_in_desc, edge_out_desc;
  int n_bcnodes_edge;
  double edge_in_f[9];
  // reference velocity of the reference-shifted 16-bit storages
  double dev_ref_ux, dev_ref_uy;
};

struct View {
  const double* p;
  int64_t sx, sy, sc;
};
struct OutView {
  double* p;
  int64_t sx, sy, sc;
};

struct KParams {
  GeoK g;
  // columns [xb, xe) handled by the one-node-per-thread kernel (xe == 0: all)
  int xb, xe;
  const void* pop_in;
  void* pop_out;
  int64_t pitch, plane;
  const void* aux_in;
  void* aux_out;
  View f_in, rho_in, u_in;
  OutView f_out, rho_out, u_out;
  double omega;
  // optional probe: the fused step at node (probe_x, probe_y) appends its
  // pre-collision velocity to probe_buf[2 * t], t = (*probe_count)++
  int probe_x, probe_y, probe_cap;
  double* probe_buf;
  int* probe_count;
  // 16-bit storages: stochastic rounding of the stored deviations (sr != 0),
  // random bits hashed from (node, direction, seed); the launcher varies the
  // seed per step
  uint32_t seed;
  int sr;
  // optional device step counter: when set, a launch's random bits come from
  // hash32(seed + *step_dev) (seed then holds the unhashed base + step index),
  // so a captured CUDA graph of steps draws new bits on every replay
  const int32_t* step_dev;
  // the reference-shifted 16-bit storages (LBM_STORE_F16R, LBM_STORE_BF16R):
  // their constants in the working units of f16 ([0], scale 1024) and bf16
  // ([1], scale 1: sig in populations), filled by set_shift from g.dev_ref_*
  // and omega; dev_shift selects them in the generic kernel
  ShiftK shf[2];
  int dev_shift;
  // fixed-point storage: constants of its collision
  fx::QConsts qc;
};

__device__ __forceinline__ uint32_t launch_seed(const KParams& P) {
  return P.step_dev != nullptr ? hash32(P.seed + (uint32_t)__ldg(P.step_dev)) : P.seed;
}

// a node the body applies as a plain inlet / outlet node itself (edges on)
__device__ __forceinline__ bool plain_edge_node(const KParams& P, int x, int y) {
  const uint32_t want = x == 0 ? P.g.edge_in_desc : (x == P.g.nx - 1 ? P.g.edge_out_desc : 0u);
  return want != 0u && __ldg(P.g.desc + y * P.g.nx + x) == want;
}

// skip_bc: a body without its boundary block leaves the probe of a node that
// the batched boundary-node pass recomputes (a listed boundary node other than
// the plain edge nodes the body applies itself when ``edges`` is set, or,
// under the pressure rewrite, a node of column 1 or nx-2) to that pass
template <typename R>
__device__ __forceinline__ void write_probe(const KParams& P, int x, int y, R ux, R uy, bool skip_bc = false,
                                            bool edges = false) {
  if (P.probe_buf != nullptr && x == P.probe_x && y == P.probe_y) {
    if (skip_bc && ((P.g.pressure && (x == 1 || x == P.g.nx - 2)) ||
                    (P.g.bcmask != nullptr && ((__ldg(P.g.bcmask + y * P.g.words + (x >> 5)) >> (x & 31)) & 1u) &&
                     !(edges && plain_edge_node(P, x, y)))))
      return;
    const int t = *P.probe_count;
    if (t < P.probe_cap) {
      P.probe_buf[2 * t] = (double)ux;
      P.probe_buf[2 * t + 1] = (double)uy;
    }
    *P.probe_count = t + 1;
  }
}

// ---------------------------------------------------------------------------
// Vectorised fused step.  Each thread owns NPT consecutive nodes of one row
// (one aligned vector per population plane).  The six planes with cx = +-1
// need the chunk shifted by one node: the missing element comes from the
// neighbouring lane by a warp shuffle, or by a direct load at the first and
// last lane of a warp and at the row ends (periodic wrap).  A row whose width
// is not a multiple of NPT ends in a partial chunk: its vector loads run into
// the row padding (pitch >= nx rounded up to 32), the node at nx-1 takes its
// cx = -1 populations from x = 0, and it stores node by node.  Offsets are
// 32-bit element indices (9 * plane < 2^31).  Boundary descriptors and the
// pressure rewrite are compiled in only where a geometry may have them.
// ---------------------------------------------------------------------------
template <int STORE, int NPT, bool HAS_BC, bool HAS_PRESSURE, bool EDGES = false, bool SHIFT = false>
__device__ __forceinline__ void fused_v2_body(const KParams& P, const void* pop_in_v, void* pop_out_v,
                                              const void* aux_in_v, void* aux_out_v, int x0, int y,
                                              uint32_t seed, bool listed = false) {
  using St = Store<STORE>;
  using T = typename St::T;
  using R = typename St::R;
  // working values: scaled deviations s (f - w) for the shifted 16-bit storages
  // (the stored numbers themselves), f otherwise
  constexpr bool SH = St::kShifted;
  static_assert(!SHIFT || SH, "the reference shift applies to the 16-bit deviations");
  constexpr R kS = [] {
    if constexpr (SH) return (R)St::kDev;
    else return R(1);
  }();
  const int lane = threadIdx.x & 31;
  const int nx = P.g.nx, ny = P.g.ny;
  const int xlast = ((nx - 1) / NPT) * NPT;  // first node of the last chunk of a row
  const bool active = x0 < nx;
  if (!active) x0 = xlast;  // stays in the shuffles, stores nothing
  const int nvalid = min(NPT, nx - x0);
  const int pitch = (int)P.pitch, plane = (int)P.plane;
  const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
  const int r0 = y * pitch, rm = ym * pitch, rp = yp * pitch;
  const bool first = x0 == 0;
  const bool last = x0 == xlast;
  const int xm = first ? nx - 1 : x0 - 1;
  const int xp = x0 + NPT >= nx ? 0 : x0 + NPT;
  const T* pin = static_cast<const T*>(pop_in_v);
  auto ld_work = [&](const T* p, int i) -> R {
    if constexpr (SH) return St::ld_dev(p);
    else return St::ld(p, i);
  };
  auto work_of_raw = [&](T t, int i) -> R {
    if constexpr (SH) return St::dev(t);
    else return St::to_r(t, i);
  };
  // SHIFT (LBM_STORE_F16R, LBM_STORE_BF16R): the working values are the
  // stored numbers s (f_i - c_i) = s (f_i - w_i) - sig_i, c_i the equilibrium
  // at the reference velocity (ShiftK)
  const ShiftK& shk = P.shf[STORE == LBM_STORE_F16S ? 0 : 1];
  auto sig = [&](int i) -> R {
    if constexpr (SHIFT) return shk.sig[i];
    else return R(0);
  };
  auto work_of_f = [&](R fv, int i) -> R {
    if constexpr (SHIFT) return fma(fv - wr<R>(i), kS, -sig(i));
    else return SH ? (fv - wr<R>(i)) * kS : fv;
  };
  auto f_of_work = [&](R v, int i) -> R {
    if constexpr (SHIFT) return fma(v + sig(i), R(1) / kS, wr<R>(i));
    else return SH ? fma(v, R(1) / kS, wr<R>(i)) : v;
  };

  // the boundary mask word first: its latency overlaps the population loads.
  // The boundary-node pass on a node of the boundary list (listed) knows its
  // bit: its descriptor and its own populations (the bounce-back sources) then
  // load together with the pulled ones instead of one after another.
  const bool has_bc = HAS_BC && P.g.bcmask != nullptr;
  constexpr bool PASS = NPT == 1 && HAS_BC;
  const bool known = PASS && has_bc && listed;
  const uint32_t bcword =
      has_bc ? (known ? (1u << (x0 & 31)) : __ldg(P.g.bcmask + y * P.g.words + (x0 >> 5))) : 0u;
  const uint32_t dknown = known ? __ldg(P.g.desc + y * nx + x0) : 0u;
  R own[PASS ? 9 : 1];
  R f[9][NPT];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int row = cy(i) == 1 ? rm : (cy(i) == -1 ? rp : r0);
    const T* base = pin + i * plane + row;
    if constexpr (NPT == 1) {
      // one node per thread (the boundary-node pass): neighbours loaded directly
      f[i][0] = ld_work(base + (cx(i) == 1 ? xm : (cx(i) == -1 ? xp : x0)), i);
      if constexpr (PASS) own[i] = ld_work(pin + i * plane + r0 + x0, i);
      continue;
    }
    T raw[NPT];
    ld_vec<T, NPT>(base + x0, raw);
    R v[NPT];
#pragma unroll
    for (int k = 0; k < NPT; ++k) v[k] = work_of_raw(raw[k], i);
    if (cx(i) == 0) {
#pragma unroll
      for (int k = 0; k < NPT; ++k) f[i][k] = v[k];
    } else if (cx(i) == 1) {
      R prev = __shfl_up_sync(0xffffffffu, v[NPT - 1], 1);
      if (lane == 0 || first) prev = ld_work(base + xm, i);
      f[i][0] = prev;
#pragma unroll
      for (int k = 1; k < NPT; ++k) f[i][k] = v[k - 1];
    } else {
      R next = __shfl_down_sync(0xffffffffu, v[0], 1);
      if (lane == 31 || last) next = ld_work(base + xp, i);
#pragma unroll
      for (int k = 0; k < NPT - 1; ++k) f[i][k] = v[k + 1];
      f[i][NPT - 1] = next;
      if (nvalid < NPT) {
        // partial chunk: gather node by node, node nx-1 wraps to x = 0
#pragma unroll
        for (int k = 0; k < NPT; ++k) {
          const int xs = x0 + k + 1 < nx ? x0 + k + 1 : 0;
          f[i][k] = ld_work(base + xs, i);
        }
      }
    }
  }

  if constexpr (EDGES && !HAS_BC) {
    // the plain inlet / outlet columns, applied to every node of column 0 /
    // nx-1 (the pass recomputes the ones with other sources)
    if (first && P.g.edge_in_desc != 0u) {
#pragma unroll
      for (int i = 0; i < 9; ++i) f[i][0] = work_of_f((R)P.g.edge_in_f[i], i);
    }
    if (last && P.g.edge_out_desc != 0u && aux_in_v != nullptr) {
      const R* aux_in = static_cast<const R*>(aux_in_v);
      const int kl = nx - 1 - x0;
      const R a3 = work_of_f(aux_in[0 * ny + y], 3), a6 = work_of_f(aux_in[1 * ny + y], 6),
              a7 = work_of_f(aux_in[2 * ny + y], 7);
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        f[3][k] = k == kl ? a3 : f[3][k];
        f[6][k] = k == kl ? a6 : f[6][k];
        f[7][k] = k == kl ? a7 : f[7][k];
      }
    }
  }

  if (has_bc) {
    const uint32_t bits = (bcword >> (x0 & 31)) & ((NPT >= 32) ? 0xffffffffu : ((1u << NPT) - 1u));
    if (bits) {
      const R* aux_in = static_cast<const R*>(aux_in_v);
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        if (!((bits >> k) & 1u)) continue;
        const int x = x0 + k;
        const uint32_t d = known ? dknown : __ldg(P.g.desc + y * nx + x);
        const int ks = (d >> LBM_DESC_KSET_SHIFT) & 15, cs = (d >> LBM_DESC_CSET_SHIFT) & 15;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          const uint32_t s = (d >> (2 * i)) & 3u;
          if (s == LBM_SRC_BOUNCE) {
            R v;
            if constexpr (PASS) v = own[opp(i)];
            else v = ld_work(pin + opp(i) * plane + r0 + x, opp(i));
            v -= (R)P.g.kconst[ks][i] * kS;
            if constexpr (SHIFT) v += sig(opp(i)) - sig(i);
            f[i][k] = v;
          } else if (s == LBM_SRC_CONST)
            f[i][k] = work_of_f((R)P.g.cconst[cs][i], i);
          else if (s == LBM_SRC_OUTLET && outlet_slot(i) >= 0 && aux_in != nullptr)
            f[i][k] = work_of_f(aux_in[outlet_slot(i) * ny + y], i);
        }
      }
    }
  }

  if (aux_out_v != nullptr && active && x0 <= nx - 2 && nx - 2 < x0 + NPT) {
    // the outlet memory holds full populations in every kernel
    R* aux_out = static_cast<R*>(aux_out_v);
    const int ka = nx - 2 - x0;
    R a3 = f[3][0], a6 = f[6][0], a7 = f[7][0];
#pragma unroll
    for (int k = 1; k < NPT; ++k) {
      a3 = k == ka ? f[3][k] : a3;
      a6 = k == ka ? f[6][k] : a6;
      a7 = k == ka ? f[7][k] : a7;
    }
    aux_out[0 * ny + y] = f_of_work(a3, 3);
    aux_out[1 * ny + y] = f_of_work(a6, 6);
    aux_out[2 * ny + y] = f_of_work(a7, 7);
  }

  R pv[9];  // pressure rewrite computed by the node at column nx-2 or 1
  int pcol = -1;
  const R omega = (R)P.omega;
  const bool want_m = P.rho_out.p != nullptr || P.probe_buf != nullptr;
  // moments written out for the last step or the probe, and the pressure
  // rewrite source, of node k (working values g after the collision)
  auto node_extras = [&](int k, R sum, R rho, R ux, R uy, const R g[9]) {
    const int x = x0 + k;
    if (want_m && active && k < nvalid) {
      if (P.rho_out.p != nullptr) {
        P.rho_out.p[x * P.rho_out.sx + y * P.rho_out.sy] = SH ? 1.0 + (double)sum / (double)kS : (double)rho;
        double* up = P.u_out.p + x * P.u_out.sx + y * P.u_out.sy;
        up[0] = (double)ux;
        up[P.u_out.sc] = (double)uy;
      }
      write_probe(P, x, y, ux, uy, !HAS_BC, EDGES);
    }
    if (HAS_PRESSURE && P.g.pressure && k < nvalid && (x == nx - 2 || x == 1)) {
      R br[9];
      bracket9_fast(ux, uy, br);
      const R rb = (R)(x == nx - 2 ? P.g.rho_in : P.g.rho_out) * kS - rho;
#pragma unroll
      for (int i = 0; i < 9; ++i) pv[i] = fma(wr<R>(i) * br[i], rb, g[i]);
      pcol = x;
    }
  };
  if constexpr (SH) {
    // 16-bit storages: two nodes per packed float32 instruction (one node per
    // thread runs the same packed arithmetic on a duplicated pair, so that the
    // boundary-node pass rounds exactly as the step does)
    constexpr int K2 = NPT == 1 ? 1 : 2;
    static_assert(NPT == 1 || NPT % 2 == 0, "packed pairs");
#pragma unroll
    for (int k = 0; k < NPT; k += K2) {
      const int k1 = NPT == 1 ? k : k + 1;
      float2 g2[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) g2[i] = make_float2(f[i][k], f[i][k1]);
      float2 sum, jx, jy;
      moments9x2(g2, sum, jx, jy);
      if constexpr (SHIFT) {
        // the momentum of sig (its mass enters the collision through oS)
        jx = add2(jx, f2c(shk.sx));
        jy = add2(jy, f2c(shk.sy));
      }
      const float2 rho = add2(f2c(kS), sum);  // s rho
      const float2 inv = make_float2(rho.x != 0.0f ? rcp_nr(rho.x) : 0.0f, rho.y != 0.0f ? rcp_nr(rho.y) : 0.0f);
      const float2 ux = mul2(jx, inv), uy = mul2(jy, inv);
      if constexpr (SHIFT)
        collide_dev2_ref(g2, sum, rho, ux, uy, omega, shk);
      else
        collide_dev2(g2, sum, rho, ux, uy, omega);
      if constexpr (SHIFT) sum = add2(sum, f2c(shk.S));  // s (rho - 1) for the moments written out
      R ga[9], gb[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        ga[i] = g2[i].x;
        gb[i] = g2[i].y;
        f[i][k] = ga[i];
        f[i][k1] = gb[i];
      }
      node_extras(k, sum.x, rho.x, ux.x, uy.x, ga);
      if (NPT > 1) node_extras(k1, sum.y, rho.y, ux.y, uy.y, gb);
    }
  } else {
#pragma unroll
    for (int k = 0; k < NPT; ++k) {
      R g[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) g[i] = f[i][k];
      R sum, jx, jy;
      moments9(g, sum, jx, jy);
      const R rho = SH ? kS + sum : sum;  // s rho for the 16-bit storages
      const R inv = rho != R(0) ? rcp_nr(rho) : R(0);
      const R ux = jx * inv, uy = jy * inv;
      if constexpr (SH)
        collide_dev(g, sum, rho, ux, uy, omega);
      else
        collide_fast(g, rho, ux, uy, omega);
      node_extras(k, sum, rho, ux, uy, g);
#pragma unroll
      for (int i = 0; i < 9; ++i) f[i][k] = g[i];
    }
  }

  if (!active) return;
  // working value -> stored element (stochastic rounding for 16-bit deviations)
  const bool sr = SH && P.sr;
  auto to_store = [&](R v, int i, uint32_t rbits) -> T {
    if constexpr (SH) return sr ? St::dev_sr(v, rbits) : St::dev_rn(v);
    else return St::from_r(v, i);
  };
  // random bits: one short hash per node, then one multiply-add step per
  // direction; each store takes the high bits of the current word
  uint32_t hk[NPT];
#pragma unroll
  for (int k = 0; k < NPT; ++k) hk[k] = sr ? mix32((uint32_t)(y * nx + x0 + k) * 0x9E3779B1u ^ seed) : 0u;
  T* pout = static_cast<T*>(pop_out_v);
  const bool pr = HAS_PRESSURE && P.g.pressure;
  if (nvalid == NPT && !(pr && (first || last))) {
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      T raw[NPT];
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        raw[k] = to_store(f[i][k], i, hk[k]);
        hk[k] = hk[k] * 0x2C1B3C6Du + 0x297A2D39u;
      }
      st_vec<T, NPT>(pout + i * plane + r0 + x0, raw);
    }
  } else {
    // partial chunk, or a row end under the pressure rewrite: column 0 skips the
    // inlet-side directions, column nx-1 the outlet side
#pragma unroll
    for (int i = 0; i < 9; ++i) {
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        const int x = x0 + k;
        const bool skip = k >= nvalid || (pr && ((x == 0 && ((P.g.pin >> i) & 1u)) ||
                                                 (x == nx - 1 && ((P.g.pout >> i) & 1u))));
        if (!skip) pout[i * plane + r0 + x] = to_store(f[i][k], i, hk[k]);
        hk[k] = hk[k] * 0x2C1B3C6Du + 0x297A2D39u;
      }
    }
  }
  if (pr && pcol >= 0) {
    const uint32_t dirs = pcol == nx - 2 ? P.g.pin : P.g.pout;
    const int dst = pcol == nx - 2 ? 0 : nx - 1;
    uint32_t hp = sr ? mix32((uint32_t)(y * nx + dst) * 0x9E3779B1u ^ seed ^ 0x5bd1e995u) : 0u;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      if ((dirs >> i) & 1u) pout[i * plane + r0 + dst] = to_store(pv[i], i, hp);
      hp = hp * 0x2C1B3C6Du + 0x297A2D39u;
    }
  }
}

// ---------------------------------------------------------------------------
// Vectorised fused step of the fixed-point storage (LBM_STORE_FX64).  The same
// chunking, shuffles and boundary sources as fused_v2_body, on 64-bit integers:
// pull, bounce-back and the outlet copy move populations exactly, the boundary
// constants are rounded to fixed point, and fx::collide_q collides each node in
// its range.  Nodes outside it, the moments written out (last step, probe) and
// the pressure rewrite of columns 0 / nx-1 use float64 on the converted values.
// The outlet memory holds the stored integers, as in the generic kernel.
// ---------------------------------------------------------------------------
template <int NPT, bool HAS_BC, bool HAS_PRESSURE, bool EDGES = false>
__device__ __forceinline__ void fused_fx_body(const KParams& P, const void* pop_in_v, void* pop_out_v,
                                              const void* aux_in_v, void* aux_out_v, int x0, int y) {
  using T = long long;
  const int lane = threadIdx.x & 31;
  const int nx = P.g.nx, ny = P.g.ny;
  const int xlast = ((nx - 1) / NPT) * NPT;
  const bool active = x0 < nx;
  if (!active) x0 = xlast;
  const int nvalid = min(NPT, nx - x0);
  const int pitch = (int)P.pitch, plane = (int)P.plane;
  const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
  const int r0 = y * pitch, rm = ym * pitch, rp = yp * pitch;
  const bool first = x0 == 0;
  const bool last = x0 == xlast;
  const int xm = first ? nx - 1 : x0 - 1;
  const int xp = x0 + NPT >= nx ? 0 : x0 + NPT;
  const T* pin = static_cast<const T*>(pop_in_v);

  // the boundary mask word first: its latency overlaps the population loads
  const bool has_bc = HAS_BC && P.g.bcmask != nullptr;
  const uint32_t bcword = has_bc ? __ldg(P.g.bcmask + y * P.g.words + (x0 >> 5)) : 0u;
  T f[9][NPT];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int row = cy(i) == 1 ? rm : (cy(i) == -1 ? rp : r0);
    const T* base = pin + i * plane + row;
    if constexpr (NPT == 1) {
      // one node per thread: the x neighbours come straight from L1
      f[i][0] = __ldg(base + (cx(i) == 1 ? xm : (cx(i) == -1 ? xp : x0)));
      continue;
    }
    T v[NPT];
    ld_vec<T, NPT>(base + x0, v);
    if (cx(i) == 0) {
#pragma unroll
      for (int k = 0; k < NPT; ++k) f[i][k] = v[k];
    } else if (cx(i) == 1) {
      T prev = __shfl_up_sync(0xffffffffu, v[NPT - 1], 1);
      if (lane == 0 || first) prev = __ldg(base + xm);
      f[i][0] = prev;
#pragma unroll
      for (int k = 1; k < NPT; ++k) f[i][k] = v[k - 1];
    } else {
      T next = __shfl_down_sync(0xffffffffu, v[0], 1);
      if (lane == 31 || last) next = __ldg(base + xp);
#pragma unroll
      for (int k = 0; k < NPT - 1; ++k) f[i][k] = v[k + 1];
      f[i][NPT - 1] = next;
      if constexpr (NPT > 1) {
        if (nvalid < NPT) {
#pragma unroll
          for (int k = 0; k < NPT; ++k) {
            const int xs = x0 + k + 1 < nx ? x0 + k + 1 : 0;
            f[i][k] = __ldg(base + xs);
          }
        }
      }
    }
  }

  if constexpr (EDGES && !HAS_BC) {
    // the plain inlet / outlet columns, applied to every node of column 0 /
    // nx-1 (the pass recomputes the ones with other sources)
    if (first && P.g.edge_in_desc != 0u) {
#pragma unroll
      for (int i = 0; i < 9; ++i) f[i][0] = fx::to_fx(P.g.edge_in_f[i], wd(i));
    }
    if (last && P.g.edge_out_desc != 0u && aux_in_v != nullptr) {
      const T* aux_in = static_cast<const T*>(aux_in_v);
      const int kl = nx - 1 - x0;
      const T a3 = aux_in[0 * ny + y], a6 = aux_in[1 * ny + y], a7 = aux_in[2 * ny + y];
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        f[3][k] = k == kl ? a3 : f[3][k];
        f[6][k] = k == kl ? a6 : f[6][k];
        f[7][k] = k == kl ? a7 : f[7][k];
      }
    }
  }

  if (has_bc) {
    const uint32_t bits = (bcword >> (x0 & 31)) & ((NPT >= 32) ? 0xffffffffu : ((1u << NPT) - 1u));
    if (bits) {
      const T* aux_in = static_cast<const T*>(aux_in_v);
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        if (!((bits >> k) & 1u)) continue;
        const int x = x0 + k;
        const uint32_t d = __ldg(P.g.desc + y * nx + x);
        const int ks = (d >> LBM_DESC_KSET_SHIFT) & 15, cs = (d >> LBM_DESC_CSET_SHIFT) & 15;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          const uint32_t s = (d >> (2 * i)) & 3u;
          if (s == LBM_SRC_BOUNCE)
            f[i][k] = __ldg(pin + opp(i) * plane + r0 + x) - fx::round_scaled(P.g.kconst[ks][i], fx::kS);
          else if (s == LBM_SRC_CONST)
            f[i][k] = fx::to_fx(P.g.cconst[cs][i], wd(i));
          else if (s == LBM_SRC_OUTLET && outlet_slot(i) >= 0 && aux_in != nullptr)
            f[i][k] = aux_in[outlet_slot(i) * ny + y];
        }
      }
    }
  }

  if (aux_out_v != nullptr && active && x0 <= nx - 2 && nx - 2 < x0 + NPT) {
    T* aux_out = static_cast<T*>(aux_out_v);
    const int ka = nx - 2 - x0;
    T a3 = f[3][0], a6 = f[6][0], a7 = f[7][0];
#pragma unroll
    for (int k = 1; k < NPT; ++k) {
      a3 = k == ka ? f[3][k] : a3;
      a6 = k == ka ? f[6][k] : a6;
      a7 = k == ka ? f[7][k] : a7;
    }
    aux_out[0 * ny + y] = a3;
    aux_out[1 * ny + y] = a6;
    aux_out[2 * ny + y] = a7;
  }

  T pv[9];  // pressure rewrite computed by the node at column nx-2 or 1
  int pcol = -1;
  const bool want_m = P.rho_out.p != nullptr || P.probe_buf != nullptr;
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    int64_t g[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i] = f[i][k];
    const int x = x0 + k;
    const bool pnode = HAS_PRESSURE && P.g.pressure && k < nvalid && (x == nx - 2 || x == 1);
    const bool out = want_m && active && k < nvalid &&
                     (P.rho_out.p != nullptr || (P.probe_buf != nullptr && x == P.probe_x && y == P.probe_y));
    double rho = 1.0, ux = 0.0, uy = 0.0;
    if (out || pnode) {
      double d[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) d[i] = fx::from_fx(g[i], wd(i));
      rho = density9(d);
      velocity_fast(d, rho, ux, uy);
      if (out) {
        if (P.rho_out.p != nullptr) {
          P.rho_out.p[x * P.rho_out.sx + y * P.rho_out.sy] = rho;
          double* up = P.u_out.p + x * P.u_out.sx + y * P.u_out.sy;
          up[0] = ux;
          up[P.u_out.sc] = uy;
        }
        write_probe(P, x, y, ux, uy, !HAS_BC, EDGES);
      }
    }
    if (!fx::collide_q(g, P.qc)) {
      double d[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) d[i] = fx::from_fx(g[i], wd(i));
      const double r2 = density9(d);
      double u2x, u2y;
      velocity_fast(d, r2, u2x, u2y);
      collide_fast(d, r2, u2x, u2y, P.omega);
#pragma unroll
      for (int i = 0; i < 9; ++i) g[i] = fx::to_fx(d[i], wd(i));
    }
    if (pnode) {
      double br[9];
      bracket9_fast(ux, uy, br);
      const double rb = (x == nx - 2 ? P.g.rho_in : P.g.rho_out) - rho;
#pragma unroll
      for (int i = 0; i < 9; ++i) pv[i] = fx::to_fx(fma(wd(i) * br[i], rb, fx::from_fx(g[i], wd(i))), wd(i));
      pcol = x;
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) f[i][k] = g[i];
  }

  if (!active) return;
  T* pout = static_cast<T*>(pop_out_v);
  const bool pr = HAS_PRESSURE && P.g.pressure;
  if ((NPT == 1 || nvalid == NPT) && !(pr && (first || last))) {
#pragma unroll
    for (int i = 0; i < 9; ++i) st_vec<T, NPT>(pout + i * plane + r0 + x0, f[i]);
  } else {
#pragma unroll
    for (int i = 0; i < 9; ++i) {
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        const int x = x0 + k;
        const bool skip = k >= nvalid || (pr && ((x == 0 && ((P.g.pin >> i) & 1u)) ||
                                                 (x == nx - 1 && ((P.g.pout >> i) & 1u))));
        if (!skip) pout[i * plane + r0 + x] = f[i][k];
      }
    }
  }
  if (pr && pcol >= 0) {
    const uint32_t dirs = pcol == nx - 2 ? P.g.pin : P.g.pout;
    const int dst = pcol == nx - 2 ? 0 : nx - 1;
#pragma unroll
    for (int i = 0; i < 9; ++i)
      if ((dirs >> i) & 1u) pout[i * plane + r0 + dst] = pv[i];
  }
}

// ---------------------------------------------------------------------------
// Batched step: many lattices of different sizes advance one time step in one
// launch.  The work is a flat list of tiles of one lattice each, and a grid
// strides over the list.  With the boundary-node pass (large batches) a tile
// is `rows` runs of THREADS consecutive chunks (NPT nodes each, chunks
// numbered row by row, so a run may cross a row end); with the sources inside
// the step (small batches) it is `rows` rows of one segment of THREADS chunks.
// Lattice e is live for global steps [s0, s_end); at global step g its input
// buffer is A when (g - s0) is even.  g = *gbase + k, so a captured graph of
// launches k = 0..K-1 followed by lbm_batch_advance stays valid across replays.
// ---------------------------------------------------------------------------
struct __align__(16) BatchEntry {
  KParams P;
  void* pop_a;
  void* pop_b;
  void* aux_a;
  void* aux_b;
  int cpr;             // chunks (of NPT nodes) per row
  uint32_t cpr_magic;  // floor(2^32 / cpr), capped at 2^32 - 1: c / cpr by a multiply-high
  int xblocks;         // row segments of THREADS chunks per row
  int rows;            // runs (or rows) per tile
  int s0, s_end;
};

// ---- host-side checks shared by the launchers --------------------------------
inline bool to_geok(const lbm_geometry* g, GeoK& k) {
  if (g == nullptr) return set_error(LBM_ERR_ARG, "geometry is NULL"), false;
  if (g->nx < 1 || g->ny < 1) return set_error(LBM_ERR_ARG, "nx and ny must be >= 1"), false;
  if (g->bcmask != nullptr && g->desc == nullptr)
    return set_error(LBM_ERR_ARG, "bcmask given without desc"), false;
  if (g->n_kset < 0 || g->n_kset > LBM_MAX_SETS || g->n_cset < 0 || g->n_cset > LBM_MAX_SETS)
    return set_error(LBM_ERR_ARG, "constant-set count out of range"), false;
  if (g->pressure && g->nx < 2)
    return set_error(LBM_ERR_ARG, "the pressure rewrite needs nx >= 2"), false;
  if (g->outlet && g->nx < 2) return set_error(LBM_ERR_ARG, "the outlet needs nx >= 2"), false;
  std::memset(&k, 0, sizeof(k));
  k.nx = g->nx;
  k.ny = g->ny;
  k.words = (g->nx + 31) / 32;
  k.bcmask = g->bcmask;
  k.desc = g->desc;
  k.pressure = g->pressure;
  k.pin = g->pressure_in_dirs & 0x1FFu;
  k.pout = g->pressure_out_dirs & 0x1FFu;
  k.rho_in = g->rho_in;
  k.rho_out = g->rho_out;
  k.outlet = g->outlet;
  std::memcpy(k.kconst, g->kconst, sizeof(k.kconst));
  std::memcpy(k.cconst, g->cconst, sizeof(k.cconst));
  k.bcnodes = g->n_bcnodes > 0 ? g->bcnodes : nullptr;
  k.n_bcnodes = k.bcnodes != nullptr ? g->n_bcnodes : 0;
  if (g->n_bcnodes_edge < 0 || g->n_bcnodes_edge > k.n_bcnodes)
    return set_error(LBM_ERR_ARG, "n_bcnodes_edge out of range"), false;
  if (g->edge_inlet_desc != 0u && (g->edge_inlet_desc & 0x3FFFFu) != 0x2AAAAu)
    return set_error(LBM_ERR_ARG, "edge_inlet_desc is not an all-CONST descriptor"), false;
  if (g->edge_outlet_desc != 0u && (g->edge_outlet_desc & 0x3FFFFu) != 0xF0C0u)
    return set_error(LBM_ERR_ARG, "edge_outlet_desc is not the plain outlet descriptor"), false;
  if (k.bcmask != nullptr) {
    k.edge_in_desc = g->edge_inlet_desc;
    k.edge_out_desc = g->nx >= 2 ? g->edge_outlet_desc : 0u;
    k.n_bcnodes_edge = g->n_bcnodes_edge;
    const int cs = (int)((g->edge_inlet_desc >> LBM_DESC_CSET_SHIFT) & 15u);
    if (k.edge_in_desc != 0u)
      for (int i = 0; i < 9; ++i) k.edge_in_f[i] = g->cconst[cs][i];
  }
  const double ux = g->dev_ref_ux, uy = g->dev_ref_uy;
  if (!(std::fabs(ux) < 0.5 && std::fabs(uy) < 0.5))
    return set_error(LBM_ERR_ARG, "the deviation reference velocity must lie inside (-0.5, 0.5)"), false;
  k.dev_ref_ux = ux;
  k.dev_ref_uy = uy;
  return true;
}

// The constants of the reference-shifted storages (ShiftK) for P.g's reference
// velocity and P.omega (1 where no collision runs).  The collision constants
// are rounded first; sig, S and the momentum (sx, sy) are then derived from
// the rounded values, so that the collision conserves mass exactly and the
// boundary sources and the collision agree on the stored numbers.
inline void set_shift(KParams& P) {
  const double ux = P.g.dev_ref_ux, uy = P.g.dev_ref_uy;
  const double om = (double)(float)(P.omega > 0.0 ? P.omega : 1.0);
  static const int first[4] = {1, 2, 5, 6}, second[4] = {3, 4, 7, 8};
  for (int v = 0; v < 2; ++v) {
    const double scale = v == 0 ? 1024.0 : 1.0;
    double sig[9];
    for (int i = 0; i < 9; ++i) {
      // s (c_i - w_i) = s w_i (3 c.u + 4.5 (c.u)^2 - 1.5 |u|^2) at rho = 1
      const double cu = cx(i) * ux + cy(i) * uy;
      sig[i] = scale * wd(i) * (3.0 * cu + 4.5 * cu * cu - 1.5 * (ux * ux + uy * uy));
    }
    ShiftK& h = P.shf[v];
    h.q0 = (float)(-om * sig[0]);
    double eff[9];
    eff[0] = -(double)h.q0 / om;
    for (int p = 0; p < 4; ++p) {
      const int a = first[p], b = second[p];
      h.qe[p] = (float)(-om * 0.5 * (sig[a] + sig[b]));
      h.qo[p] = (float)(-om * 0.5 * (sig[a] - sig[b]));
      eff[a] = -((double)h.qe[p] + (double)h.qo[p]) / om;
      eff[b] = -((double)h.qe[p] - (double)h.qo[p]) / om;
    }
    double S = 0.0, mx = 0.0, my = 0.0, oS = -(double)h.q0;
    for (int i = 0; i < 9; ++i) {
      h.sig[i] = (float)eff[i];
      S += eff[i];
      mx += cx(i) * eff[i];
      my += cy(i) * eff[i];
    }
    for (int p = 0; p < 4; ++p) oS -= 2.0 * (double)h.qe[p];
    h.S = (float)S;
    h.oS = (float)oS;
    h.sx = (float)mx;
    h.sy = (float)my;
  }
}

inline int check_omega(double omega) {
  if (!(omega > 0.0 && omega < 2.0)) return set_error(LBM_ERR_OMEGA, "omega must lie in (0, 2)");
  return LBM_OK;
}

inline int check_pitch(int nx, int64_t pitch) {
  if (pitch < nx || pitch % 8 != 0) return set_error(LBM_ERR_ARG, "pitch must be >= nx and a multiple of 8");
  return LBM_OK;
}

inline bool v2_fits(const KParams& P, int npt) {
  const int nx = P.g.nx;
  if (nx < npt + 2 || P.g.ny > 65535) return false;
  // the vectorised bodies give each node at most one pressure rewrite; on a
  // 3-column lattice column 1 is both nx-2 and 1 and owes two
  if (P.g.pressure && nx < 4) return false;
  if (9 * P.plane >= ((int64_t)1 << 31) || P.pitch % npt != 0 || P.pitch < (nx + npt - 1) / npt * npt) return false;
  if (((uintptr_t)P.pop_in | (uintptr_t)P.pop_out) % 16 != 0) return false;
  return true;
}


}  // namespace lbm
