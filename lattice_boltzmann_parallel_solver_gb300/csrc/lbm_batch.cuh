// lbm_batch.cuh -- the batched step kernels and their launcher (many lattices
// of different sizes advanced together, one or two launches per time step).
// Two translation units instantiate the launcher: lbm_batch_inline.cu
// (boundary sources inside the step) and lbm_batch_split.cu (boundary-free
// step + boundary-node pass).
#pragma once
#include <algorithm>
#include <cstddef>

#include "lbm_fused.cuh"

namespace lbm {

// Registers: the boundary-free 16-bit bodies and the one-node fixed-point body
// run at 1024 threads per SM (64 registers; the plain grid and the span walk
// keep little state across the body, 44 bytes of spill at 4 nodes per thread),
// the bodies with the boundary sources inside at 768; float32 at 2 nodes per
// thread without sources at 1024.
template <int STORE, int NPT, int THREADS, bool HAS_BC>
constexpr int batch_min_blocks() {
  if constexpr (STORE == LBM_STORE_F16S || STORE == LBM_STORE_BF16S || (STORE == LBM_STORE_FX64 && NPT == 1))
    return (HAS_BC ? 768 : 1024) / THREADS;
  else if constexpr (!HAS_BC && STORE == LBM_STORE_F32 && NPT <= 2)
    return 1024 / THREADS;
  else
    return 1;
}

// The entry's boundary constant tables (kconst, cconst: 2.3 KB of its 2.7 KB)
// are read only by the boundary sources; a body without them stages the 16-byte
// words before and after the tables.
constexpr int kEntryWords = (int)(sizeof(BatchEntry) / 16);
constexpr int kTablesFirst = (int)((offsetof(BatchEntry, P.g.kconst) + 15) / 16);  // first word inside the tables
constexpr int kTablesEnd = (int)(offsetof(BatchEntry, P.g.bcnodes) / 16);         // first word holding bytes after them
static_assert(offsetof(BatchEntry, P.g.cconst) == offsetof(BatchEntry, P.g.kconst) + sizeof(GeoK::kconst) &&
                  offsetof(BatchEntry, P.g.bcnodes) == offsetof(BatchEntry, P.g.cconst) + sizeof(GeoK::cconst),
              "the constant tables are contiguous, followed by bcnodes");

// stages lattice `lo`'s entry in the block's shared buffer (every thread of the
// block calls it with the same `lo`); TABLES: with the boundary constant tables
template <int THREADS, bool TABLES>
__device__ __forceinline__ void stage_entry(const BatchEntry* __restrict__ tab, int lo, unsigned char* ebuf) {
  static_assert(sizeof(BatchEntry) % 16 == 0, "entry copied in 16-byte words");
  __syncthreads();  // every thread is done with the previous entry
  const uint4* src = reinterpret_cast<const uint4*>(tab + lo);
  uint4* dst = reinterpret_cast<uint4*>(ebuf);
  constexpr int skip = TABLES ? 0 : kTablesEnd - kTablesFirst;
  for (int w = threadIdx.x; w < kEntryWords - skip; w += THREADS) {
    const int v = TABLES || w < kTablesFirst ? w : w + skip;
    dst[v] = __ldg(src + v);
  }
  __syncthreads();
}

// last index j in [0, n) with start[j] <= t (start ascending, start[0] == 0)
__device__ __forceinline__ int owner_of(const int* __restrict__ start, int n, int t) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(start + mid) <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One tile of lattice `e` (staged in shared memory) at global step g; SHIFT:
// the reference-shifted 16-bit storages.
template <int STORE, int NPT, int THREADS, bool HAS_BC, bool SHIFT>
__device__ __forceinline__ void batch_tile(const BatchEntry& e, int local, int g) {
  const bool odd = (g - e.s0) & 1;
  const void* pin = odd ? e.pop_b : e.pop_a;
  void* pout = odd ? e.pop_a : e.pop_b;
  const void* ain = odd ? e.aux_b : e.aux_a;
  void* aout = odd ? e.aux_a : e.aux_b;
  const uint32_t seed = hash32(e.P.seed + (uint32_t)(g - e.s0));
  // with the sources inside the step, lattices without the pressure rewrite
  // take the body without it; the boundary-free body leaves the rewrite to
  // the boundary-node pass
  const bool pressure = HAS_BC && e.P.g.pressure != 0;
  // the boundary-free body applies the plain inlet / outlet columns itself
  // (EDGES), the boundary-node pass the other boundary nodes
  auto step_chunk = [&](int x0, int y) {
    if constexpr (STORE == LBM_STORE_FX64) {
      if (pressure) fused_fx_body<NPT, HAS_BC, HAS_BC, !HAS_BC>(e.P, pin, pout, ain, aout, x0, y);
      else fused_fx_body<NPT, HAS_BC, false, !HAS_BC>(e.P, pin, pout, ain, aout, x0, y);
    } else {
      if (pressure) fused_v2_body<STORE, NPT, HAS_BC, HAS_BC, !HAS_BC, SHIFT>(e.P, pin, pout, ain, aout, x0, y, seed);
      else fused_v2_body<STORE, NPT, HAS_BC, false, !HAS_BC, SHIFT>(e.P, pin, pout, ain, aout, x0, y, seed);
    }
  };
  if constexpr (HAS_BC) {
    // row-segment tiles (small batches): `rows` rows of one segment of
    // THREADS chunks; the row is uniform over the block, so its addressing
    // runs in the uniform datapath (on a lone 420x180 lattice 15 % faster
    // than runs across row ends)
    const int yb = local / e.xblocks, xb = local - yb * e.xblocks;
    const int x0 = (xb * THREADS + (int)threadIdx.x) * NPT;
    const int y1 = min((yb + 1) * e.rows, e.P.g.ny);
    for (int y = yb * e.rows; y < y1; ++y) step_chunk(x0, y);
  } else {
    // runs of THREADS consecutive chunks, chunks numbered row by row: no
    // idle lanes at row ends.  The lanes of a run past the lattice's last
    // chunk stay idle (x0 = nx).  The body takes x0 and y per thread: at a
    // row end inside a warp the x neighbours come by direct loads.
    for (int r = 0; r < e.rows; ++r) {
      const int c = (local * e.rows + r) * THREADS + (int)threadIdx.x;
      const int cpr = e.cpr;
      int y = (int)__umulhi((uint32_t)c, e.cpr_magic);
      int xc = c - y * cpr;
      if (xc >= cpr) {
        xc -= cpr;
        ++y;
      }
      int x0 = xc * NPT;
      if (y >= e.P.g.ny) {
        y = e.P.g.ny - 1;
        x0 = e.P.g.nx;
      }
      step_chunk(x0, y);
    }
  }
}

// The persistent form: block b walks the contiguous span of tiles
// [b T / B, (b + 1) T / B) (T tiles, B blocks), so consecutive tiles mostly
// belong to one lattice: the owner search and the entry staging happen once per
// lattice the span touches, not once per tile, and the spans differ by at most
// one tile (no tail of partly filled waves).
template <int STORE, int NPT, int THREADS, bool HAS_BC, bool SHIFT>
__global__ void __launch_bounds__(THREADS, batch_min_blocks<STORE, NPT, THREADS, HAS_BC>())
    batch_kernel(const BatchEntry* __restrict__ tab, const int* __restrict__ tile_start, int n_inst,
                 int total_tiles, const int* __restrict__ gbase, int k) {
  // the current lattice's entry, staged in shared memory: the body reads its
  // parameters many times per tile, and in global memory the streaming
  // population traffic would evict them from L1
  __shared__ __align__(16) unsigned char ebuf[sizeof(BatchEntry)];
  const BatchEntry& e = *reinterpret_cast<const BatchEntry*>(ebuf);
  const int per = total_tiles / (int)gridDim.x, extra = total_tiles % (int)gridDim.x;
  const int b = (int)blockIdx.x;
  const int t0 = b * per + min(b, extra), t1 = t0 + per + (b < extra ? 1 : 0);
  if (t0 >= t1) return;
  const int g = *gbase + k;
  int lo = owner_of(tile_start, n_inst, t0);
  int first = __ldg(tile_start + lo);
  int next = lo + 1 < n_inst ? __ldg(tile_start + lo + 1) : total_tiles;
  stage_entry<THREADS, HAS_BC>(tab, lo, ebuf);
  for (int tile = t0; tile < t1; ++tile) {
    if (tile >= next) {
      do {
        ++lo;
        first = next;
        next = lo + 1 < n_inst ? __ldg(tile_start + lo + 1) : total_tiles;
      } while (tile >= next);
      stage_entry<THREADS, HAS_BC>(tab, lo, ebuf);
    }
    if (g >= e.s0 && g < e.s_end) batch_tile<STORE, NPT, THREADS, HAS_BC, SHIFT>(e, tile - first, g);
  }
}

// The plain-grid form (one tile per block, block b = tile b).  The block
// copies the lattices' tile starts into shared memory (one round trip) and
// finds its lattice there, instead of a search through global memory (a
// dependent L2 round trip per halving).
constexpr int kStartSmem = 512;

// owner_of for a whole block: the start list is copied into shared memory
// (one round trip) and searched there when it has at most kStartSmem entries
template <int THREADS>
__device__ __forceinline__ int owner_of_staged(const int* __restrict__ start, int n, int t) {
  __shared__ int sstart[kStartSmem];
  if (n > kStartSmem) return owner_of(start, n, t);
  for (int j = (int)threadIdx.x; j < n; j += THREADS) sstart[j] = __ldg(start + j);
  __syncthreads();
  int a = 0, b = n - 1;
  while (a < b) {
    const int mid = (a + b + 1) >> 1;
    if (sstart[mid] <= t) a = mid;
    else b = mid - 1;
  }
  return a;
}

template <int STORE, int NPT, int THREADS, bool HAS_BC, bool SHIFT>
__global__ void __launch_bounds__(THREADS, batch_min_blocks<STORE, NPT, THREADS, HAS_BC>())
    batch_grid_kernel(const BatchEntry* __restrict__ tab, const int* __restrict__ tile_start, int n_inst,
                      const int* __restrict__ gbase, int k) {
  __shared__ __align__(16) unsigned char ebuf[sizeof(BatchEntry)];
  const BatchEntry& e = *reinterpret_cast<const BatchEntry*>(ebuf);
  const int tile = (int)blockIdx.x;
  const int lo = owner_of_staged<THREADS>(tile_start, n_inst, tile);
  stage_entry<THREADS, HAS_BC>(tab, lo, ebuf);
  const int g = *gbase + k;
  if (g < e.s0 || g >= e.s_end) return;
  batch_tile<STORE, NPT, THREADS, HAS_BC, SHIFT>(e, tile - __ldg(tile_start + lo), g);
}

// The batched boundary-node pass: after batch_kernel<..., false> stepped every
// node of every live lattice without boundary sources or pressure rewrite
// (but with the plain inlet / outlet columns), one thread per pass node
// recomputes that node with them and overwrites its outputs (the body at one
// node per thread, the same arithmetic and random bits as the in-step
// sources).  A lattice's pass nodes are its listed boundary nodes other than
// the plain edge nodes, then, under the pressure rewrite, columns 1 and nx-2 of
// every row (those not listed already), whose nodes write the rewritten
// populations of columns nx-1 and 0.  Block b takes chunk b of the chunk list: lattice j owns
// chunks [bc_start[j], bc_start[j + 1]) of kFixupChunk pass nodes.
constexpr int kFixupChunk = 128;

// batches below this many nodes in total keep the sources inside one launch
// per step (a second launch per step would double a small batch's fixed cost)
constexpr int64_t kBatchSplitNodes = (int64_t)1 << 20;

inline int64_t pass_nodes(const GeoK& g) {
  return (g.bcmask != nullptr ? (int64_t)(g.n_bcnodes - g.n_bcnodes_edge) : 0) + (g.pressure ? 2 * (int64_t)g.ny : 0);
}

// 64 registers: 8 blocks of the latency-bound pass per SM (f16 takes 66
// without the cap, 7 blocks); the fixed-point body would spill under it
template <int STORE, bool SHIFT>
__global__ void __launch_bounds__(kFixupChunk, STORE == LBM_STORE_FX64 ? 1 : 8)
    batch_fixup_kernel(const BatchEntry* __restrict__ tab, const int* __restrict__ bc_start, int n_inst,
                       const int* __restrict__ gbase, int k) {
  __shared__ __align__(16) unsigned char ebuf[sizeof(BatchEntry)];
  const BatchEntry& e = *reinterpret_cast<const BatchEntry*>(ebuf);
  const int g = *gbase + k;
  const int j = owner_of_staged<kFixupChunk>(bc_start, n_inst, (int)blockIdx.x);
  stage_entry<kFixupChunk, true>(tab, j, ebuf);
  if (g < e.s0 || g >= e.s_end) return;
  const int t = ((int)blockIdx.x - __ldg(bc_start + j)) * kFixupChunk + (int)threadIdx.x;
  const int nx = e.P.g.nx;
  const int listed = e.P.g.bcmask != nullptr ? e.P.g.n_bcnodes - e.P.g.n_bcnodes_edge : 0;
  int x, y;
  if (t < listed) {
    const int node = __ldg(e.P.g.bcnodes + t);
    y = node / nx;
    x = node - y * nx;
  } else {
    // a pressure column node: (1, y) for even q, (nx-2, y) for odd q
    const int q = t - listed;
    if (!e.P.g.pressure || q >= 2 * e.P.g.ny) return;
    y = q >> 1;
    x = (q & 1) ? nx - 2 : 1;
    if ((q & 1) && nx - 2 == 1) return;  // one column: its even entry covers it
    if (e.P.g.bcmask != nullptr && ((__ldg(e.P.g.bcmask + y * e.P.g.words + (x >> 5)) >> (x & 31)) & 1u) &&
        !plain_edge_node(e.P, x, y))
      return;  // listed already
  }
  const bool odd = (g - e.s0) & 1;
  const void* pin = odd ? e.pop_b : e.pop_a;
  void* pout = odd ? e.pop_a : e.pop_b;
  const void* ain = odd ? e.aux_b : e.aux_a;
  void* aout = odd ? e.aux_a : e.aux_b;
  if constexpr (STORE == LBM_STORE_FX64) {
    if (e.P.g.pressure) fused_fx_body<1, true, true>(e.P, pin, pout, ain, aout, x, y);
    else fused_fx_body<1, true, false>(e.P, pin, pout, ain, aout, x, y);
  } else {
    const uint32_t seed = hash32(e.P.seed + (uint32_t)(g - e.s0));
    const bool in_list = t < listed;
    if (e.P.g.pressure)
      fused_v2_body<STORE, 1, true, true, false, SHIFT>(e.P, pin, pout, ain, aout, x, y, seed, in_list);
    else
      fused_v2_body<STORE, 1, true, false, false, SHIFT>(e.P, pin, pout, ain, aout, x, y, seed, in_list);
  }
}

// one copy per translation unit (each unit launches its own)
static __global__ void batch_advance_kernel(int* gbase, int k) { *gbase += k; }

template <int STORE, int NPT, int THREADS, bool HAS_BC, bool SHIFT = false>
inline int launch_batch(const void* table, int n, int tiles, int bc_chunks, int* gbase, int nsteps, int blocks,
                        cudaStream_t s) {
  const BatchEntry* tab = static_cast<const BatchEntry*>(table);
  const int* start = reinterpret_cast<const int*>(static_cast<const char*>(table) + (size_t)n * sizeof(BatchEntry));
  const int* bc_start = start + n;
  if (blocks <= 0) {
    // resident blocks of this kernel on the whole GPU, queried on the first
    // call (make that call outside stream capture) and reused afterwards
    static int fill = 0;
    if (fill == 0) {
      int per_sm = 0, sms = 0, dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<STORE, NPT, THREADS, HAS_BC, SHIFT>,
                                                    THREADS, 0);
      fill = std::max(1, sms * std::max(1, per_sm));
    }
    blocks = fill;
  }
  // a grid of more than half the tile count is a plain grid of one tile per
  // block; otherwise persistent blocks walk contiguous spans of tiles
  const bool plain = (int64_t)blocks * 2 > (int64_t)tiles;
  blocks = std::min(blocks, std::max(1, tiles));
  for (int k = 0; k < nsteps; ++k) {
    if (plain && tiles > 0) {
      batch_grid_kernel<STORE, NPT, THREADS, HAS_BC, SHIFT><<<tiles, THREADS, 0, s>>>(tab, start, n, gbase, k);
      count_launch();
      if (int e = check_launch("batch_grid_kernel")) return e;
    } else {
      batch_kernel<STORE, NPT, THREADS, HAS_BC, SHIFT><<<blocks, THREADS, 0, s>>>(tab, start, n, tiles, gbase, k);
      count_launch();
      if (int e = check_launch("batch_kernel")) return e;
    }
    if (!HAS_BC && bc_chunks > 0) {
      batch_fixup_kernel<STORE, SHIFT><<<bc_chunks, kFixupChunk, 0, s>>>(tab, bc_start, n, gbase, k);
      count_launch();
      if (int e = check_launch("batch_fixup_kernel")) return e;
    }
  }
  batch_advance_kernel<<<1, 1, 0, s>>>(gbase, nsteps);
  count_launch();
  return check_launch("batch_advance_kernel");
}


// dispatch over (storage, npt, threads) to launch_batch<..., HAS_BC>
int batch_launch_inline(const void* table, int n, int tiles, int bc_chunks, int storage, int npt, int threads,
                        int* gbase, int nsteps, int blocks, cudaStream_t s);
int batch_launch_split(const void* table, int n, int tiles, int bc_chunks, int storage, int npt, int threads,
                       int* gbase, int nsteps, int blocks, cudaStream_t s);

#define LBM_BATCH_DISPATCH(HAS_BC)                                                                           \
  do {                                                                                                       \
    LBM_BATCH_NPT(LBM_STORE_F64, 2, HAS_BC)                                                                  \
    LBM_BATCH_NPT(LBM_STORE_F64, 4, HAS_BC)                                                                  \
    LBM_BATCH_NPT(LBM_STORE_FX64, 1, HAS_BC)                                                                 \
    LBM_BATCH_NPT(LBM_STORE_FX64, 2, HAS_BC)                                                                 \
    LBM_BATCH_NPT(LBM_STORE_F32, 2, HAS_BC)                                                                  \
    LBM_BATCH_NPT(LBM_STORE_F32, 4, HAS_BC)                                                                  \
    LBM_BATCH_NPT(LBM_STORE_F16S, 2, HAS_BC)                                                                 \
    LBM_BATCH_NPT(LBM_STORE_F16S, 4, HAS_BC)                                                                 \
    LBM_BATCH_NPT(LBM_STORE_F16S, 8, HAS_BC)                                                                 \
    LBM_BATCH_NPT(LBM_STORE_BF16S, 2, HAS_BC)                                                                \
    LBM_BATCH_NPT(LBM_STORE_BF16S, 4, HAS_BC)                                                                \
    LBM_BATCH_NPT(LBM_STORE_BF16S, 8, HAS_BC)                                                                \
    LBM_BATCH_REF(LBM_STORE_F16R, LBM_STORE_F16S, 2, HAS_BC)                                                 \
    LBM_BATCH_REF(LBM_STORE_F16R, LBM_STORE_F16S, 4, HAS_BC)                                                 \
    LBM_BATCH_REF(LBM_STORE_BF16R, LBM_STORE_BF16S, 2, HAS_BC)                                               \
    LBM_BATCH_REF(LBM_STORE_BF16R, LBM_STORE_BF16S, 4, HAS_BC)                                               \
    return set_error(LBM_ERR_UNSUPPORTED, "no batched kernel for this storage / npt / threads");              \
  } while (0)
#define LBM_BATCH_CASE(ST, NP, TH, HAS_BC)               \
  if (storage == ST && npt == NP && threads == TH)       \
    return launch_batch<ST, NP, TH, HAS_BC>(table, n, tiles, bc_chunks, gbase, nsteps, blocks, s);
// the reference-shifted storages: 128 threads only
#define LBM_BATCH_REF(ST, BASE, NP, HAS_BC)                  \
  if (storage == ST && npt == NP && threads == 128)          \
    return launch_batch<BASE, NP, 128, HAS_BC, true>(table, n, tiles, bc_chunks, gbase, nsteps, blocks, s);
#define LBM_BATCH_NPT(ST, NP, HAS_BC) \
  LBM_BATCH_CASE(ST, NP, 64, HAS_BC) LBM_BATCH_CASE(ST, NP, 128, HAS_BC) LBM_BATCH_CASE(ST, NP, 256, HAS_BC)

}  // namespace lbm
