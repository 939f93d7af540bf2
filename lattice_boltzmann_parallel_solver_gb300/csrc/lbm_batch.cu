// lbm_batch.cu -- many lattices of different sizes advanced by one launch per
// time step (the batched sweep and the serving loop run on it).
#include <algorithm>
#include <cstring>
#include <vector>

#include "lbm_fused.cuh"

namespace lbm {

// Tiles are handed out in groups of `group` consecutive tiles (mostly of one
// lattice), so the owner search and the staged entry are shared by the group;
// groups are strided over the persistent grid.  The launcher makes groups
// smaller when there are too few tiles to give every block several groups.
constexpr int kTileGroup = 8;

// registers capped so that 768 threads fit on an SM (the body with every
// boundary form compiled in needs more than the single-lattice kernels' 64)
template <int STORE, int NPT, int THREADS>
__global__ void __launch_bounds__(THREADS, (STORE == LBM_STORE_FX64 && NPT == 1) || STORE == LBM_STORE_F16S ||
                                                   STORE == LBM_STORE_BF16S
                                               ? 768 / THREADS
                                               : 1)
    batch_kernel(const BatchEntry* __restrict__ tab, const int* __restrict__ tile_start, int n_inst,
                 int total_tiles, const int* __restrict__ gbase, int k, int group) {
  // the current lattice's entry, staged in shared memory: the body reads its
  // parameters many times per tile, and in global memory the streaming
  // population traffic would evict them from L1
  static_assert(sizeof(BatchEntry) % 16 == 0, "entry copied in 16-byte words");
  __shared__ __align__(16) unsigned char ebuf[sizeof(BatchEntry)];
  const BatchEntry& e = *reinterpret_cast<const BatchEntry*>(ebuf);
  int staged = -1;
  const int g = *gbase + k;
  const int groups = (total_tiles + group - 1) / group;
  for (int grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    const int t0 = grp * group, t1 = min(total_tiles, t0 + group);
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(tile_start + mid) <= t0) lo = mid;
      else hi = mid - 1;
    }
    int next = lo + 1 < n_inst ? __ldg(tile_start + lo + 1) : total_tiles;
    for (int tile = t0; tile < t1; ++tile) {
      while (tile >= next) {
        ++lo;
        next = lo + 1 < n_inst ? __ldg(tile_start + lo + 1) : total_tiles;
      }
      if (lo != staged) {
        __syncthreads();  // every thread is done with the previous entry
        const uint4* src = reinterpret_cast<const uint4*>(tab + lo);
        uint4* dst = reinterpret_cast<uint4*>(ebuf);
        for (int w = threadIdx.x; w < (int)(sizeof(BatchEntry) / 16); w += THREADS) dst[w] = __ldg(src + w);
        __syncthreads();
        staged = lo;
      }
      if (g < e.s0 || g >= e.s_end) continue;
      const int local = tile - __ldg(tile_start + lo);
      const int yb = local / e.xblocks, xb = local - yb * e.xblocks;
      const bool odd = (g - e.s0) & 1;
      const void* pin = odd ? e.pop_b : e.pop_a;
      void* pout = odd ? e.pop_a : e.pop_b;
      const void* ain = odd ? e.aux_b : e.aux_a;
      void* aout = odd ? e.aux_a : e.aux_b;
      const int x0 = (xb * THREADS + threadIdx.x) * NPT;
      const uint32_t seed = hash32(e.P.seed + (uint32_t)(g - e.s0));
      const int y1 = min((yb + 1) * e.rows, e.P.g.ny);
      // lattices without the pressure rewrite take the body without it
      const bool pressure = e.P.g.pressure != 0;
      for (int y = yb * e.rows; y < y1; ++y) {
        if constexpr (STORE == LBM_STORE_FX64) {
          if (pressure) fused_fx_body<NPT, true, true>(e.P, pin, pout, ain, aout, x0, y);
          else fused_fx_body<NPT, true, false>(e.P, pin, pout, ain, aout, x0, y);
        } else {
          if (pressure) fused_v2_body<STORE, NPT, true, true>(e.P, pin, pout, ain, aout, x0, y, seed);
          else fused_v2_body<STORE, NPT, true, false>(e.P, pin, pout, ain, aout, x0, y, seed);
        }
      }
    }
  }
}

__global__ void batch_advance_kernel(int* gbase, int k) { *gbase += k; }

}  // namespace lbm

using namespace lbm;

extern "C" {

size_t lbm_batch_table_bytes(int32_t n) {
  return (size_t)n * sizeof(BatchEntry) + (size_t)n * sizeof(int) + 256;
}

int lbm_batch_build(const lbm_batch_lattice* lat, int32_t n, int32_t npt, int32_t threads, void* table,
                    size_t table_bytes, int32_t* total_tiles, void* stream) {
  if (lat == nullptr || n < 1 || table == nullptr || total_tiles == nullptr)
    return set_error(LBM_ERR_ARG, "bad batch arguments");
  if (table_bytes < lbm_batch_table_bytes(n)) return set_error(LBM_ERR_ARG, "batch table buffer too small");
  if (!(npt == 1 || npt == 2 || npt == 4 || npt == 8) || !(threads == 64 || threads == 128 || threads == 256))
    return set_error(LBM_ERR_ARG, "npt must be 1, 2, 4 or 8 and threads 64, 128 or 256");
  if ((uintptr_t)table % 16 != 0) return set_error(LBM_ERR_ARG, "batch table must be 16-byte aligned");
  std::vector<BatchEntry> ent((size_t)n);
  std::vector<int> start((size_t)n);
  int64_t tiles = 0;
  for (int j = 0; j < n; ++j) {
    const lbm_batch_lattice& L = lat[j];
    BatchEntry& e = ent[(size_t)j];
    std::memset(&e, 0, sizeof(e));
    if (!to_geok(L.g, e.P.g)) return last_status();
    if (int st = check_omega(L.omega)) return st;
    if (int st = check_pitch(L.g->nx, L.pitch)) return st;
    if (L.pop_a == nullptr || L.pop_b == nullptr) return set_error(LBM_ERR_ARG, "batch lattice without buffers");
    if (L.g->outlet && (L.aux_a == nullptr || L.aux_b == nullptr))
      return set_error(LBM_ERR_ARG, "batch lattice with an outlet needs aux buffers");
    e.P.pitch = L.pitch;
    e.P.plane = L.pitch * L.g->ny;
    e.P.omega = L.omega;
    e.P.pop_in = L.pop_a;
    e.P.pop_out = L.pop_b;
    e.P.probe_x = L.probe_x;
    e.P.probe_y = L.probe_y;
    e.P.probe_cap = L.probe_cap;
    e.P.probe_buf = L.probe_buf;
    e.P.probe_count = L.probe_count;
    e.P.seed = L.seed;
    e.P.qc = fx::q_consts(L.omega);
    e.P.sr = (L.flags & LBM_FLAG_STOCHASTIC) != 0;
    if (L.probe_buf != nullptr && L.probe_count == nullptr)
      return set_error(LBM_ERR_ARG, "a probe needs its counter");
    if (!v2_fits(e.P, npt)) return set_error(LBM_ERR_UNSUPPORTED, "a batch lattice is too narrow or too large for npt");
    e.pop_a = L.pop_a;
    e.pop_b = L.pop_b;
    e.aux_a = L.aux_a;
    e.aux_b = L.aux_b;
    e.s0 = L.s0;
    e.s_end = L.s_end;
    const int chunks = (L.g->nx + npt - 1) / npt;
    e.xblocks = (chunks + threads - 1) / threads;
    e.rows = L.rows > 0 ? L.rows : 1;
    start[(size_t)j] = (int)tiles;
    tiles += (int64_t)e.xblocks * ((L.g->ny + e.rows - 1) / e.rows);
  }
  if (tiles >= ((int64_t)1 << 31)) return set_error(LBM_ERR_ARG, "too many tiles");
  char* dst = static_cast<char*>(table);
  cudaError_t err = cudaMemcpyAsync(dst, ent.data(), ent.size() * sizeof(BatchEntry), cudaMemcpyHostToDevice,
                                    (cudaStream_t)stream);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(dst + ent.size() * sizeof(BatchEntry), start.data(), start.size() * sizeof(int),
                          cudaMemcpyHostToDevice, (cudaStream_t)stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize((cudaStream_t)stream);
  if (err != cudaSuccess) return set_error(LBM_ERR_CUDA, cudaGetErrorString(err));
  *total_tiles = (int32_t)tiles;
  return LBM_OK;
}

}  // extern "C"

template <int STORE, int NPT, int THREADS>
static int launch_batch(const void* table, int n, int tiles, int* gbase, int nsteps, int blocks, cudaStream_t s) {
  const BatchEntry* tab = static_cast<const BatchEntry*>(table);
  const int* start = reinterpret_cast<const int*>(static_cast<const char*>(table) + (size_t)n * sizeof(BatchEntry));
  if (blocks <= 0) {
    // resident blocks of this kernel on the whole GPU, queried on the first
    // call (make that call outside stream capture) and reused afterwards
    static int fill = 0;
    if (fill == 0) {
      int per_sm = 0, sms = 0, dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<STORE, NPT, THREADS>, THREADS, 0);
      fill = std::max(1, sms * std::max(1, per_sm));
    }
    blocks = fill;
  }
  // groups of up to kTileGroup tiles, but at least two groups per block
  const int group = std::max(1, std::min(kTileGroup, tiles / (2 * blocks)));
  blocks = std::min(blocks, std::max(1, (tiles + group - 1) / group));
  for (int k = 0; k < nsteps; ++k) {
    batch_kernel<STORE, NPT, THREADS><<<blocks, THREADS, 0, s>>>(tab, start, n, tiles, gbase, k, group);
    count_launch();
    if (int e = check_launch("batch_kernel")) return e;
  }
  batch_advance_kernel<<<1, 1, 0, s>>>(gbase, nsteps);
  count_launch();
  return check_launch("batch_advance_kernel");
}

extern "C" int lbm_batch_run(const void* table, int32_t n, int32_t total_tiles, int32_t storage, int32_t npt,
                             int32_t threads, int32_t* gbase, int32_t nsteps, int32_t blocks, void* stream) {
  if (table == nullptr || gbase == nullptr || n < 1 || total_tiles < 0 || nsteps < 0)
    return set_error(LBM_ERR_ARG, "bad batch run arguments");
  cudaStream_t s = (cudaStream_t)stream;
#define LBM_BATCH_CASE(ST, NP, TH) \
  if (storage == ST && npt == NP && threads == TH) return launch_batch<ST, NP, TH>(table, n, total_tiles, gbase, nsteps, blocks, s);
#define LBM_BATCH_NPT(ST, NP) LBM_BATCH_CASE(ST, NP, 64) LBM_BATCH_CASE(ST, NP, 128) LBM_BATCH_CASE(ST, NP, 256)
  LBM_BATCH_NPT(LBM_STORE_F64, 2)
  LBM_BATCH_NPT(LBM_STORE_F64, 4)
  LBM_BATCH_NPT(LBM_STORE_FX64, 1)
  LBM_BATCH_NPT(LBM_STORE_FX64, 2)
  LBM_BATCH_NPT(LBM_STORE_F32, 2)
  LBM_BATCH_NPT(LBM_STORE_F32, 4)
  LBM_BATCH_NPT(LBM_STORE_F16S, 2)
  LBM_BATCH_NPT(LBM_STORE_F16S, 4)
  LBM_BATCH_NPT(LBM_STORE_F16S, 8)
  LBM_BATCH_NPT(LBM_STORE_BF16S, 2)
  LBM_BATCH_NPT(LBM_STORE_BF16S, 4)
  LBM_BATCH_NPT(LBM_STORE_BF16S, 8)
#undef LBM_BATCH_NPT
#undef LBM_BATCH_CASE
  return set_error(LBM_ERR_UNSUPPORTED, "no batched kernel for this storage / npt / threads");
}


