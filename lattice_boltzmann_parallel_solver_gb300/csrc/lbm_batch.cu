// lbm_batch.cu -- the batch work table and the C ABI of the batched steps
// (kernels in lbm_batch.cuh).
#include <cstring>
#include <vector>

#include "lbm_batch.cuh"

using namespace lbm;

extern "C" {

size_t lbm_batch_table_bytes(int32_t n) {
  return (size_t)n * sizeof(BatchEntry) + 2 * (size_t)n * sizeof(int) + 256;
}

int lbm_batch_build(const lbm_batch_lattice* lat, int32_t n, int32_t npt, int32_t threads, void* table,
                    size_t table_bytes, int32_t* total_tiles, int32_t* bc_chunks, void* stream) {
  if (lat == nullptr || n < 1 || table == nullptr || total_tiles == nullptr || bc_chunks == nullptr)
    return set_error(LBM_ERR_ARG, "bad batch arguments");
  if (table_bytes < lbm_batch_table_bytes(n)) return set_error(LBM_ERR_ARG, "batch table buffer too small");
  if (!(npt == 1 || npt == 2 || npt == 4 || npt == 8) || !(threads == 64 || threads == 128 || threads == 256))
    return set_error(LBM_ERR_ARG, "npt must be 1, 2, 4 or 8 and threads 64, 128 or 256");
  if ((uintptr_t)table % 16 != 0) return set_error(LBM_ERR_ARG, "batch table must be 16-byte aligned");
  std::vector<BatchEntry> ent((size_t)n);
  std::vector<int> start((size_t)n), bc_start((size_t)n);
  int64_t tiles = 0, chunks_bc = 0, nodes = 0;
  bool inline_bc = false;  // some lattice has boundary nodes but no list of them
  bool force_split = false;
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
    set_shift(e.P);
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
    e.cpr = (L.g->nx + npt - 1) / npt;
    e.cpr_magic = e.cpr == 1 ? 0xFFFFFFFFu : (uint32_t)((1ull << 32) / (uint64_t)e.cpr);
    e.xblocks = (e.cpr + threads - 1) / threads;
    e.rows = L.rows > 0 ? L.rows : 1;
    if (e.P.g.bcmask != nullptr && (e.P.g.n_bcnodes == 0 || (L.flags & LBM_FLAG_BC_INLINE))) inline_bc = true;
    if (L.flags & LBM_FLAG_BC_SPLIT) force_split = true;
    nodes += (int64_t)L.g->nx * L.g->ny;
    bc_start[(size_t)j] = (int)chunks_bc;
    chunks_bc += (pass_nodes(e.P.g) + kFixupChunk - 1) / kFixupChunk;
  }
  // small batches keep one launch per step (the pass would double their fixed cost)
  if (nodes < kBatchSplitNodes && !force_split) inline_bc = true;
  // tiles: runs across row ends with the pass, row segments without it
  for (int j = 0; j < n; ++j) {
    const BatchEntry& e = ent[(size_t)j];
    start[(size_t)j] = (int)tiles;
    if (inline_bc) {
      tiles += (int64_t)e.xblocks * ((e.P.g.ny + e.rows - 1) / e.rows);
    } else {
      const int64_t run = (int64_t)threads * e.rows;
      tiles += ((int64_t)e.cpr * e.P.g.ny + run - 1) / run;
    }
  }
  if (tiles >= ((int64_t)1 << 31) || chunks_bc >= ((int64_t)1 << 31))
    return set_error(LBM_ERR_ARG, "too many tiles");
  char* dst = static_cast<char*>(table);
  const size_t eb = ent.size() * sizeof(BatchEntry), ib = (size_t)n * sizeof(int);
  cudaError_t err = cudaMemcpyAsync(dst, ent.data(), eb, cudaMemcpyHostToDevice, (cudaStream_t)stream);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(dst + eb, start.data(), ib, cudaMemcpyHostToDevice, (cudaStream_t)stream);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(dst + eb + ib, bc_start.data(), ib, cudaMemcpyHostToDevice, (cudaStream_t)stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize((cudaStream_t)stream);
  if (err != cudaSuccess) return set_error(LBM_ERR_CUDA, cudaGetErrorString(err));
  *total_tiles = (int32_t)tiles;
  *bc_chunks = inline_bc ? -1 : (int32_t)chunks_bc;
  return LBM_OK;
}

}  // extern "C"

extern "C" int lbm_batch_run(const void* table, int32_t n, int32_t total_tiles, int32_t bc_chunks, int32_t storage,
                             int32_t npt, int32_t threads, int32_t* gbase, int32_t nsteps, int32_t blocks,
                             void* stream) {
  if (table == nullptr || gbase == nullptr || n < 1 || total_tiles < 0 || nsteps < 0)
    return set_error(LBM_ERR_ARG, "bad batch run arguments");
  cudaStream_t s = (cudaStream_t)stream;
  if (bc_chunks >= 0)
    return batch_launch_split(table, n, total_tiles, bc_chunks, storage, npt, threads, gbase, nsteps, blocks, s);
  return batch_launch_inline(table, n, total_tiles, bc_chunks, storage, npt, threads, gbase, nsteps, blocks, s);
}
