// lbm_batch_inline.cu -- batched steps with the boundary sources applied inside
// the step (one launch per step).
#include "lbm_batch.cuh"

namespace lbm {

int batch_launch_inline(const void* table, int n, int tiles, int bc_chunks, int storage, int npt, int threads,
                        int* gbase, int nsteps, int blocks, cudaStream_t s) {
  LBM_BATCH_DISPATCH(true);
}

}  // namespace lbm
