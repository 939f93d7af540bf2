// lbm_batch_split.cu -- batched steps as a boundary-free step followed by the
// boundary-node pass.
#include "lbm_batch.cuh"

namespace lbm {

int batch_launch_split(const void* table, int n, int tiles, int bc_chunks, int storage, int npt, int threads,
                       int* gbase, int nsteps, int blocks, cudaStream_t s) {
  LBM_BATCH_DISPATCH(false);
}

}  // namespace lbm
