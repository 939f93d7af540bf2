// lbm_reduce.cu -- exact global mass and momentum of a reference-layout state.
//
// Each population is turned into the 64-bit fixed-point value round(f 2^53)
// and summed in 128-bit integers, so the totals do not depend on the order of
// the additions: the same state always gives the same float64 result, on any
// grid shape.  This replaces host-side np.sum reductions of the reference's
// drivers (for example the mass checks of tests/test_mass_preservation.py and
// the flux areas of experiments.py:428-431) without a host round trip.
#include <algorithm>
#include <cstring>

#include "lbm_fx.cuh"
#include "lbm_host.h"

namespace lbm {

constexpr int kRedThreads = 256;

__device__ __forceinline__ void acc_add(unsigned long long& lo, long long& hi, long long v) {
  const unsigned long long n = lo + (unsigned long long)v;
  hi += (v < 0 ? -1LL : 0LL) + (n < lo ? 1LL : 0LL);
  lo = n;
}

// per-block 128-bit partial sums of rho, jx, jy, and a flag for values outside
// the fixed-point range
__global__ void __launch_bounds__(kRedThreads) reduce_partial_kernel(const double* __restrict__ f, int64_t n,
                                                                       unsigned long long* __restrict__ part,
                                                                       int* __restrict__ bad) {
  unsigned long long lo[3] = {0, 0, 0};
  long long hi[3] = {0, 0, 0};
  for (int64_t k = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; k < n; k += (int64_t)gridDim.x * kRedThreads) {
    int64_t F[9];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 9; ++i) ok &= fx::to_fixed(f[k * 9 + i], F[i]);
    if (!ok) {
      atomicOr(bad, 1);
      continue;
    }
    acc_add(lo[0], hi[0], ((F[0] + F[1]) + (F[2] + F[3])) + ((F[4] + F[5]) + (F[6] + F[7])) + F[8]);
    acc_add(lo[1], hi[1], (F[1] + F[5] + F[8]) - (F[3] + F[6] + F[7]));
    acc_add(lo[2], hi[2], (F[2] + F[5] + F[6]) - (F[4] + F[7] + F[8]));
  }
  __shared__ unsigned long long slo[3][kRedThreads];
  __shared__ long long shi[3][kRedThreads];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    slo[c][threadIdx.x] = lo[c];
    shi[c][threadIdx.x] = hi[c];
  }
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        unsigned long long a = slo[c][threadIdx.x];
        long long h = shi[c][threadIdx.x] + shi[c][threadIdx.x + s];
        const unsigned long long b = slo[c][threadIdx.x + s];
        const unsigned long long sum = a + b;
        h += sum < a ? 1 : 0;
        slo[c][threadIdx.x] = sum;
        shi[c][threadIdx.x] = h;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      part[(size_t)blockIdx.x * 6 + 2 * c] = slo[c][0];
      part[(size_t)blockIdx.x * 6 + 2 * c + 1] = (unsigned long long)shi[c][0];
    }
  }
}

// 128-bit total / 2^53 -> float64 (within one unit in the last place)
__device__ double i128_to_double(unsigned long long lo, long long hi) {
  const bool neg = hi < 0;
  if (neg) {  // two's complement negate
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0 ? 1 : 0);
  }
  const double r = ((double)(unsigned long long)hi * 18446744073709551616.0 + (double)lo) * 1.1102230246251565e-16;
  return neg ? -r : r;
}

__global__ void reduce_final_kernel(const unsigned long long* __restrict__ part, int nblocks, const int* bad,
                                    double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int c = 0; c < 3; ++c) {
    unsigned long long lo = 0;
    long long hi = 0;
    for (int b = 0; b < nblocks; ++b) {
      const unsigned long long v = part[(size_t)b * 6 + 2 * c];
      const unsigned long long s = lo + v;
      hi += (long long)part[(size_t)b * 6 + 2 * c + 1] + (s < lo ? 1 : 0);
      lo = s;
    }
    out[c] = *bad ? __longlong_as_double(0x7ff8000000000000LL) : i128_to_double(lo, hi);
  }
}

}  // namespace lbm

using namespace lbm;

extern "C" {

size_t lbm_reduce_scratch_bytes(int64_t n_nodes) {
  (void)n_nodes;
  return (size_t)1024 * 6 * sizeof(unsigned long long) + 256;
}

int lbm_reduce_moments_f64(const double* f, int64_t n_nodes, void* scratch, size_t scratch_bytes, double* out,
                           void* stream) {
  if (f == nullptr || out == nullptr || scratch == nullptr || n_nodes < 1)
    return set_error(LBM_ERR_ARG, "bad reduction arguments");
  if (scratch_bytes < lbm_reduce_scratch_bytes(n_nodes)) return set_error(LBM_ERR_ARG, "reduction scratch too small");
  const int blocks = (int)std::min<int64_t>(1024, (n_nodes + kRedThreads - 1) / kRedThreads);
  unsigned long long* part = static_cast<unsigned long long*>(scratch);
  int* bad = reinterpret_cast<int*>(part + 1024 * 6);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(int), s);
  if (e != cudaSuccess) return set_error(LBM_ERR_CUDA, cudaGetErrorString(e));
  reduce_partial_kernel<<<blocks, kRedThreads, 0, s>>>(f, n_nodes, part, bad);
  count_launch();
  if (int st = check_launch("reduce_partial_kernel")) return st;
  reduce_final_kernel<<<1, 32, 0, s>>>(part, blocks, bad, out);
  count_launch();
  return check_launch("reduce_final_kernel");
}

}  // extern "C"
