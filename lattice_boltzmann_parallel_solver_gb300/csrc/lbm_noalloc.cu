// lbm_noalloc.cu -- the fused drop-in step for callers that cannot allocate
// device memory.
//
// lbm_step_f64 needs a scratch buffer for the collided populations between
// its two kernels, and asks the caller for it.  Some callers cannot provide
// one: code that runs where cudaMalloc is forbidden or unavailable (inside a
// host callback or another library's critical section, under an allocator
// that has handed all memory to a pool it owns, or in a plugin whose host
// application gives it no allocator).  lbm_step_f64_noalloc serves them from
// a fixed scratch array compiled into this library instead.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds LBM_NOALLOC_SCRATCH_BYTES of it until the process exits.  Its
// address is looked up once per device with cudaGetSymbolAddress (host code
// cannot use the symbol itself as a device pointer).  Every call on a device
// shares the same array, so calls that overlap on the GPU (different streams,
// or threads with no ordering between their streams) race on it.
#include <cstdio>
#include <mutex>

#include "lbm_host.h"

namespace {

// [9][ny][pitch] collided populations, then [3][ny] outlet column, float64
__device__ __align__(256) unsigned char g_noalloc_scratch[LBM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Address of g_noalloc_scratch on the current device, looked up on first use.
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "cudaGetDevice: %s", cudaGetErrorString(e));
    return lbm::set_error(LBM_ERR_CUDA, buf);
  }
  if (dev < 0 || dev >= kMaxDevices) return lbm::set_error(LBM_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (g_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      char buf[256];
      std::snprintf(buf, sizeof(buf), "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
      return lbm::set_error(LBM_ERR_CUDA, buf);
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return LBM_OK;
}

}  // namespace

extern "C" int lbm_step_f64_noalloc(const lbm_geometry* g, const double* f, const double* rho, const double* u,
                                    double omega, double* f_out, double* rho_out, double* u_out, int32_t flags,
                                    void* stream) {
  if (g == nullptr) return lbm::set_error(LBM_ERR_ARG, "geometry is NULL");
  if (g->nx < 1 || g->ny < 1) return lbm::set_error(LBM_ERR_ARG, "nx and ny must be >= 1");
  if (f == nullptr || rho == nullptr || u == nullptr || f_out == nullptr || rho_out == nullptr || u_out == nullptr)
    return lbm::set_error(LBM_ERR_ARG, "f, rho, u, f_out, rho_out and u_out are required");
  const int64_t pitch = ((int64_t)g->nx + 31) / 32 * 32;
  const int64_t need = (9 * pitch * g->ny + 3 * (int64_t)g->ny) * (int64_t)sizeof(double);
  if (need > (int64_t)LBM_NOALLOC_SCRATCH_BYTES) {
    char buf[256];
    std::snprintf(buf, sizeof(buf),
                  "a %d x %d lattice needs %lld bytes of scratch, more than the %lld-byte static scratch of "
                  "lbm_step_f64_noalloc; use lbm_step_f64 with a caller-allocated scratch buffer",
                  g->nx, g->ny, (long long)need, (long long)LBM_NOALLOC_SCRATCH_BYTES);
    return lbm::set_error(LBM_ERR_ARG, buf);
  }
  void* base = nullptr;
  if (int e = scratch_address(&base)) return e;
  // Every scratch element the read-out kernel reads is written by the
  // collision kernel earlier in this call, so nothing needs clearing.
  double* pop = static_cast<double*>(base);
  double* aux = g->outlet ? pop + 9 * pitch * g->ny : nullptr;
  if (int e = lbm_lattice_init(g, LBM_STORE_F64, f, rho, u, omega, pop, pitch, aux, flags, stream)) return e;
  return lbm_lattice_read(g, LBM_STORE_F64, pop, pitch, aux, f_out, rho_out, u_out, stream);
}
