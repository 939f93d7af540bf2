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
// address is looked up with cudaGetSymbolAddress (host code cannot use the
// symbol itself as a device pointer) once per device context and cached under
// the context's unique id, so a context created later on the same device
// (after cudaDeviceReset, or another driver context made current) gets a
// fresh lookup instead of an address that belonged to the old one.  Every call
// in a context shares the same array, so calls that overlap on the GPU
// (different streams, or threads with no ordering between their streams) race
// on it.
#include <cuda.h>

#include <cstdio>
#include <mutex>

#include "lbm_host.h"

namespace {

// [9][ny][pitch] collided populations, then [3][ny] outlet column, float64
__device__ __align__(256) unsigned char g_noalloc_scratch[LBM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxContexts = 64;
std::mutex g_mutex;
unsigned long long g_ctx_id[kMaxContexts] = {};
void* g_scratch_addr[kMaxContexts] = {};
int g_next = 0;

using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrent g_get_current = nullptr;
CtxGetId g_get_id = nullptr;

int cuda_error(const char* what, cudaError_t e) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return lbm::set_error(LBM_ERR_CUDA, buf);
}

// unique id of the current driver context (0 when none is current yet);
// the driver functions come through the runtime, so no driver library is linked
int current_context_id(unsigned long long* id) {
  if (g_get_current == nullptr || g_get_id == nullptr) {
    cudaDriverEntryPointQueryResult q1, q2;
    void* a = nullptr;
    void* b = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &q1);
    if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !a || !b)
      return lbm::set_error(LBM_ERR_CUDA, "cuCtxGetCurrent / cuCtxGetId not available from the driver");
    g_get_current = reinterpret_cast<CtxGetCurrent>(a);
    g_get_id = reinterpret_cast<CtxGetId>(b);
  }
  CUcontext ctx = nullptr;
  if (g_get_current(&ctx) != CUDA_SUCCESS) return lbm::set_error(LBM_ERR_CUDA, "cuCtxGetCurrent failed");
  *id = 0;
  if (ctx != nullptr && g_get_id(ctx, id) != CUDA_SUCCESS) return lbm::set_error(LBM_ERR_CUDA, "cuCtxGetId failed");
  return LBM_OK;
}

// Address of g_noalloc_scratch in the current context, looked up on first use
// in that context.
int scratch_address(void** out) {
  std::lock_guard<std::mutex> lock(g_mutex);
  unsigned long long id = 0;
  if (int e = current_context_id(&id)) return e;
  if (id != 0)
    for (int k = 0; k < kMaxContexts; ++k)
      if (g_ctx_id[k] == id) {
        *out = g_scratch_addr[k];
        return LBM_OK;
      }
  // first use in this context: the lookup also makes the device's primary
  // context current when no context is yet
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr) return cuda_error("cudaGetSymbolAddress(scratch)", e);
  if (id == 0)
    if (int st = current_context_id(&id)) return st;
  if (id != 0) {
    g_ctx_id[g_next] = id;
    g_scratch_addr[g_next] = p;
    g_next = (g_next + 1) % kMaxContexts;
  }
  *out = p;
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
