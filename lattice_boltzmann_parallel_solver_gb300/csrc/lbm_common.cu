// lbm_common.cu -- library version, per-thread error state and launch counter.
#include <cstdio>
#include <cstring>

#include "lbm_host.h"

namespace lbm {
namespace {
thread_local char g_msg[512] = "";
thread_local int g_status = LBM_OK;
thread_local int64_t g_launches = 0;
}  // namespace

int set_error(int code, const char* msg) {
  g_status = code;
  std::snprintf(g_msg, sizeof(g_msg), "%s", msg);
  return code;
}

int last_status() { return g_status; }

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return set_error(LBM_ERR_CUDA, buf);
  }
  return LBM_OK;
}

void count_launch() { ++g_launches; }
}  // namespace lbm

extern "C" {
int lbm_version(void) { return 10000; }
const char* lbm_last_error(void) { return lbm::g_msg; }
int64_t lbm_launch_count(int reset) {
  int64_t n = lbm::g_launches;
  if (reset) lbm::g_launches = 0;
  return n;
}
}
