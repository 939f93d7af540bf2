// lbm_host.h -- host-side helpers shared by the C ABI translation units:
// per-thread error message, status codes and the launch counter.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lbm_gb300.h"

namespace lbm {
int set_error(int code, const char* msg);
int last_status();
int check_launch(const char* what);
void count_launch();
}  // namespace lbm
