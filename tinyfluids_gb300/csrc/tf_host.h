// Host-side helpers of the C ABI: error reporting and launch checks.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include "../../include/tinyfluids_gb300.h"

namespace tf {

// Records a message for tf_last_error() on this thread and returns `status`.
int set_error(int status, const char* fmt, ...);

inline int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return TF_OK;
  return set_error(TF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Status of the launches just enqueued.
inline int launch_check(const char* what) { return cuda_check(cudaGetLastError(), what); }

int sm_count();  // multiprocessors of the current device (cached per device)

}  // namespace tf

#define TF_TRY(expr)              \
  do {                            \
    int _st = (expr);             \
    if (_st != TF_OK) return _st; \
  } while (0)
