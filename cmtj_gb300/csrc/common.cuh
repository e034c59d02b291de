// Shared host/device helpers of libcmtj_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cmtj_gpu.h"

// Records a printf-style message as the calling host thread's last error.
void cmtj_set_error(const char *fmt, ...);

// Checks a CUDA runtime call, recording the failing expression.
#define CMTJ_CUDA_TRY(expr)                                                            \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess) {                                                           \
      cmtj_set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, \
                     __LINE__);                                                        \
      return CMTJ_ERR_CUDA;                                                            \
    }                                                                                  \
  } while (0)

// Checks the launch that was just issued.
#define CMTJ_LAUNCH_CHECK(name)                                                          \
  do {                                                                                   \
    cudaError_t _e = cudaGetLastError();                                                 \
    if (_e != cudaSuccess) {                                                             \
      cmtj_set_error("launch of %s failed: %s", name, cudaGetErrorString(_e));           \
      return CMTJ_ERR_CUDA;                                                              \
    }                                                                                    \
  } while (0)

static inline cudaStream_t cmtj_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }
