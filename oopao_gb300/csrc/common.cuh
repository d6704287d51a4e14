// Shared helpers for the oopao_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/oopao_gb300.h"

#define OOPAO_CUDA_TRY(expr)                                  \
  do {                                                        \
    cudaError_t _e = (expr);                                  \
    if (_e != cudaSuccess) {                                  \
      oopao_set_last_error(cudaGetErrorString(_e), __FILE__, __LINE__); \
      return OOPAO_ERR_CUDA;                                  \
    }                                                         \
  } while (0)

#define OOPAO_CHECK_ARG(cond, msg)                            \
  do {                                                        \
    if (!(cond)) {                                            \
      oopao_set_last_error(msg, __FILE__, __LINE__);          \
      return OOPAO_ERR_INVALID;                               \
    }                                                         \
  } while (0)

// Records a message for oopao_last_error(); thread-local.
void oopao_set_last_error(const char* msg, const char* file, int line);
// Adds n to the process-wide kernel-launch counter (oopao_launch_count).
void oopao_count_launches(int n);

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float cabs2(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }

static inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
