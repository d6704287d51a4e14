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

// Programmatic dependent launch: the kernel may start while the previous
// kernel of the stream finishes; it must call pdl_wait() before it reads or
// writes anything that kernel (or an earlier one) touches.  Only the work
// before the wait (loading plan tables into shared memory, index set-up)
// overlaps the predecessor's tail.  Launched without the attribute, the
// wait returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
