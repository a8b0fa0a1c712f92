// Shared definitions for the mermake_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mermake_gb300.h"

#define MM_CUDA_TRY(expr)                                                   \
    do {                                                                    \
        cudaError_t _e = (expr);                                            \
        if (_e != cudaSuccess) {                                            \
            mm_set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,          \
                         cudaGetErrorString(_e));                           \
            return MM_EDEVICE;                                              \
        }                                                                   \
    } while (0)

#define MM_CHECK_LAUNCH()                                                   \
    do {                                                                    \
        mm_launch_counter_add();                                            \
        cudaError_t _e = cudaGetLastError();                                \
        if (_e != cudaSuccess) {                                            \
            mm_set_error("%s:%d launch: %s", __FILE__, __LINE__,             \
                         cudaGetErrorString(_e));                           \
            return MM_EDEVICE;                                              \
        }                                                                   \
    } while (0)

#define MM_REQUIRE(cond, ...)                                               \
    do {                                                                    \
        if (!(cond)) {                                                      \
            mm_set_error(__VA_ARGS__);                                      \
            return MM_EINVAL;                                               \
        }                                                                   \
    } while (0)

// Records a message for mm_last_error() (thread-local).
void mm_set_error(const char *fmt, ...);
// Counts kernel launches made by this library (mm_launch_count()).
void mm_launch_counter_add();
// Raises a kernel's dynamic shared-memory limit to `bytes` once per (device,
// kernel) and size: later launches make no attribute call, so launches
// recorded into a CUDA graph after one eager pass make no driver call but the
// launch itself.
int mm_set_smem(const void *fn, size_t bytes);
unsigned long long mm_launch_counter_get();

static inline int mm_cdiv(long a, long b) { return (int)((a + b - 1) / b); }

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// Block-wide sum of one double per thread in a fixed order (warp shuffles,
// then the warps' sums by warp 0): thread 0 gets the total.  All threads of
// the block must call it; blockDim.x is a multiple of 32, at most 1024.
#ifdef __CUDACC__
__device__ __forceinline__ double mm_block_sum(double v) {
    __shared__ double part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    v = 0.0;
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}
#endif
