// ct_common.cuh -- shared helpers of the sm_103a CT kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "ctgb.h"

namespace ct {

// Last-error message of the calling host thread (ct_last_error()).
void set_error(const std::string &msg);

// Record a CUDA failure and map it to a ct_status.
int cuda_status(cudaError_t e, const char *what);

#define CT_CUDA(call, what)                                   \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return ct::cuda_status(_e, what); \
    } while (0)

#define CT_LAUNCH_CHECK(what)                                 \
    do {                                                      \
        cudaError_t _e = cudaGetLastError();                  \
        if (_e != cudaSuccess) {                              \
            ct::set_error(std::string(what) + ": " + cudaGetErrorString(_e)); \
            return CT_ERR_LAUNCH;                             \
        }                                                     \
    } while (0)

#define CT_REQUIRE(cond, msg)                                 \
    do {                                                      \
        if (!(cond)) { ct::set_error(msg); return CT_ERR_ARG; } \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (152 on GB300), cached per process.
int sm_count();

// ---------------------------------------------------------------------------
// Device-side numerics
// ---------------------------------------------------------------------------

// 1/x in double from the single-precision reciprocal and one Newton step
// (relative error ~ 2^-46, enough for the Siddon entry/exit parameters).
__device__ __forceinline__ double drcp(double x) {
    double y = (double)__frcp_rn((float)x);
    y = y * (2.0 - x * y);
    return y * (2.0 - x * y);
}

// Warp-level sum.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-level sum of a double into *out with one atomic per block.
// Call with all threads of the block; blockDim.x*y*z must be a multiple of 32.
template <int NWARPS>
__device__ __forceinline__ void block_sum_atomic(double v, double *out) {
    __shared__ double part[NWARPS];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    v = warp_sum(v);
    if ((tid & 31) == 0) part[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        double w = (tid < NWARPS) ? part[tid] : 0.0;
        w = warp_sum(w);
        if (tid == 0) atomicAdd(out, w);
    }
}

// The same for per-thread FP32 terms: the warp sums (32 terms) run in FP32,
// the per-warp partials and the atomic in FP64.  GB300 runs FP64 at a small
// fraction of its FP32 rate, so a per-element FP64 reduction can bound an
// otherwise memory-bound kernel; these sums normalise steps and report
// residuals, for which FP32 partials of 32 terms are ample.  Integer-valued
// terms below 2^19 sum exactly.
template <int NWARPS>
__device__ __forceinline__ void block_sum_atomic_f(float v, double *out) {
    __shared__ double part[NWARPS];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    v = warp_sum(v);
    if ((tid & 31) == 0) part[tid >> 5] = (double)v;
    __syncthreads();
    if (tid < 32) {
        double w = (tid < NWARPS) ? part[tid] : 0.0;
        w = warp_sum(w);
        if (tid == 0) atomicAdd(out, w);
    }
}

}  // namespace ct
