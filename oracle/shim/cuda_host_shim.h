/*
 * cuda_host_shim.h -- lets the reference's __global__ kernel functions compile
 * as plain host C++ so the checker can run them on the CPU, one simulated
 * thread at a time.  TEST INFRASTRUCTURE ONLY (used by oracle/build_ref.py).
 *
 * A launch <<<grid, block>>> becomes two nested loops that set blockIdx.x and
 * threadIdx.x before each call.  Threads of a block therefore run to
 * completion one after another; the kernels used with this shim have no
 * barriers, and the one kernel whose result depends on thread interleaving
 * (the in-place pre-weight of PreWeightFilter) is only driven here in ways
 * that make the interleaving irrelevant (see the harness files).
 */
#pragma once
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>
using namespace std;

struct shim_dim3 { unsigned int x, y, z; };
static shim_dim3 threadIdx = {0, 0, 0};
static shim_dim3 blockIdx = {0, 0, 0};
static shim_dim3 blockDim = {1, 1, 1};
static shim_dim3 gridDim = {1, 1, 1};

#define __global__
#define __device__
#define __host__
#define __syncthreads() ((void)0)

#define SHIM_LAUNCH(grid, block, call)                                   \
    do {                                                                 \
        gridDim.x = (grid); blockDim.x = (block);                        \
        for (unsigned int _b = 0; _b < (unsigned int)(grid); ++_b) {     \
            blockIdx.x = _b;                                             \
            for (unsigned int _t = 0; _t < (unsigned int)(block); ++_t) { \
                threadIdx.x = _t;                                        \
                call;                                                    \
            }                                                            \
        }                                                                \
    } while (0)

#define SHIM_EXPORT extern "C" __attribute__((visibility("default")))
