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
 *
 * With SHIM_THREADED defined, the block/thread indices are thread-local and
 * __syncthreads() is a barrier: a harness then runs each simulated thread of
 * a block as an OS thread (SHIM_LAUNCH_BLOCK), which gives kernels that
 * weight in place, synchronise and then read their neighbours (ImplementUI.cu
 * PreWeightFiltration) their barrier semantics.
 */
#pragma once
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>
using namespace std;

struct shim_dim3 { unsigned int x, y, z; };

#ifdef SHIM_THREADED
#include <pthread.h>
#include <vector>
static thread_local shim_dim3 threadIdx = {0, 0, 0};
static thread_local shim_dim3 blockIdx = {0, 0, 0};
static shim_dim3 blockDim = {1, 1, 1};
static shim_dim3 gridDim = {1, 1, 1};
static pthread_barrier_t shim_barrier;
#define __syncthreads() ((void)pthread_barrier_wait(&shim_barrier))

/* Run one block (bx, by) of `block` threads, each an OS thread calling fn(t). */
template <typename F>
static void shim_launch_block(unsigned int bx, unsigned int by, unsigned int block, F fn)
{
    struct Arg { F *fn; unsigned int bx, by, t; };
    blockDim.x = block;
    pthread_barrier_init(&shim_barrier, nullptr, block);
    std::vector<pthread_t> th(block);
    std::vector<Arg> args(block);
    for (unsigned int t = 0; t < block; ++t) {
        args[t] = Arg{&fn, bx, by, t};
        pthread_create(&th[t], nullptr, [](void *p) -> void * {
            Arg *a = (Arg *)p;
            blockIdx.x = a->bx; blockIdx.y = a->by; threadIdx.x = a->t;
            (*a->fn)(a->t);
            return nullptr;
        }, &args[t]);
    }
    for (unsigned int t = 0; t < block; ++t) pthread_join(th[t], nullptr);
    pthread_barrier_destroy(&shim_barrier);
}
#else
static shim_dim3 threadIdx = {0, 0, 0};
static shim_dim3 blockIdx = {0, 0, 0};
static shim_dim3 blockDim = {1, 1, 1};
static shim_dim3 gridDim = {1, 1, 1};
#define __syncthreads() ((void)0)
#endif

#define __global__
#define __device__
#define __host__

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

/* Two-dimensional grid (blockIdx.x, blockIdx.y), one-dimensional blocks. */
#define SHIM_LAUNCH2(gx, gy, block, call)                                \
    do {                                                                 \
        gridDim.x = (gx); gridDim.y = (gy); blockDim.x = (block);        \
        for (unsigned int _by = 0; _by < (unsigned int)(gy); ++_by)      \
            for (unsigned int _b = 0; _b < (unsigned int)(gx); ++_b) {   \
                blockIdx.x = _b; blockIdx.y = _by;                       \
                for (unsigned int _t = 0; _t < (unsigned int)(block); ++_t) { \
                    threadIdx.x = _t;                                    \
                    call;                                                \
                }                                                        \
            }                                                            \
    } while (0)

#define SHIM_EXPORT extern "C" __attribute__((visibility("default")))
