// unet_conv.cu -- BF16 3x3x3 / 1x1x1 convolutions of the warm-start U-Net on
// the sm_103a tensor cores (tcgen05), with FP32 accumulation in tensor memory.
//
// Both kernels are one GEMM D[128 x N] = sum_k A[128 x 32k] B[N x 32k]^T whose
// 32-wide K slices are fetched by TMA into shared memory (64-byte rows,
// 64-byte swizzle), multiplied by tcgen05.mma (M = 128, K = 16 per
// instruction) issued by one thread, and accumulated in TMEM:
//
// * conv_fwd_kernel (forward, and data gradient with the flipped weights):
//   rows = 128 output voxels (a bx x by x bz block), columns = the
//   output channels, K = taps x input channels.  Activations are channels-last
//   bf16 [n][z][y][x][c]; the tap offset moves the TMA box, whose zero fill
//   outside the volume is the convolution's zero padding.  Two inputs are
//   concatenated along K (the skip connection) without a copy.  The epilogue
//   adds the bias, applies ReLU or the ReLU-derivative mask of a saved
//   activation, rounds to bf16 and splits the channels over one or two outputs.
// * conv_wgrad_kernel (weight gradient): rows = (tap, input channel), columns
//   = output channels, K = voxels in 64-voxel slices (128-byte rows, 128-byte
//   swizzle).  Activations and output gradients are read channel-major
//   [n][c][z][y*x]; x offsets come from three x-shifted copies (so the
//   innermost TMA coordinate stays on the 16-byte grid), y and z offsets move
//   the box.  Split-K over voxel ranges; partial sums are added to an FP32
//   gradient with atomics.
//
// A warp-specialised pipeline per CTA: thread 0 issues TMA loads into a
// 4-stage ring, thread 32 issues the MMAs, and after the last MMA all four
// warps read the accumulator from TMEM (tcgen05.ld) for the epilogue.  Every
// mbarrier wait is bounded by a 2 s timer; a timeout sets a device error flag
// (read by ct_unet_status), drains the loads in flight and frees TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "ct_common.cuh"

namespace ct {

namespace {

__device__ int g_unet_err;

constexpr int kStages = 4;
constexpr int kRowBytes = 64;                 // one K slice: 32 bf16
constexpr int kTileM = 128;
constexpr uint32_t kABytes = kTileM * kRowBytes;
constexpr unsigned long long kWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of the given parity; false after limit_ns (kWaitNs).
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, unsigned long long limit_ns = kWaitNs) {
    if (mbar_try(b, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        for (int i = 0; i < 256; ++i)
            if (mbar_try(b, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// Flag bit of a bounded wait that gave up in wait_selftest_kernel.
constexpr int kErrSelftest = 8;

// One thread waits, through the convolutions' own bounded wait, on an
// mbarrier that nothing arrives on; the wait gives up after limit_ns and sets
// the error flag as a timed-out convolution does.  No copy or tensor-memory
// operation is in flight, so the kernel simply returns.
__global__ void __launch_bounds__(32) wait_selftest_kernel(unsigned long long limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        if (!mbar_wait(&bar, 0, limit_ns)) atomicOr(&g_unet_err, kErrSelftest);
    }
}

__device__ __forceinline__ void tma_load5(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2,
                                          int c3, int c4) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6, %7}], "
        "[%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
        : "memory");
}

__device__ __forceinline__ void tma_load4(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2,
                                          int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6}], "
        "[%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
        : "memory");
}

__device__ __forceinline__ void tma_load3(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}

// Shared-memory matrix descriptor of a K-major operand in the 64-byte swizzle
// layout: 64-byte rows, 8-row atoms of 512 bytes (stride byte offset), the
// leading byte offset unused, descriptor version 1, layout code 4.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>(1) << 16;
    d |= static_cast<uint64_t>(512 >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    d |= static_cast<uint64_t>(4) << 61;
    return d;
}

// The same for the 128-byte swizzle layout: 128-byte rows, 8-row atoms of
// 1024 bytes, layout code 2.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>(1) << 16;
    d |= static_cast<uint64_t>(1024 >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    d |= static_cast<uint64_t>(2) << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
    return reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~static_cast<uintptr_t>(1023));
}

// Shared control block after the stage ring.
struct Ctrl {
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t done;
    uint32_t tmem;
    int abort;
};

__device__ __forceinline__ void tap_offsets(int tap, int ntaps, int &dz, int &dy, int &dx) {
    if (ntaps == 27) {
        dz = tap / 9 - 1;
        dy = (tap / 3) % 3 - 1;
        dx = tap % 3 - 1;
    } else {
        dz = dy = dx = 0;
    }
}

__device__ __forceinline__ void fail(Ctrl *c, int code) {
    atomicOr(&g_unet_err, code);
    *reinterpret_cast<volatile int *>(&c->abort) = 1;
}

__device__ __forceinline__ bool aborted(Ctrl *c) { return *reinterpret_cast<volatile int *>(&c->abort) != 0; }

// After an abort: wait (bounded) for the loads issued into each of the S stages.
template <int S>
__device__ void drain_loads(Ctrl *c, int issued) {
    for (int s = 0; s < S && s < issued; ++s) {
        const int last = (issued - 1 - s) / S;   // use index of the last load into stage s
        mbar_wait(&c->full[s], static_cast<uint32_t>(last & 1));
    }
}

// The MMA side of one CTA over an S-stage ring of (A_BYTES of A, NG * N rows
// of B) stages with ROWB-byte rows (64: 64-byte swizzle, 128: 128-byte
// swizzle): per K step, NG groups of ROWB / 32 instructions of 128 x N x 16,
// group g reading A from byte offset g * A_STEP and the g-th B tile.
template <int N, int S, uint32_t A_BYTES, int NG, uint32_t A_STEP, int ROWB = kRowBytes>
__device__ __forceinline__ void mma_loop(Ctrl *c, uint8_t *ring, uint32_t tmem, int ksteps) {
    constexpr uint32_t stage = A_BYTES + NG * N * ROWB;
    constexpr uint32_t idesc = idesc_bf16(kTileM, N);
    constexpr int KK = ROWB / 32;
    for (int k = 0; k < ksteps; ++k) {
        const int s = k % S;
        if (aborted(c)) break;
        if (!mbar_wait(&c->full[s], static_cast<uint32_t>((k / S) & 1))) {
            fail(c, 2);
            break;
        }
        tc_fence_after();
        const uint32_t sa = smem_u32(ring + s * stage), sb = sa + A_BYTES;
#pragma unroll
        for (int g = 0; g < NG; ++g)
#pragma unroll
            for (int kk = 0; kk < KK; ++kk) {
                const uint32_t ao = sa + g * A_STEP + kk * 32, bo = sb + g * N * ROWB + kk * 32;
                const uint64_t ad = ROWB == 128 ? sw128_desc(ao) : sw64_desc(ao);
                const uint64_t bd = ROWB == 128 ? sw128_desc(bo) : sw64_desc(bo);
                umma_bf16(tmem, ad, bd, idesc, k | g | kk);
            }
        umma_commit(&c->empty[s]);
    }
    umma_commit(&c->done);
}

// y-halo mode of the forward kernel: 8 x 16 voxel tiles of one slice; one box of
// 8 x 18 voxels per (dz, dx, channel chunk) serves the three dy taps, whose A
// operands start 0, 8 and 16 rows (512-byte swizzle atoms) into it.
constexpr int kYBx = 8, kYBy = 16;
constexpr uint32_t kYABytes = kYBx * (kYBy + 2) * kRowBytes;
constexpr int kYStages = 3;

// weight-gradient ring: K slices of 64 voxels (128-byte rows, 128-byte swizzle)
constexpr int kWK = 64;
constexpr int kWRowBytes = 2 * kWK;
constexpr int kWStages = 3;

struct FwdArgs {
    int c1, c2;              // channels of input 1 and input 2 (0: one input)
    int ntaps;               // 27 (3x3x3) or 1
    int nx, ny, nz;          // volume size, x fastest
    int bx, by, bz;          // voxel block of one tile (bx * by * bz = 128)
    int ksteps;              // ntaps * (c1 + c2) / 32
    const float *bias;       // [N] or null
    int relu;
    __nv_bfloat16 *out1, *out2;
    int co1, co2;            // channels written to out1 / out2 (co1 + co2 = N)
    const __nv_bfloat16 *mask1, *mask2;   // ReLU-derivative masks (same layout as out1 / out2) or null
};

template <int N, bool YR>
__global__ void __launch_bounds__(128, 1)
conv_fwd_kernel(const __grid_constant__ CUtensorMap mx1, const __grid_constant__ CUtensorMap mx2,
                const __grid_constant__ CUtensorMap mw, const FwdArgs a) {
    constexpr int S = YR ? kYStages : kStages;
    constexpr uint32_t a_bytes = YR ? kYABytes : kABytes;
    constexpr int ng = YR ? 3 : 1;
    constexpr uint32_t stage = a_bytes + ng * N * kRowBytes;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *ring = align1024(smem_raw);
    Ctrl *c = reinterpret_cast<Ctrl *>(ring + S * stage);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    int t = blockIdx.x;
    const int tx = a.nx / a.bx, ty = a.ny / a.by, tz = a.nz / a.bz;
    const int x0 = (t % tx) * a.bx;
    t /= tx;
    const int y0 = (t % ty) * a.by;
    t /= ty;
    const int z0 = (t % tz) * a.bz, n0 = t / tz;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&c->full[s], 1);
            mbar_init(&c->empty[s], 1);
        }
        mbar_init(&c->done, 1);
        c->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) tmem_alloc(&c->tmem, N);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = c->tmem;

    if (threadIdx.x == 0) {
        const int nch = (a.c1 + a.c2) / 32;
        int issued = 0;
        for (int k = 0; k < a.ksteps; ++k) {
            const int s = k % S;
            if (aborted(c)) break;
            if (k >= S && !mbar_wait(&c->empty[s], static_cast<uint32_t>((k / S - 1) & 1))) {
                fail(c, 1);
                break;
            }
            // K order: (tap or (dz, dx) group) major, 32-channel chunks inner
            const int grp = k / nch, ch = (k % nch) * 32;
            int dz, dy, dx;
            if (YR) {
                dz = grp / 3 - 1;
                dx = grp % 3 - 1;
                dy = -1;                          // the box starts one row above the tile
            } else {
                tap_offsets(grp, a.ntaps, dz, dy, dx);
            }
            uint8_t *sa = ring + s * stage;
            mbar_expect_tx(&c->full[s], stage);
            if (ch < a.c1)
                tma_load5(sa, &mx1, &c->full[s], ch, x0 + dx, y0 + dy, z0 + dz, n0);
            else
                tma_load5(sa, &mx2, &c->full[s], ch - a.c1, x0 + dx, y0 + dy, z0 + dz, n0);
            if (YR) {
#pragma unroll
                for (int g = 0; g < 3; ++g)                 // dy = g - 1
                    tma_load3(sa + a_bytes + g * N * kRowBytes, &mw, &c->full[s], ch, (dz + 1) * 9 + g * 3 + (dx + 1),
                              0);
            } else {
                tma_load3(sa + a_bytes, &mw, &c->full[s], ch, grp, 0);
            }
            ++issued;
        }
        if (aborted(c)) drain_loads<S>(c, issued);
    } else if (threadIdx.x == 32) {
        mma_loop<N, S, a_bytes, ng, kYBx * kRowBytes>(c, ring, tmem, a.ksteps);
    }
    __syncwarp();

    // epilogue: thread = tile row = voxel
    const bool ok = mbar_wait(&c->done, 0);
    if (!ok) fail(c, 4);
    tc_fence_after();
    const int r = warp * 32 + lane;
    const int rxy = a.bx * a.by;
    const long long vox = ((static_cast<long long>(n0) * a.nz + z0 + r / rxy) * a.ny + (y0 + (r % rxy) / a.bx)) *
                              a.nx +
                          (x0 + r % a.bx);
    const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        tmem_ld16(trow + c0, v);
        if (!ok) continue;
        const bool first = c0 < a.co1;
        __nv_bfloat16 *o = first ? a.out1 : a.out2;
        const __nv_bfloat16 *m = first ? a.mask1 : a.mask2;
        const int cc = first ? c0 : c0 - a.co1, stride = first ? a.co1 : a.co2;
        if (a.bias) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] += __ldg(a.bias + c0 + j);
        }
        if (a.relu) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j], 0.0f);
        }
        if (m) {
            const uint4 *mp = reinterpret_cast<const uint4 *>(m + vox * stride + cc);
            const uint4 q0 = __ldg(mp), q1 = __ldg(mp + 1);
            const __nv_bfloat16 *mb0 = reinterpret_cast<const __nv_bfloat16 *>(&q0);
            const __nv_bfloat16 *mb1 = reinterpret_cast<const __nv_bfloat16 *>(&q1);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (!(__bfloat162float(mb0[j]) > 0.0f)) v[j] = 0.0f;
                if (!(__bfloat162float(mb1[j]) > 0.0f)) v[8 + j] = 0.0f;
            }
        }
        uint4 w0, w1;
        uint32_t *p0 = reinterpret_cast<uint32_t *>(&w0), *p1 = reinterpret_cast<uint32_t *>(&w1);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const __nv_bfloat162 h0 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
            const __nv_bfloat162 h1 = __floats2bfloat162_rn(v[8 + 2 * j], v[8 + 2 * j + 1]);
            p0[j] = *reinterpret_cast<const uint32_t *>(&h0);
            p1[j] = *reinterpret_cast<const uint32_t *>(&h1);
        }
        uint4 *op = reinterpret_cast<uint4 *>(o + vox * stride + cc);
        op[0] = w0;
        op[1] = w1;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 2) tmem_dealloc(tmem, N);
}

struct WgradArgs {
    int cin, ntaps;
    int rows_per_tap, taps_per_tile, cblocks;
    int nxy, nx, nz;         // y*x plane size, x size, slices
    long long kchunks;       // 64-voxel K slices over all samples
    int pchunks;             // 64-voxel slices per y*x plane (the last may run past the plane: zero fill)
    int kper;                // K slices per CTA
    float *dw;               // [N][ntaps][cin], FP32, accumulated
};

template <int N>
__global__ void __launch_bounds__(128, 1)
conv_wgrad_kernel(const __grid_constant__ CUtensorMap mxm, const __grid_constant__ CUtensorMap mx0,
                  const __grid_constant__ CUtensorMap mxp, const __grid_constant__ CUtensorMap mdy,
                  const WgradArgs a) {
    constexpr uint32_t a_bytes = kTileM * kWRowBytes;
    constexpr uint32_t stage = a_bytes + N * kWRowBytes;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *ring = align1024(smem_raw);
    Ctrl *c = reinterpret_cast<Ctrl *>(ring + kWStages * stage);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int tgroup = blockIdx.x / a.cblocks, cb = blockIdx.x % a.cblocks;
    const int tap0 = tgroup * a.taps_per_tile, ci0 = cb * a.rows_per_tap;
    const long long k0 = static_cast<long long>(blockIdx.y) * a.kper;
    const int ksteps = static_cast<int>(min(static_cast<long long>(a.kper), a.kchunks - k0));

    if (threadIdx.x == 0) {
        for (int s = 0; s < kWStages; ++s) {
            mbar_init(&c->full[s], 1);
            mbar_init(&c->empty[s], 1);
        }
        mbar_init(&c->done, 1);
        c->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) tmem_alloc(&c->tmem, N);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = c->tmem;

    if (threadIdx.x == 0) {
        const int pchunks = a.pchunks;
        int issued = 0;
        for (int k = 0; k < ksteps; ++k) {
            const int s = k % kWStages;
            if (aborted(c)) break;
            if (k >= kWStages && !mbar_wait(&c->empty[s], static_cast<uint32_t>((k / kWStages - 1) & 1))) {
                fail(c, 1);
                break;
            }
            long long q = k0 + k;
            const int p = static_cast<int>(q % pchunks) * kWK;
            q /= pchunks;
            const int z = static_cast<int>(q % a.nz), n = static_cast<int>(q / a.nz);
            uint8_t *sa = ring + s * stage;
            mbar_expect_tx(&c->full[s], stage);
            for (int j = 0; j < a.taps_per_tile; ++j) {
                const int tap = min(tap0 + j, a.ntaps - 1);
                int dz, dy, dx;
                tap_offsets(tap, a.ntaps, dz, dy, dx);
                const CUtensorMap *m = dx < 0 ? &mxm : (dx > 0 ? &mxp : &mx0);
                tma_load4(sa + j * a.rows_per_tap * kWRowBytes, m, &c->full[s], p + dy * a.nx, z + dz, ci0, n);
            }
            tma_load4(sa + a_bytes, &mdy, &c->full[s], p, z, 0, n);
            ++issued;
        }
        if (aborted(c)) drain_loads<kWStages>(c, issued);
    } else if (threadIdx.x == 32) {
        mma_loop<N, kWStages, a_bytes, 1, 0, kWRowBytes>(c, ring, tmem, ksteps);
    }
    __syncwarp();

    const bool ok = mbar_wait(&c->done, 0);
    if (!ok) fail(c, 4);
    tc_fence_after();
    const int r = warp * 32 + lane;
    const int tap = tap0 + r / a.rows_per_tap, ci = ci0 + r % a.rows_per_tap;
    const bool valid = ok && ksteps > 0 && tap < a.ntaps;
    const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    float *dst = a.dw + (valid ? static_cast<long long>(tap) * a.cin + ci : 0);   // rows past the last tap: unused
    const long long cstride = static_cast<long long>(a.ntaps) * a.cin;
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        tmem_ld16(trow + c0, v);
        if (valid) {
#pragma unroll
            for (int j = 0; j < 16; ++j) atomicAdd(dst + (c0 + j) * cstride, v[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 2) tmem_dealloc(tmem, N);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// bf16 tensor map of the given rank; dims innermost first, strides in bytes
// for dims 1.., 64-byte swizzle, zero fill outside.
int make_map(CUtensorMap *m, const void *base, int rank, const uint64_t *dims, const uint64_t *strides,
             const uint32_t *box, CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_64B) {
    auto fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return CT_ERR_CUDA;
    }
    cuuint64_t gd[5], gs[4];
    cuuint32_t bd[5], es[5];
    for (int i = 0; i < rank; ++i) {
        gd[i] = dims[i];
        bd[i] = box[i];
        es[i] = 1;
        if (i + 1 < rank) gs[i] = strides[i];
    }
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, const_cast<void *>(base), gd, gs, bd, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (" + std::to_string(static_cast<int>(r)) + ")");
        return CT_ERR_ARG;
    }
    return CT_OK;
}

// channels-last activation [n][z][y][x][c]: box 32 channels x bx x by x bz
int map_ndhwc(CUtensorMap *m, const void *p, int c, int nx, int ny, int nz, int nb, int bx, int by, int bz) {
    const uint64_t dims[5] = {(uint64_t)c, (uint64_t)nx, (uint64_t)ny, (uint64_t)nz, (uint64_t)nb};
    const uint64_t e = 2;
    const uint64_t st[4] = {c * e, (uint64_t)nx * c * e, (uint64_t)ny * nx * c * e, (uint64_t)nz * ny * nx * c * e};
    const uint32_t box[5] = {32, (uint32_t)bx, (uint32_t)by, (uint32_t)bz, 1};
    return make_map(m, p, 5, dims, st, box);
}

// channel-major activation [n][c][z][y*x]: box 64 voxels x rows channels, 128-byte swizzle
int map_ncdhw(CUtensorMap *m, const void *p, int c, int nxy, int nz, int nb, int rows) {
    const uint64_t dims[4] = {(uint64_t)nxy, (uint64_t)nz, (uint64_t)c, (uint64_t)nb};
    const uint64_t e = 2;
    const uint64_t st[3] = {(uint64_t)nxy * e, (uint64_t)nz * nxy * e, (uint64_t)c * nz * nxy * e};
    const uint32_t box[4] = {(uint32_t)kWK, 1, (uint32_t)rows, 1};
    return make_map(m, p, 4, dims, st, box, CU_TENSOR_MAP_SWIZZLE_128B);
}

// Dynamic shared memory of a ring (plus alignment slack and the control block).
// Every size here keeps the CTAs an SM can hold at <= 512 TMEM columns in total.
template <int N>
size_t ring_smem() {
    return 1024 + kStages * (kABytes + N * kRowBytes) + sizeof(Ctrl);
}

template <int N>
size_t wring_smem() {
    return 1024 + kWStages * (kTileM * kWRowBytes + N * kWRowBytes) + sizeof(Ctrl);
}

template <int N>
size_t yring_smem() {
    return 1024 + kYStages * (kYABytes + 3 * N * kRowBytes) + sizeof(Ctrl);
}

template <int N, bool YR>
int launch_fwd(const CUtensorMap &m1, const CUtensorMap &m2, const CUtensorMap &mw, const FwdArgs &a, int tiles,
               cudaStream_t st) {
    const size_t smem = YR ? yring_smem<N>() : ring_smem<N>();
    static bool attr = false;
    if (!attr) {
        CT_CUDA(cudaFuncSetAttribute(conv_fwd_kernel<N, YR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "conv_fwd smem");
        attr = true;
    }
    conv_fwd_kernel<N, YR><<<tiles, 128, smem, st>>>(m1, m2, mw, a);
    CT_LAUNCH_CHECK("conv_fwd_kernel");
    return CT_OK;
}

template <int N>
int launch_wgrad(const CUtensorMap &mm, const CUtensorMap &m0, const CUtensorMap &mp, const CUtensorMap &md,
                 const WgradArgs &a, dim3 grid, cudaStream_t st) {
    const size_t smem = wring_smem<N>();
    static bool attr = false;
    if (!attr) {
        CT_CUDA(cudaFuncSetAttribute(conv_wgrad_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "conv_wgrad smem");
        attr = true;
    }
    conv_wgrad_kernel<N><<<grid, 128, smem, st>>>(mm, m0, mp, md, a);
    CT_LAUNCH_CHECK("conv_wgrad_kernel");
    return CT_OK;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

bool valid_n(int n) { return n == 32 || n == 64 || n == 128 || n == 256; }

}  // namespace

}  // namespace ct

using namespace ct;

extern "C" {

int ct_unet_conv3d(const void *x1, int c1, const void *x2, int c2, int nb, int nz, int ny, int nx, const void *w,
                   int ntaps, const float *bias, int relu, void *out1, int co1, void *out2, int co2,
                   const void *mask1, const void *mask2, void *stream) {
    CT_REQUIRE(x1 && w && out1, "conv3d: null pointer");
    CT_REQUIRE(ntaps == 1 || ntaps == 27, "conv3d: ntaps must be 1 or 27");
    CT_REQUIRE(c1 > 0 && c1 % 32 == 0 && c2 >= 0 && c2 % 32 == 0 && (c2 == 0 || x2),
               "conv3d: input channels must be positive multiples of 32");
    const int n = co1 + co2;
    CT_REQUIRE(valid_n(n) && co1 > 0 && co1 % 16 == 0 && co2 % 16 == 0 && (co2 == 0 || out2),
               "conv3d: output channels must total 32, 64, 128 or 256, split at a multiple of 16");
    CT_REQUIRE(nb > 0 && nz > 0 && ny > 0 && nx > 0, "conv3d: empty volume");
    // y-halo tiles (8 x 16 voxels, the three dy taps from one box) where they fit
    const bool yr = ntaps == 27 && n <= 128 && nx % kYBx == 0 && ny % kYBy == 0;
    int bx, by, bz;
    if (yr) {
        bx = kYBx;
        by = kYBy;
        bz = 1;
    } else {
        bx = nx >= 128 ? 128 : nx;
        CT_REQUIRE(128 % bx == 0 && nx % bx == 0, "conv3d: x must be a divisor or a multiple of 128");
        by = ny >= 128 / bx ? 128 / bx : ny;
        CT_REQUIRE((128 / bx) % by == 0 && ny % by == 0, "conv3d: y must fit the 128-voxel tile");
        bz = 128 / (bx * by);
        CT_REQUIRE(nz % bz == 0, "conv3d: z must be a multiple of 128 / (x * y) for small slices");
    }
    CT_REQUIRE(aligned16(x1) && aligned16(w) && aligned16(out1) && (!x2 || aligned16(x2)) &&
                   (!out2 || aligned16(out2)) && (!mask1 || aligned16(mask1)) && (!mask2 || aligned16(mask2)),
               "conv3d: pointers must be 16-byte aligned");
    const long long tiles = (long long)nb * (nz / bz) * (ny / by) * (nx / bx);
    CT_REQUIRE(tiles < (1ll << 31), "conv3d: too many tiles");
    CUtensorMap m1, m2, mw;
    int s;
    const int box_y = yr ? by + 2 : by;
    if ((s = map_ndhwc(&m1, x1, c1, nx, ny, nz, nb, bx, box_y, bz))) return s;
    if ((s = map_ndhwc(&m2, c2 ? x2 : x1, c2 ? c2 : c1, nx, ny, nz, nb, bx, box_y, bz))) return s;
    {
        const int cin = c1 + c2;
        const uint64_t dims[3] = {(uint64_t)cin, (uint64_t)ntaps, (uint64_t)n};
        const uint64_t st[2] = {(uint64_t)cin * 2, (uint64_t)ntaps * cin * 2};
        const uint32_t box[3] = {32, 1, (uint32_t)n};
        if ((s = make_map(&mw, w, 3, dims, st, box))) return s;
    }
    FwdArgs a{};
    a.c1 = c1;
    a.c2 = c2;
    a.ntaps = ntaps;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.bx = bx;
    a.by = by;
    a.bz = bz;
    a.ksteps = (yr ? 9 : ntaps) * (c1 + c2) / 32;
    a.bias = bias;
    a.relu = relu;
    a.out1 = static_cast<__nv_bfloat16 *>(out1);
    a.out2 = static_cast<__nv_bfloat16 *>(out2);
    a.co1 = co1;
    a.co2 = co2;
    a.mask1 = static_cast<const __nv_bfloat16 *>(mask1);
    a.mask2 = static_cast<const __nv_bfloat16 *>(mask2);
    cudaStream_t st = as_stream(stream);
    if (yr) {
        switch (n) {
            case 32: return launch_fwd<32, true>(m1, m2, mw, a, (int)tiles, st);
            case 64: return launch_fwd<64, true>(m1, m2, mw, a, (int)tiles, st);
            default: return launch_fwd<128, true>(m1, m2, mw, a, (int)tiles, st);
        }
    }
    switch (n) {
        case 32: return launch_fwd<32, false>(m1, m2, mw, a, (int)tiles, st);
        case 64: return launch_fwd<64, false>(m1, m2, mw, a, (int)tiles, st);
        case 128: return launch_fwd<128, false>(m1, m2, mw, a, (int)tiles, st);
        default: return launch_fwd<256, false>(m1, m2, mw, a, (int)tiles, st);
    }
}

int ct_unet_conv3d_wgrad(const void *xm, const void *x0, const void *xp, int cin, const void *dy, int cout, int nb,
                         int nz, int ny, int nx, int ntaps, int kper, float *dw, void *stream) {
    CT_REQUIRE(x0 && dy && dw && (ntaps == 1 || (xm && xp)), "conv3d_wgrad: null pointer");
    CT_REQUIRE(ntaps == 1 || ntaps == 27, "conv3d_wgrad: ntaps must be 1 or 27");
    CT_REQUIRE(cin > 0 && cin % 32 == 0, "conv3d_wgrad: input channels must be a positive multiple of 32");
    CT_REQUIRE(valid_n(cout), "conv3d_wgrad: output channels must be 32, 64, 128 or 256");
    CT_REQUIRE(nb > 0 && nz > 0 && ny > 0 && nx > 0 && nx % 8 == 0 && (long long)nx * ny < (1ll << 30),
               "conv3d_wgrad: x must be a multiple of 8");
    CT_REQUIRE(kper > 0, "conv3d_wgrad: kper must be positive");
    CT_REQUIRE(aligned16(x0) && aligned16(dy) && (!xm || aligned16(xm)) && (!xp || aligned16(xp)),
               "conv3d_wgrad: pointers must be 16-byte aligned");
    const int nxy = nx * ny;
    const int rows = cin >= 128 ? 128 : cin;
    CUtensorMap mm, m0, mp, md;
    int s;
    if ((s = map_ncdhw(&m0, x0, cin, nxy, nz, nb, rows))) return s;
    if ((s = map_ncdhw(&mm, ntaps == 27 ? xm : x0, cin, nxy, nz, nb, rows))) return s;
    if ((s = map_ncdhw(&mp, ntaps == 27 ? xp : x0, cin, nxy, nz, nb, rows))) return s;
    if ((s = map_ncdhw(&md, dy, cout, nxy, nz, nb, cout))) return s;
    WgradArgs a{};
    a.cin = cin;
    a.ntaps = ntaps;
    a.rows_per_tap = rows;
    a.taps_per_tile = 128 / rows;
    a.cblocks = cin / rows;
    a.nxy = nxy;
    a.nx = nx;
    a.nz = nz;
    // a slice past the end of a plane reads zeros for dY, so it adds nothing
    a.pchunks = (nxy + kWK - 1) / kWK;
    a.kchunks = (long long)nb * nz * a.pchunks;
    a.kper = kper;
    a.dw = dw;
    const int ttiles = (ntaps + a.taps_per_tile - 1) / a.taps_per_tile;
    const long long ksplit = (a.kchunks + kper - 1) / kper;
    CT_REQUIRE(ksplit <= 65535, "conv3d_wgrad: too many K splits (raise kper)");
    dim3 grid(ttiles * a.cblocks, (unsigned)ksplit);
    cudaStream_t st = as_stream(stream);
    switch (cout) {
        case 32: return launch_wgrad<32>(mm, m0, mp, md, a, grid, st);
        case 64: return launch_wgrad<64>(mm, m0, mp, md, a, grid, st);
        case 128: return launch_wgrad<128>(mm, m0, mp, md, a, grid, st);
        default: return launch_wgrad<256>(mm, m0, mp, md, a, grid, st);
    }
}

int ct_unet_wait_selftest(long long limit_ns, void *stream) {
    CT_REQUIRE(limit_ns >= 1000 && limit_ns <= 1000000000LL, "unet_wait_selftest: limit must be in [1 us, 1 s]");
    wait_selftest_kernel<<<1, 32, 0, as_stream(stream)>>>((unsigned long long)limit_ns);
    CT_LAUNCH_CHECK("wait_selftest_kernel");
    return CT_OK;
}

int ct_unet_status(int *flags) {
    CT_REQUIRE(flags, "unet_status: null pointer");
    int zero = 0;
    CT_CUDA(cudaMemcpyFromSymbol(flags, g_unet_err, sizeof(int)), "unet_status read");
    CT_CUDA(cudaMemcpyToSymbol(g_unet_err, &zero, sizeof(int)), "unet_status reset");
    if (*flags) {
        set_error("a tensor-core convolution gave up on a bounded wait (flags " + std::to_string(*flags) + ")");
        return CT_ERR_TIMEOUT;
    }
    return CT_OK;
}

}  // extern "C"
