// filter.cu -- pre-weight + Shepp-Logan-form ramp filtering of detector rows.
//
// out[p] = dP * sum_q in'[q] * G[(np-1) + p - q], G the taps of GFunction
// (FDK.cu:6-19): G[np-1] = 1/(pi dP)^2, G[np-1 +- n] = -1/(pi dP)^2/(4n^2-1).
// in' is the row after the cosine pre-weight w (FDK: D/sqrt(D^2+P^2+xi^2),
// FDK.cu:34; FBPfan: R/sqrt(R^2+P^2), FBPfan.cu:32; FBPparallel: none).
//
// The reference applies w in place inside the same kernel that convolves the
// row, one P-tile (256 samples for FDK, 128 for FBPfan) per launch and
// `limit` taps per launch chunk (FDK.cu:333-477).  LAUNCH_ORDER mode models
// what that produces on a GPU: the outputs of a P-tile see the tiles launched
// before it fully weighted, their own tile weighted once per chunk processed
// so far, and later tiles unweighted; rows of the residual row tile launch
// the residual P-tile first.  CLEAN mode weights the whole row once.
//
// Options beyond the reference's GPU path: other ramp taps (Ram-Lak) only
// change G; short-scan (Parker) weights multiply the raw row as it is loaded,
// as a caller weighting the sinogram before the call would; a Hamming
// smoothing window runs over each finished filtered row.
//
// One block per row; the row, its mixed copy and the taps live in shared
// memory.  A thread computes FJ consecutive outputs: the taps they need at
// one input sample are consecutive, so one tap load per sample slides a
// register window.  Partial sums are exact float pairs flushed into a double
// every 256 taps; each chunk result is added into the float output as the
// reference's `dev_Rcov[...] += PInt * Rcovsum` does.
#include "kernels.cuh"

namespace ct {


namespace {

constexpr int FT = 256;
// Consecutive outputs per thread: 4 where the rows fill the GPU (measured at
// 256^3 FDK, 360 x 384 rows of 512: 2 / 4 / 8 outputs per thread 10.47 / 8.90 /
// 9.00 ms against 11.75 with one), else 1 (a 2D scan of a few hundred rows keeps
// more threads per row: 360 rows of 512, 0.23 ms with 1 against 0.28 with 4).
constexpr int FJ_WIDE = 4;

template <int FJ>
__global__ void __launch_bounds__(FT)
row_filter_kernel(const RowFilter f, const float *__restrict__ R, float *__restrict__ out) {
    extern __shared__ float sm[];
    const int np = f.np;
    float *raw = sm;
    float *mix = sm + np;
    float *G = sm + 2 * np;
    const int row = blockIdx.x;
    const float *in = R + (long long)row * np;
    float *o = out + (long long)row * np;
    const double *w = f.w ? f.w + (long long)(row % f.wrows) * np : nullptr;
    const float *pw = f.pw ? f.pw + (long long)(row / f.pw_div) * np : nullptr;
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
        raw[q] = pw ? __fmul_rn(in[q], pw[q]) : in[q];
        o[q] = 0.0f;
    }
    for (int q = threadIdx.x; q < 2 * np - 1 + FJ; q += blockDim.x) G[q] = q < 2 * np - 1 ? f.G[q] : 0.0f;
    __syncthreads();

    const int gtime = (np + f.limit - 1) / f.limit;
    const int nfull = np / f.tile, resid = np % f.tile;
    const int ntiles = nfull + (resid ? 1 : 0);
    const bool launch_order = f.launch_order && w;
    // launch position of each P-tile for this row
    const int ridx = row % f.rowmod;
    const bool resid_rows = (f.rowmod % f.row_block) != 0 && ridx >= (f.rowmod / f.row_block) * f.row_block;
    auto pos_of = [&](int k) { return (resid_rows && resid) ? (k == nfull ? 0 : k + 1) : k; };

    const int nsteps = launch_order ? ntiles : 1;
    for (int step = 0; step < nsteps; ++step) {
        int k = 0, p0 = 0, p1 = np;
        if (launch_order) {
            for (int j = 0; j < ntiles; ++j)
                if (pos_of(j) == step) k = j;
            p0 = k * f.tile;
            p1 = (k == nfull) ? np : p0 + f.tile;
        }
        for (int c = 0; c < gtime; ++c) {
            const int g0 = c * f.limit, g1 = (c == gtime - 1) ? np : (c + 1) * f.limit;
            // the row as this chunk's launch reads it
            for (int q = g0 + threadIdx.x; q < g1; q += blockDim.x) {
                float v = raw[q];
                if (w) {
                    int e = 1;
                    if (launch_order) {
                        const int j = q / f.tile;
                        const int pj = pos_of(j);
                        e = (pj < step) ? gtime : (j == k ? c + 1 : 0);
                    }
                    for (int i = 0; i < e; ++i) v = (float)((double)v * w[q]);
                }
                mix[q] = v;
            }
            __syncthreads();
            for (int pb = p0 + FJ * threadIdx.x; pb < p1; pb += FJ * blockDim.x) {
                // The reference rounds each float*float product to float and sums
                // in double (FDK.cu:41-45).  Here: the same rounded products,
                // summed per output as an unevaluated pair (s + c) with the TwoSum
                // error-free transformation (Knuth), flushed into a double every
                // 256 taps.  Output pb + j takes tap G[(np - 1) + pb + j - q] at
                // sample q: the window w[j] of the FJ outputs moves by one tap per
                // sample (G carries FJ zeros past its end for the window's start).
                double dacc[FJ];
#pragma unroll
                for (int j = 0; j < FJ; ++j) dacc[j] = 0.0;
                const float *gp = G + (np - 1) + pb;
                // chunks of 256 taps keep the double flush out of the inner loop
                for (int q0 = g0; q0 < g1; q0 += 256) {
                    const int q1 = min(q0 + 256, g1);
                    float sh[FJ], sl[FJ], w[FJ];
#pragma unroll
                    for (int j = 0; j < FJ; ++j) {
                        sh[j] = 0.0f;
                        sl[j] = 0.0f;
                        w[j] = gp[j + 1 - q0];   // the window of sample q0 - 1
                    }
#pragma unroll 4
                    for (int q = q0; q < q1; ++q) {
#pragma unroll
                        for (int j = FJ - 1; j > 0; --j) w[j] = w[j - 1];
                        w[0] = gp[-q];
                        const float m = mix[q];
#pragma unroll
                        for (int j = 0; j < FJ; ++j) {
                            const float prod = __fmul_rn(m, w[j]);
                            const float t = __fadd_rn(sh[j], prod);
                            const float bp = __fsub_rn(t, sh[j]);
                            const float err = __fadd_rn(__fsub_rn(sh[j], __fsub_rn(t, bp)), __fsub_rn(prod, bp));
                            sh[j] = t;
                            sl[j] = __fadd_rn(sl[j], err);
                        }
                    }
#pragma unroll
                    for (int j = 0; j < FJ; ++j) dacc[j] += (double)sh[j] + (double)sl[j];
                }
#pragma unroll
                for (int j = 0; j < FJ; ++j)
                    if (pb + j < p1) o[pb + j] = (float)((double)o[pb + j] + (double)f.pint * dacc[j]);
            }
            __syncthreads();
        }
    }
    if (f.win) {
        // smoothing of the filtered row: o[p] = sum_i win[i] x[p + i - wlen/2] / wsum,
        // x zero outside the row; sequential double sum without contraction
        for (int q = threadIdx.x; q < np; q += blockDim.x) raw[q] = o[q];
        __syncthreads();
        const int c = f.wlen / 2;
        for (int p = threadIdx.x; p < np; p += blockDim.x) {
            double acc = 0.0;
            for (int i = 0; i < f.wlen; ++i) {
                const int k = p + i - c;
                if (k >= 0 && k < np) acc = __dadd_rn(acc, __dmul_rn((double)raw[k], f.win[i]));
            }
            o[p] = (float)__ddiv_rn(acc, f.wsum);
        }
    }
}

}  // namespace

int row_filter_launch(const RowFilter &f, const float *R, float *out, cudaStream_t st) {
    CT_REQUIRE(f.np >= 2, "row filter: at least 2 detector samples");
    const int wide = f.nrow >= 8 * sm_count();
    const int fj = wide ? FJ_WIDE : 1;
    const size_t smem = sizeof(float) * (size_t)(4 * f.np - 1 + fj);
    CT_REQUIRE(smem <= 200 * 1024, "row filter: detector row too long for shared memory");
    if (smem > 48 * 1024) {
        if (wide)
            CT_CUDA(cudaFuncSetAttribute(row_filter_kernel<FJ_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem),
                    "row_filter smem attribute");
        else
            CT_CUDA(cudaFuncSetAttribute(row_filter_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "row_filter smem attribute");
    }
    // fj outputs per thread over a P-tile (launch order) or the row, so no thread idles
    const int span = (f.launch_order && f.w) ? f.tile : f.np;
    const int block = std::min(FT, std::max(32, ((span + fj - 1) / fj + 31) / 32 * 32));
    if (wide) row_filter_kernel<FJ_WIDE><<<f.nrow, block, smem, st>>>(f, R, out);
    else row_filter_kernel<1><<<f.nrow, block, smem, st>>>(f, R, out);
    CT_LAUNCH_CHECK("row_filter_kernel");
    return CT_OK;
}

}  // namespace ct
