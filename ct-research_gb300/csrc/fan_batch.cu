// fan_batch.cu -- many 2D fan slices of uneven size in one launch per operator.
//
// The slices of a batch (own image size, views, detector bins and geometry)
// share one flat block index space: slice k owns the blocks
// [blk0[k], blk0[k+1]) of the forward-projection grid (its rays) and of the
// backprojection grid (its pixels).  A block finds its slice by binary search
// over the descriptor table, so the work of all slices is balanced by the
// hardware scheduler with no per-slice launches.  Images and sinograms live in
// two packed device buffers at the descriptor's offsets.  Per-slice residual
// norms are reduced per block into norms[2k], norms[2k+1].
//
// The per-ray and per-pixel arithmetic is the single-slice operators'
// (fan2d_dev.cuh), so a batch reproduces the single-slice results exactly.
#include "fan2d_dev.cuh"

namespace ct {

namespace {

__device__ __forceinline__ int find_slice(const BatchSlice *__restrict__ sl, int nsl, bool pixels) {
    __shared__ int s_k;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nsl - 1;
        const int b = (int)blockIdx.x;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            const int start = pixels ? sl[mid].pix_blk0 : sl[mid].ray_blk0;
            if (start <= b) lo = mid; else hi = mid - 1;
        }
        s_k = lo;
    }
    __syncthreads();
    return s_k;
}

template <int MODE>
// blocks per SM of the batched projection: 4 (32 registers) measured 6.04 ms on
// 64 uneven slices against 6.17 / 6.32 ms at 3 / 2
#ifndef CT_FANB_FP_MINB
#define CT_FANB_FP_MINB 4
#endif
__global__ void __launch_bounds__(512, CT_FANB_FP_MINB)
fan_batch_fp_kernel(const BatchSlice *__restrict__ sl, int nsl, const float *__restrict__ img,
                    float *__restrict__ out, const float *__restrict__ b, const float *__restrict__ rowsum,
                    float eps, double *__restrict__ norms, const GrazeList gl) {
    const int k = find_slice(sl, nsl, false);
    const FanGeom g = sl[k].g;
    const long long r = (long long)(blockIdx.x - sl[k].ray_blk0) * blockDim.x + threadIdx.x;
    const bool active = r < (long long)g.nb * g.np;
    float r2 = 0.0f, b2 = 0.0f;
    if (active) {
        bool grazing;
        const float val = fan_ray_value(g, img + sl[k].img_off, r, grazing);
        const long long o = sl[k].sino_off + r;
        if (grazing) graze_push(gl, ((unsigned long long)k << 40) | (unsigned long long)r, (unsigned long long)o);
        if (MODE == 0) {
            out[o] = val;
        } else {
            const float bb = b[o];
            const float rr = bb - val;
            const float sc = rowsum ? 1.0f / (rowsum[o] + eps) : 1.0f;
            out[o] = rr * sc;
            r2 = grazing ? 0.0f : rr * rr;   // grazing rays: added by the FP64 re-walk
            b2 = bb * bb;
        }
    }
    if (MODE == 1) {
        block_sum_any_f(r2, norms + 2 * k);
        block_sum_any_f(b2, norms + 2 * k + 1);
    }
}

// blocks of 512 threads per SM the batched backprojection's registers aim at:
// 3 (40 registers, a few bytes spilled by the chord weighting) measured 11.06 ms
// per backprojection with update on 64 uneven slices, against 11.28 ms at 4
// and 11.50 ms with the compiler's own choice (64 registers)
#ifndef CT_FANB_BP_MINB
#define CT_FANB_BP_MINB 3
#endif
template <int WMODE, bool UPDATE>
__global__ void __launch_bounds__(512, CT_FANB_BP_MINB)
fan_batch_bp_kernel(const BatchSlice *__restrict__ sl, int nsl, const float *__restrict__ R, float *__restrict__ img,
                    const float *__restrict__ colsum, float eps, float lambda, float lo, float hi) {
    const int k = find_slice(sl, nsl, true);
    const FanGeom g = sl[k].g;
    const int i = (int)(blockIdx.x - sl[k].pix_blk0) * blockDim.x + threadIdx.x;
    if (i >= g.nt * g.ns) return;
    const float acc = fan_pixel_sum<WMODE>(g, R + sl[k].sino_off, i);
    const long long o = sl[k].img_off + i;
    if (UPDATE) {
        const float x = img[o] + lambda * acc / (colsum[o] + eps);
        img[o] = fminf(fmaxf(x, lo), hi);
    } else {
        img[o] = acc;
    }
}

}  // namespace

int fan_batch_fp_launch(const BatchSlice *d_sl, int nsl, int nblocks, int block, const float *img, float *out,
                        const float *b, const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl,
                        cudaStream_t st) {
    CT_REQUIRE(block >= 32 && block <= 512 && block % 32 == 0, "batch: block size must be a multiple of 32 <= 512");
    CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(*gl.count), st), "graze list reset");
    if (mode == 0)
        fan_batch_fp_kernel<0><<<nblocks, block, 0, st>>>(d_sl, nsl, img, out, nullptr, nullptr, 0.f, nullptr, gl);
    else
        fan_batch_fp_kernel<1><<<nblocks, block, 0, st>>>(d_sl, nsl, img, out, b, rowsum, eps, norms, gl);
    CT_LAUNCH_CHECK("fan_batch_fp_kernel");
    return fan_batch_fixup_launch(d_sl, nsl, img, out, b, rowsum, eps, norms, mode, gl, st);
}

int fan_batch_bp_launch(const BatchSlice *d_sl, int nsl, int nblocks, int block, const float *R, float *img, int wmode,
                        const float *colsum, float eps, float lambda, float lo, float hi, bool update,
                        cudaStream_t st) {
    CT_REQUIRE(block >= 32 && block <= 512 && block % 32 == 0, "batch: block size must be a multiple of 32 <= 512");
#define CT_FB_CASE(W, U) \
    fan_batch_bp_kernel<W, U><<<nblocks, block, 0, st>>>(d_sl, nsl, R, img, colsum, eps, lambda, lo, hi)
    if (update) {
        if (wmode == 0) CT_FB_CASE(BP2_BACKPROJ, true);
        else if (wmode == 1) CT_FB_CASE(BP2_FBPFAN, true);
        else CT_FB_CASE(BP2_FBPPAR, true);
    } else {
        if (wmode == 0) CT_FB_CASE(BP2_BACKPROJ, false);
        else if (wmode == 1) CT_FB_CASE(BP2_FBPFAN, false);
        else CT_FB_CASE(BP2_FBPPAR, false);
    }
#undef CT_FB_CASE
    CT_LAUNCH_CHECK("fan_batch_bp_kernel");
    return CT_OK;
}

}  // namespace ct
