// fan2d_dev.cuh -- per-ray and per-pixel device code of the 2D fan / parallel
// operators, shared by the single-slice kernels (fan2d.cu) and the batched
// uneven-slice kernels (fan_batch.cu).
//
// Forward projection: the Siddon walk of siddon.cuh on a one-slice volume
// (n[2] = 1, no z crossings).
//  * fan (ProjectionFan_2D.cu:19-216): source (C_t - D sin b, C_s + D cos b),
//    ray through the point P on the line through the centre perpendicular to
//    the central ray: d = (P cos b + D sin b, P sin b - D cos b).
//  * parallel (ProjectionParallel_2D.cu:23-243): ray of offset t at angle th,
//    direction (-sin th, cos th) in (x, y) = (width, height) coordinates,
//    through (C_x + t cos th, C_y + t sin th).
// Backprojection: one pixel, all views, the sum in a register.
//  * BP2_BACKPROJ (BackprojectionFan2D.cu:7-116): linear interpolation of R at
//    the pixel's detector position P/U times the reference's weight
//    2 * |T1S1 - End|: End is the far point 2*Rscan along the source->pixel
//    line and T1S1 its crossing with the pixel's low t edge (accepted when the
//    crossing's s lies in [0, s_high], as the reference tests) or else its low
//    s edge (t in [0, t_high]); pixel-views with neither add nothing.
//  * BP2_FBPFAN (FBPfan.cu:45-96): filtered R interpolated, times dbeta / U^2.
//  * BP2_FBPPAR (FBPparallel.cu:41-89): filtered R at t = x cos th + y sin th, times dth.
// Detector interpolation: index floor(|P - P0| / PInt), weights from the
// domain values (BackprojectionFan2D.cu:44-53).
#pragma once
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {

enum { BP2_BACKPROJ = 0, BP2_FBPFAN = 1, BP2_FBPPAR = 2 };

// Walk set-up of ray r = view * np + bin; false for rays that miss the image.
__device__ __forceinline__ bool fan_ray_setup(const FanGeom &g, long long r, RayWalk &w) {
    const int p = (int)(r % g.np), v = (int)(r / g.np);
    const double2 tr = g.trig_d[v];
    const double sb = tr.x, cb = tr.y;
    const double P = g.Pd[p];
    double src[3], d[3];
    const int n[3] = {g.nt, g.ns, 1};
    const double res[3] = {g.res[0], g.res[1], 1.0};
    if (g.parallel) {
        // x = width axis (t index), y = height axis (s index)
        src[0] = 0.5 * g.size[0] + P * cb + g.smax * sb;
        src[1] = 0.5 * g.size[1] + P * sb - g.smax * cb;
        d[0] = -sb;
        d[1] = cb;
    } else {
        src[0] = 0.5 * g.size[0] - g.D * sb;
        src[1] = 0.5 * g.size[1] + g.D * cb;
        d[0] = P * cb + g.D * sb;
        d[1] = P * sb - g.D * cb;
    }
    src[2] = 0.5;
    d[2] = 0.0;
    return siddon_setup(src, d, n, res, w);
}

// Line integral of ray r = view * np + bin; sets `grazing` for rays the FP64
// re-walk must redo (ref_walk.cu).
__device__ __forceinline__ float fan_ray_value(const FanGeom &g, const float *__restrict__ img, long long r,
                                               bool &grazing) {
    RayWalk w;
    grazing = false;
    if (!fan_ray_setup(g, r, w)) return 0.0f;
    grazing = w.grazing;
    return ray_integral(w, img, g.nt * g.ns - 1);
}

// Sum over all views for pixel i (t fastest) with the weighting WMODE.
template <int WMODE>
__device__ __forceinline__ float fan_pixel_sum(const FanGeom &g, const float *__restrict__ R, int i) {
    const int ti = i % g.nt, si = i / g.nt;
    const float it = (float)((ti + 0.5) * g.res[0] - 0.5 * g.size[0]);
    const float is = (float)((si + 0.5) * g.res[1] - 0.5 * g.size[1]);
    const float Rs = (float)g.D;
    const float ipint = 1.0f / g.pint;
    // pixel edges in world coordinates (BackprojectionFan2D.cu:82)
    const float tlo = (float)(ti * g.res[0]), thi_ = (float)((ti + 1) * g.res[0]);
    const float slo = (float)(si * g.res[1]), shi_ = (float)((si + 1) * g.res[1]);
    const float ct_ = (float)(0.5 * g.size[0]), cs_ = (float)(0.5 * g.size[1]);
    float acc = 0.0f;
    for (int v = 0; v < g.nb; ++v) {
        const float2 tr = g.trig_f[v];
        const float sb = tr.x, cb = tr.y;
        const float P = fmaf(it, cb, is * sb);
        float Pd = P, u = 1.0f;
        if (WMODE != BP2_FBPPAR) {
            const float S = fmaf(is, cb, -it * sb);
            u = (Rs - S) / Rs;
            Pd = P / u;
        }
        float val = 0.0f;
        if (Pd >= g.minp && Pd < g.maxp) {
            int p1 = (int)(fabsf(Pd - g.p0) * ipint);
            p1 = min(max(p1, 0), g.np - 2);
            const float w1 = fabsf(Pd - __ldg(g.Pf + p1)) * ipint;
            const float w0 = fabsf(__ldg(g.Pf + p1 + 1) - Pd) * ipint;
            const float *Rv = R + (long long)v * g.np + p1;
            val = fmaf(w0, __ldg(Rv), w1 * __ldg(Rv + 1));
        }
        if (WMODE == BP2_BACKPROJ) {
            // unit direction of the source->detector-point line and its far end
            const float ex0 = fmaf(Pd, cb, Rs * sb), ey0 = fmaf(Pd, sb, -Rs * cb);
            const float inv = rsqrtf(fmaf(ex0, ex0, ey0 * ey0));
            const float ex = ex0 * inv, ey = ey0 * inv;
            const float st = ct_ - Rs * sb, ss = cs_ + Rs * cb;
            const float a_end = 2.0f * Rs;
            float a;
            const float at = (tlo - st) / ex;
            const float s_at = fmaf(at, ey, ss);
            if (s_at >= 0.0f && s_at <= shi_) {
                a = at;
            } else {
                const float as = (slo - ss) / ey;
                const float t_as = fmaf(as, ex, st);
                if (t_as >= 0.0f && t_as <= thi_) a = as;
                else continue;
            }
            acc = fmaf(val, 2.0f * fabsf(a_end - a), acc);
        } else if (WMODE == BP2_FBPFAN) {
            acc += val / (u * u) * g.bint;
        } else {
            acc += val * g.bint;
        }
    }
    return acc;
}

// Block-level sum of a double into *out with one atomic per block, for any
// blockDim.x that is a multiple of 32 and at most 1024.
__device__ __forceinline__ void block_sum_any(double v, double *out) {
    __shared__ double part[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) part[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double w = lane < nw ? part[lane] : 0.0;
        w = warp_sum(w);
        if (lane == 0) atomicAdd(out, w);
    }
    __syncthreads();
}

// block_sum_any for per-thread FP32 terms (FP32 warp sums, FP64 partials).
__device__ __forceinline__ void block_sum_any_f(float v, double *out) {
    __shared__ double part[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) part[wid] = (double)v;
    __syncthreads();
    if (wid == 0) {
        double w = lane < nw ? part[lane] : 0.0;
        w = warp_sum(w);
        if (lane == 0) atomicAdd(out, w);
    }
    __syncthreads();
}

}  // namespace ct
