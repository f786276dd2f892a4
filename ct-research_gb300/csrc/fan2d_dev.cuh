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
#include "ffloat.cuh"
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {

enum { BP2_BACKPROJ = 0, BP2_FBPFAN = 1, BP2_FBPPAR = 2 };

// Walk set-up of ray r = view * np + bin, computed; false for rays that miss the image.
__device__ __forceinline__ bool fan_ray_setup_compute(const FanGeom &g, long long r, RayWalk &w) {
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
    const double ires[3] = {g.ires[0], g.ires[1], 1.0}, ext[3] = {g.ext[0], g.ext[1], 1.0};
    return siddon_setup(src, d, n, res, ires, ext, w);
}

// Walk set-up of ray r: from the geometry's set-up table when it has one (the
// same values, stored once per plan), else computed.
__device__ __forceinline__ bool fan_ray_setup(const FanGeom &g, long long r, RayWalk &w) {
    if (!g.ray_tab) return fan_ray_setup_compute(g, r, w);
    const float4 *q = reinterpret_cast<const float4 *>(g.ray_tab + r);
    const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2);
    const int flags = __float_as_int(q2.z);
    const float inf = __int_as_float(0x7f800000);
    w.a0 = q0.x; w.a1 = q0.y; w.a2 = inf;
    w.n0 = q0.x; w.n1 = q0.y; w.n2 = inf;
    w.d0 = q0.z; w.d1 = q0.w; w.d2 = 0.0f;
    w.k0 = w.k1 = w.k2 = 0.0f;
    w.L = q1.x;
    w.scale = q1.y;
    w.idx = __float_as_int(q1.z);
    w.nseg = __float_as_int(q1.w);
    w.s0 = __float_as_int(q2.x);
    w.s1 = __float_as_int(q2.y);
    w.s2 = 0;
    w.grazing = (flags & 2) != 0;
    return (flags & 1) != 0;
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

// The reference's weight 2 |T1S1 - End| of one pixel-view in FP64
// (BackprojectionFan2D.cu:56-114), each operation rounded on its own as the
// reference's double arithmetic: End is the point 2 Rscan along the ray from
// the source through the detector point pd (angle atan(pd / Rscan)), T1S1 the
// line's crossing with the pixel's low t edge when its s lies in [0, s_high],
// else with its low s edge when its t lies in [0, t_high]; 0 when neither (the
// reference's thread returns).  Used where the FP32 tests lie within rounding
// distance of those bounds.
static __device__ __noinline__ float fan_chord_fp64(const FanGeom &g, int ti, int si, double sb, double cb, double pd) {
    const double R = g.D, ct = 0.5 * g.size[0], cs = 0.5 * g.size[1];
    const double src_t = __dsub_rn(ct, __dmul_rn(R, sb)), src_s = __dadd_rn(cs, __dmul_rn(R, cb));
    const double th = atan(__ddiv_rn(pd, R));
    const double smax = __dmul_rn(2.0, R);
    const double st = __dmul_rn(smax, sin(th)), cr = __dsub_rn(R, __dmul_rn(smax, cos(th)));
    const double end_t = __dsub_rn(__dadd_rn(ct, __dmul_rn(st, cb)), __dmul_rn(cr, sb));
    const double end_s = __dadd_rn(__dadd_rn(cs, __dmul_rn(st, sb)), __dmul_rn(cr, cb));
    const double dt = __dsub_rn(end_t, src_t), ds = __dsub_rn(end_s, src_s);
    double t2s = __ddiv_rn(ds, dt == 0.0 ? __dadd_rn(dt, 1e-15) : dt);
    double s2t = __ddiv_rn(dt, ds == 0.0 ? __dadd_rn(ds, 1e-15) : ds);
    t2s = fmin(fmax(t2s, -1e16), 1e16);
    s2t = fmin(fmax(s2t, -1e16), 1e16);
    const double tlo = __dmul_rn((double)ti, g.res[0]), thi = __dmul_rn((double)(ti + 1), g.res[0]);
    const double slo = __dmul_rn((double)si, g.res[1]), shi = __dmul_rn((double)(si + 1), g.res[1]);
    const double tlo_s = __dadd_rn(src_s, __dmul_rn(__dsub_rn(tlo, src_t), t2s));
    const double slo_t = __dadd_rn(src_t, __dmul_rn(__dsub_rn(slo, src_s), s2t));
    double T1, S1;
    if (tlo_s >= 0.0 && tlo_s <= shi) {
        T1 = tlo;
        S1 = tlo_s;
    } else if (slo_t >= 0.0 && slo_t <= thi) {
        T1 = slo_t;
        S1 = slo;
    } else {
        return 0.0f;
    }
    const double et = __dsub_rn(T1, end_t), es = __dsub_rn(S1, end_s);
    return (float)__dmul_rn(2.0, __dsqrt_rn(__dadd_rn(__dmul_rn(et, et), __dmul_rn(es, es))));
}

// a >= b and a < b for a float-float value and a float bound
__device__ __forceinline__ bool ff_ge(ff a, float b) { return a.hi > b || (a.hi == b && a.lo >= 0.0f); }
__device__ __forceinline__ bool ff_lt(ff a, float b) { return a.hi < b || (a.hi == b && a.lo < 0.0f); }

// The reference's detector coordinate P / U of pixel (ti, si) in one view in
// float-float (ffloat.cuh), for the pixel-views where the FP32 value lies near
// a decision boundary.  The pixel centre (ti + 1/2) res - size / 2 comes from
// the geometry's float-float constants (fan_geom_derive), so this runs no
// FP64.  One division, by a reciprocal and a float-float correction.
static __device__ __noinline__ ff fan_pd_ff(const FanGeom &g, int ti, int si, float sb, float cb, int wmode) {
    const ff it2 = ff_sub(ff_mul_f(ff{g.res_ff[0].x, g.res_ff[0].y}, (float)ti + 0.5f),
                          ff{g.hsize_ff[0].x, g.hsize_ff[0].y});
    const ff is2 = ff_sub(ff_mul_f(ff{g.res_ff[1].x, g.res_ff[1].y}, (float)si + 0.5f),
                          ff{g.hsize_ff[1].x, g.hsize_ff[1].y});
    const ff P2 = ff_add(ff_mul_f(it2, cb), ff_mul_f(is2, sb));
    if (wmode == BP2_FBPPAR) return P2;
    const ff R2 = {g.D_ff.x, g.D_ff.y};
    const ff den = ff_sub(R2, ff_sub(ff_mul_f(is2, cb), ff_mul_f(it2, sb)));   // Rscan - S
    const ff num = ff_mul(P2, R2);                                             // P / ((Rscan - S) / Rscan)
    const float r = __frcp_rn(den.hi);
    const float q1 = __fmul_rn(num.hi, r);
    const ff rem = ff_sub(num, ff_mul_f(den, q1));
    return ff_fast2sum(q1, __fmul_rn(rem.hi, r));
}

// Sum over all views for pixel i (t fastest) with the weighting WMODE.
// The bin is the reference's floor(|Pd - P0| / PInt), PInt the spacing of the
// first two samples, with weights |Pd - P[i]| / PInt from the actual sample
// values: a discontinuous rule (float samples drift from the implied grid, by
// ~1e-3 mm over 1024 bins) that an FP32 Pd reproduces except near a bin or
// range boundary.  There (about 1e-3 of the pixel-views) Pd is recomputed in
// float-float, as the reference's FP64 value.
template <int WMODE>
__device__ __forceinline__ float fan_pixel_sum(const FanGeom &g, const float *__restrict__ R, int i) {
    const int ti = i % g.nt, si = i / g.nt;
    const float it = (float)((ti + 0.5) * g.res[0] - 0.5 * g.size[0]);
    const float is = (float)((si + 0.5) * g.res[1] - 0.5 * g.size[1]);
    const float Rs = (float)g.D;
    const float ipint = 1.0f / g.pint;
    // pixel edges in world coordinates (BackprojectionFan2D.cu:82)
    const float tlo = (float)(ti * g.res[0]), slo = (float)(si * g.res[1]);
    const float ct_ = (float)(0.5 * g.size[0]), cs_ = (float)(0.5 * g.size[1]);
    // pixel centre and half sizes, in world coordinates
    const float pct = (float)((ti + 0.5) * g.res[0]), pcs = (float)((si + 0.5) * g.res[1]);
    const float ht = (float)(0.5 * g.res[0]), hs = (float)(0.5 * g.res[1]);
    // FP32 error of Pd is a few ulp of the scan's extent (~3e-4 bins at 1024 bins of
    // 0.78 mm): within 3x that of a bin or range boundary Pd is recomputed
    const float near_m = 6e-7f * (Rs + (float)(g.size[0] + g.size[1])) * ipint;
    float acc = 0.0f;
    for (int v = 0; v < g.nb; ++v) {
        const float2 tr = g.trig_f[v];
        const float sb = tr.x, cb = tr.y;
        const float P = fmaf(it, cb, is * sb);
        float Pd = P, u = 1.0f;
        if (WMODE == BP2_FBPFAN) {
            const float S = fmaf(is, cb, -it * sb);
            u = (Rs - S) / Rs;
            Pd = P / u;
        } else if (WMODE == BP2_BACKPROJ) {
            // P / U = P Rs / (Rs - S), approximate division (2 ulp): with the products'
            // rounding Pd is within ~4 ulp, inside the margin below, and the bin
            // decision is re-taken in float-float near a boundary either way
            const float S = fmaf(is, cb, -it * sb);
            Pd = __fdividef(__fmul_rn(P, Rs), __fsub_rn(Rs, S));
        }
        float Plo = 0.0f;   // low part of Pd where it is recomputed in float-float
        const float qf = fabsf(Pd - g.p0) * ipint;
        const bool near = fabsf(qf - rintf(qf)) < near_m || fabsf(Pd - g.minp) * ipint < near_m ||
                          fabsf(Pd - g.maxp) * ipint < near_m;
        if (near) {
            const ff Pd2 = fan_pd_ff(g, ti, si, sb, cb, WMODE);
            Pd = Pd2.hi;
            Plo = Pd2.lo;
        }
        const ff Pd2 = {Pd, Plo};
        float val = 0.0f;
        if (ff_ge(Pd2, g.minp) && ff_lt(Pd2, g.maxp)) {
            // far from a bin boundary the FP32 quotient has the reference's floor
            int p1 = near ? ff_floor(ff_mul(ff_abs(ff_sub(Pd2, ff{g.p0, 0.0f})), ff{g.ipint_ff.x, g.ipint_ff.y}))
                          : (int)qf;
            p1 = min(max(p1, 0), g.np - 2);
            const float pa = __ldg(g.Pf + p1), pb = __ldg(g.Pf + p1 + 1);
            const float w1 = fabsf(__fadd_rn(__fsub_rn(Pd, pa), Plo)) * ipint;
            const float w0 = fabsf(__fsub_rn(__fsub_rn(pb, Pd), Plo)) * ipint;
            const float *Rv = R + (long long)v * g.np + p1;
            val = fmaf(w0, __ldg(Rv), w1 * __ldg(Rv + 1));
        }
        if (WMODE == BP2_BACKPROJ) {
            // unit direction of the source->detector-point line and its far end
            const float ex0 = fmaf(Pd, cb, Rs * sb), ey0 = fmaf(Pd, sb, -Rs * cb);
            const float inv = rsqrtf(fmaf(ex0, ex0, ey0 * ey0));
            const float ex = ex0 * inv, ey = ey0 * inv;
            const float st = fmaf(-Rs, sb, ct_), ss = fmaf(Rs, cb, cs_);
            const float a_end = 2.0f * Rs;
            float w;
            // The line passes through the pixel centre, so its crossing with the low t
            // edge lies ds_t = -ht ey / ex from the centre in s, and with the low s edge
            // dt_s = -hs ex / ey in t.  The reference's tests s in [0, s_high] and t in
            // [0, t_high] are decided on these small offsets, whose FP32 error is ~1e-7 of
            // their size (approximate reciprocals, a few ulp); within 1e-5 of a bound the
            // FP64 construction decides.
            // (explicitly rounded products: no FMA contraction, so the single-slice and
            // batched builds of this function give identical results)
            const float iex = __fdividef(1.0f, ex);
            const float ds_t = __fmul_rn(__fmul_rn(-ht, ey), iex);
            const float c1 = pcs + ds_t, c2 = hs - ds_t;           // s_at >= 0, s_at <= s_high
            bool tie = fabsf(c1) < 1e-5f * (pcs + fabsf(ds_t)) || fabsf(c2) < 1e-5f * (hs + fabsf(ds_t));
            bool none = false;
            float a = __fmul_rn(__fsub_rn(tlo, st), iex);
            if (!(c1 >= 0.0f && c2 >= 0.0f)) {
                const float iey = __fdividef(1.0f, ey);
                const float dt_s = __fmul_rn(__fmul_rn(-hs, ex), iey);
                const float d1 = pct + dt_s, d2 = ht - dt_s;       // t_as >= 0, t_as <= t_high
                tie = tie || fabsf(d1) < 1e-5f * (pct + fabsf(dt_s)) || fabsf(d2) < 1e-5f * (ht + fabsf(dt_s));
                a = __fmul_rn(__fsub_rn(slo, ss), iey);
                none = !(d1 >= 0.0f && d2 >= 0.0f);
            }
            if (tie) {
                // the FP64 construction needs the reference's P / U, not the FP32 one
                const ff pe = near ? Pd2 : fan_pd_ff(g, ti, si, sb, cb, WMODE);
                w = fan_chord_fp64(g, ti, si, (double)sb, (double)cb, (double)pe.hi + (double)pe.lo);
            } else {
                if (none) continue;
                w = 2.0f * fabsf(a_end - a);
            }
            acc = fmaf(val, w, acc);
        } else if (WMODE == BP2_FBPFAN) {
            acc = fmaf(val / (u * u), g.bint, acc);
        } else {
            acc = fmaf(val, g.bint, acc);
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
