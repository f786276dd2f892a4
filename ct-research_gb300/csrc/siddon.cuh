// siddon.cuh -- FP32 alpha-parameter Siddon walk with an FP64 entry/exit set-up.
//
// Produces the segments of the reference's grid walks (ProjectionCone_3D.cu:
// 270-375, ProjectionFan_2D.cu:162-216, ProjectionParallel_2D.cu:163-243):
// the line is cut at every t, s and z plane and each piece is charged to the
// voxel it lies in.  The entry and exit parameters and voxels come from an
// FP64 slab test (voxel assignment at the box boundary needs it); the walk
// itself runs in FP32 registers, each plane-crossing parameter recomputed from
// an integer crossing counter with one FMA, so no rounding accumulates along
// the ray.  Volumes are [z][s][t] with t fastest; 2D images use n[2] = 1.
#pragma once
#include "ct_common.cuh"

namespace ct {

struct RayWalk {
    float n0, n1, n2;      // next crossing parameter per axis (INF when none)
    float a0, a1, a2;      // parameter of the first crossing per axis
    float d0, d1, d2;      // parameter step between crossings per axis
    float k0, k1, k2;      // crossings taken per axis
    int s0, s1, s2;        // linear-index step per axis
    int idx;               // current voxel
    int nseg;              // segments along the ray
    float L;               // exit parameter
    float scale;           // |d| in mm per parameter unit
    bool grazing;          // runs along a grid plane to FP64 precision (see ref_walk.cu)
};

// FP64 slab test against the box [0, n*res] and walk set-up for the line
// src + alpha * d.  Returns false for lines that miss the box.  ires = 1 / res
// and ext = n * res per axis, as the host computes them (IEEE double, the same
// values a device division would give).
__device__ __forceinline__ bool siddon_setup(const double src[3], const double d[3], const int n[3],
                                             const double res[3], const double ires[3], const double ext[3],
                                             RayWalk &w) {
    double inv[3];
    double a_in = -1.0e300, a_out = 1.0e300;
    int ax_in = -1, ax_out = -1;   // axes whose faces the line enters and leaves through
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double hi = ext[a];
        if (d[a] != 0.0) {
            inv[a] = drcp(d[a]);
            const double t0 = (0.0 - src[a]) * inv[a];
            const double t1 = (hi - src[a]) * inv[a];
            const double lo_t = fmin(t0, t1), hi_t = fmax(t0, t1);
            if (lo_t > a_in) { a_in = lo_t; ax_in = a; }
            if (hi_t < a_out) { a_out = hi_t; ax_out = a; }
        } else {
            inv[a] = 0.0;
            if (!(src[a] > 0.0 && src[a] < hi)) return false;
        }
    }
    if (!(a_out > a_in)) return false;

    // FP32 copies of d (for |d| in FP32)
    const float L = (float)(a_out - a_in);
    float df[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) df[a] = (float)d[a];
    int vs[3], cnt[3], sg[3];
    float a0[3], da[3];
    bool grazing = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double ir = ires[a];
        const double gin = (src[a] + a_in * d[a]) * ir;
        const double gout = (src[a] + a_out * d[a]) * ir;
        // signs from the bits (no FP64 compare)
        const long long db = __double_as_longlong(d[a]);
        sg[a] = (db << 1) == 0 ? 0 : (db < 0 ? -1 : 1);
        // nearly parallel to the planes of this axis and within reach of one:
        // the reference's charge then depends on FP64 rounding of a clamped slope
        if (sg[a] != 0 && fabs(gout - gin) < 1e-3) {
            const double glo = fmin(gin, gout), ghi = fmax(gin, gout);
            if (floor(ghi + 1e-9) != floor(glo - 1e-9)) grazing = true;
        }
        // On the entry / exit face the voxel is known exactly; on the other axes
        // the voxel is the floor of the coordinate, as the reference's
        // midpoint-floor rule gives for lines along a grid plane.
        int s0 = (a == ax_in) ? (sg[a] > 0 ? 0 : n[a] - 1) : (int)floor(gin);
        int e0 = (a == ax_out) ? (sg[a] > 0 ? n[a] - 1 : 0) : (int)floor(gout);
        s0 = min(max(s0, 0), n[a] - 1);
        e0 = min(max(e0, 0), n[a] - 1);
        vs[a] = s0;
        cnt[a] = abs(e0 - s0);
        if (cnt[a] > 0) {
            const double step = res[a] * inv[a];            // parameter per plane, signed
            const double k1 = (double)(s0 + (sg[a] > 0 ? 1 : 0));
            a0[a] = (float)((k1 - gin) * step);
            da[a] = (float)fabs(step);
        } else {
            a0[a] = __int_as_float(0x7f800000);   // +inf: no crossing on this axis
            da[a] = 0.0f;
        }
    }
    w.a0 = a0[0]; w.a1 = a0[1]; w.a2 = a0[2];
    w.n0 = a0[0]; w.n1 = a0[1]; w.n2 = a0[2];
    w.d0 = da[0]; w.d1 = da[1]; w.d2 = da[2];
    w.k0 = w.k1 = w.k2 = 0.0f;
    w.s0 = sg[0];
    w.s1 = sg[1] * n[0];
    w.s2 = sg[2] * n[0] * n[1];
    w.idx = (vs[2] * n[1] + vs[1]) * n[0] + vs[0];
    w.nseg = 1 + cnt[0] + cnt[1] + cnt[2];
    w.grazing = grazing;
    w.L = L;
    w.scale = sqrtf(fmaf(df[0], df[0], fmaf(df[1], df[1], df[2] * df[2])));
    return true;
}

// One walk step: the parameter length of the current segment and its voxel;
// then advance to the next voxel (ties resolved t, then s, then z).  Every
// next-crossing parameter is recomputed from its counter with one FMA (an
// axis that did not advance gets its previous value back exactly), so the
// step needs no selects.  The segment ends at the next crossing; the caller
// takes nseg - 1 steps and ends the last segment at the exit parameter L.
// CLAMP keeps the index inside [0, nmax] for reads from unpadded arrays;
// without it the caller's array must extend a slice beyond both ends (where
// rounding lets a crossing of one axis come before the last one of another).
template <bool CLAMP = true>
__device__ __forceinline__ void walk_step(RayWalk &w, float &acur, int nmax, float &len, int &vox) {
    const float m12 = fminf(w.n1, w.n2);
    const float m = fminf(w.n0, m12);
    const float an = m;
    len = an - acur;
    acur = an;
    vox = w.idx;
    const bool b0 = w.n0 <= m12;
    const bool b1 = !b0 && (w.n1 <= w.n2);
    const bool b2 = !b0 && !b1;
    if (b0) w.k0 += 1.0f;
    if (b1) w.k1 += 1.0f;
    if (b2) w.k2 += 1.0f;
    w.n0 = fmaf(w.k0, w.d0, w.a0);
    w.n1 = fmaf(w.k1, w.d1, w.a1);
    w.n2 = fmaf(w.k2, w.d2, w.a2);
    const int nidx = w.idx + (b0 ? w.s0 : (b1 ? w.s1 : w.s2));
    w.idx = CLAMP ? min(max(nidx, 0), nmax) : nidx;
}

// Sum of segment length x voxel value along the ray, times |d|: nseg - 1
// segments end at crossings (four at a time, so four gathers are in flight),
// the last one at the exit L.
template <bool CLAMP = true>
__device__ __forceinline__ float ray_integral(RayWalk &w, const float *__restrict__ vol, int nmax) {
    float acc = 0.0f, acur = 0.0f;
    const int ninner = w.nseg - 1;
    int it = 0;
    for (; it + 4 <= ninner; it += 4) {
        float l0, l1, l2, l3;
        int i0, i1, i2, i3;
        walk_step<CLAMP>(w, acur, nmax, l0, i0);
        walk_step<CLAMP>(w, acur, nmax, l1, i1);
        walk_step<CLAMP>(w, acur, nmax, l2, i2);
        walk_step<CLAMP>(w, acur, nmax, l3, i3);
        const float v0 = __ldg(vol + i0), v1 = __ldg(vol + i1);
        const float v2 = __ldg(vol + i2), v3 = __ldg(vol + i3);
        acc = fmaf(l0, v0, acc);
        acc = fmaf(l1, v1, acc);
        acc = fmaf(l2, v2, acc);
        acc = fmaf(l3, v3, acc);
    }
    for (; it < ninner; ++it) {
        float l;
        int i;
        walk_step<CLAMP>(w, acur, nmax, l, i);
        acc = fmaf(l, __ldg(vol + i), acc);
    }
    acc = fmaf(w.L - acur, __ldg(vol + w.idx), acc);
    return acc * w.scale;
}

}  // namespace ct
