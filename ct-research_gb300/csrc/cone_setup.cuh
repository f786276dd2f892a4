// cone_setup.cuh -- Siddon walk set-up of one cone-beam ray on its own, for
// the system-matrix export (sysmat.cu) and the segment count (cone_fp.cu).
// The forward projector takes the in-plane part of the same set-up from a
// per-column table (cone_fp.cu); both follow the same face and voxel rules,
// so their segments differ at most by float rounding of the crossing
// parameters (A x matches the projection to ~1e-7).
#pragma once
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {

namespace {

// 1/x in FP64 from the FP32 reciprocal and one Newton-Raphson step
// y <- y + y (1 - x y): relative error ~ (2^-23)^2, ample for the slab test.
__device__ __forceinline__ double drcp1(double x) {
    const double y = (double)__frcp_rn((float)x);
    return fma(y, fma(-x, y, 1.0), y);
}

// Walk set-up of ray (v, p, x).  The source and direction follow
// ProjectionCone_3D.cu:25-42: src = (C_t - D sin b, C_s + D cos b, C_z),
// d = (P cos b + D sin b, P sin b - D cos b, xi).  An FP32 slab test picks the
// entry and exit faces; the entry / exit parameters and the entry voxel are
// then computed in FP64 from those faces (both candidates in FP64 when two
// faces tie within FP32 rounding).  The rest of the set-up is FP32.
// `tr_layout` selects the [z][t][s] copy of the volume: linear strides follow.
__device__ __forceinline__ bool ray_setup(const ConeGeom &g, int v, int p, int x, bool tr_layout, RayWalk &w) {
    const ViewSrc vs = g.vsrc[v];
    const double2 tr = g.trig[v];
    const float4 vf = g.vsrcf[v];
    const float2 trf = g.trigf[v];
    const float Pf = g.P[p], Xf = g.xi[x];
    const double Pd = g.Pd[p];
    const double src[3] = {vs.src_t, vs.src_s, g.srcz};
    const double d[3] = {fma(Pd, tr.y, vs.dsb), fma(Pd, tr.x, -vs.dcb), g.xid[x]};
    const int n[3] = {g.nt, g.ns, g.nz};
    // signs of d from the bits (no FP64 compare): -1, 0 or +1
    int sg[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const long long b = __double_as_longlong(d[a]);
        sg[a] = (b << 1) == 0 ? 0 : (b < 0 ? -1 : 1);
    }
    // FP32 slab test on FP32 inputs: picks the entry and exit faces
    const float srcf[3] = {vf.x, vf.y, g.srczf};
    const float df[3] = {fmaf(Pf, trf.y, vf.z), fmaf(Pf, trf.x, -vf.w), Xf};
    float tin[3], tout[3], idf[3];
    int ax_in = -1, ax_out = -1;
    float fin = -3.0e38f, fout = 3.0e38f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float hi = g.extf[a];
        idf[a] = __frcp_rn(df[a]);
        if (df[a] != 0.0f) {
            const float t0 = (0.0f - srcf[a]) * idf[a], t1 = (hi - srcf[a]) * idf[a];
            tin[a] = fminf(t0, t1);
            tout[a] = fmaxf(t0, t1);
        } else {
            if (!(srcf[a] > 0.0f && srcf[a] < hi)) return false;
            tin[a] = -3.0e38f;
            tout[a] = 3.0e38f;
        }
        if (tin[a] > fin) { fin = tin[a]; ax_in = a; }
        if (tout[a] < fout) { fout = tout[a]; ax_out = a; }
    }
    // clear misses end here; near-tangent rays are decided by the FP64 test below
    if (ax_in < 0 || ax_out < 0 || !(fout >= fin - 1e-5f * fabsf(fin))) return false;
    // FP64 entry / exit parameters on the chosen faces; any other face within
    // FP32 rounding of them is evaluated in FP64 too
    double a_in = -1.0e300, a_out = 1.0e300;
    const int ax_in32 = ax_in, ax_out32 = ax_out;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (sg[a] == 0) continue;
        const bool cand_in = (a == ax_in32) || (tin[a] > -3.0e38f && fabsf(tin[a] - fin) <= 1e-5f * fabsf(fin));
        const bool cand_out = (a == ax_out32) || (tout[a] < 3.0e38f && fabsf(tout[a] - fout) <= 1e-5f * fabsf(fout));
        if (!(cand_in || cand_out)) continue;
        const double inv = drcp1(d[a]);
        const double hi = g.ext[a];
        const bool pos = sg[a] > 0;
        // a line going up enters at 0 and leaves at hi; going down the reverse
        if (cand_in) {
            const double t = ((pos ? 0.0 : hi) - src[a]) * inv;
            if (t > a_in) { a_in = t; ax_in = a; }
        }
        if (cand_out) {
            const double t = ((pos ? hi : 0.0) - src[a]) * inv;
            if (t < a_out) { a_out = t; ax_out = a; }
        }
    }
    if (!(a_out > a_in)) return false;
    const float L = (float)(a_out - a_in);
    int vs0[3], cnt[3];
    float a0[3], da[3];
    bool grazing = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // entry coordinate in voxel units: exact on the entry face, FP64 elsewhere
        const double gin = (a == ax_in) ? (sg[a] > 0 ? 0.0 : (double)n[a]) : fma(a_in, d[a], src[a]) * g.ires[a];
        const float ginf = (float)gin;
        const float gstep = df[a] * g.iresf[a];               // voxel units per parameter unit
        const float stepf = fabsf(__frcp_rn(gstep));                // parameter per plane
        const float gout = fmaf(L, gstep, ginf);                    // exit coordinate, FP32
        int s0 = (a == ax_in) ? (sg[a] > 0 ? 0 : n[a] - 1) : (int)floor(gin);
        int e0 = (a == ax_out) ? (sg[a] > 0 ? n[a] - 1 : 0) : (int)floorf(gout);
        s0 = min(max(s0, 0), n[a] - 1);
        e0 = min(max(e0, 0), n[a] - 1);
        vs0[a] = s0;
        cnt[a] = (sg[a] == 0) ? 0 : abs(e0 - s0);
        if (sg[a] != 0) {
            const float glo = fminf(ginf, gout), ghi = fmaxf(ginf, gout);
            if (ghi - glo < 1e-3f && floorf(ghi + 1e-6f) != floorf(glo - 1e-6f)) grazing = true;
        }
        if (cnt[a] > 0) {
            const int k1 = s0 + (sg[a] > 0 ? 1 : 0);
            a0[a] = (float)fabs((double)k1 - gin) * stepf;
            da[a] = stepf;
        } else {
            a0[a] = __int_as_float(0x7f800000);   // +inf: no crossing on this axis
            da[a] = 0.0f;
        }
    }
    w.a0 = a0[0]; w.a1 = a0[1]; w.a2 = a0[2];
    w.n0 = a0[0]; w.n1 = a0[1]; w.n2 = a0[2];
    w.d0 = da[0]; w.d1 = da[1]; w.d2 = da[2];
    w.k0 = w.k1 = w.k2 = 0.0f;
    if (tr_layout) {   // [z][t][s]
        w.s0 = sg[0] * g.ns;
        w.s1 = sg[1];
        w.s2 = sg[2] * g.nt * g.ns;
        w.idx = (vs0[2] * g.nt + vs0[0]) * g.ns + vs0[1];
    } else {           // [z][s][t]
        w.s0 = sg[0];
        w.s1 = sg[1] * g.nt;
        w.s2 = sg[2] * g.nt * g.ns;
        w.idx = (vs0[2] * g.ns + vs0[1]) * g.nt + vs0[0];
    }
    w.nseg = 1 + cnt[0] + cnt[1] + cnt[2];
    w.grazing = grazing;
    w.L = L;
    w.scale = sqrtf(fmaf(df[0], df[0], fmaf(df[1], df[1], df[2] * df[2])));
    return true;
}

}  // namespace

}  // namespace ct

