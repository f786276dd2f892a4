// cone_fp.cu -- cone-beam Siddon forward projection for sm_103a.
//
// One thread per ray (beta, xi, P).  The ray geometry is that of
// ProjectionCone (ProjectionCone_3D.cu:25-42): source at
// (C_t - D sin b, C_s + D cos b, C_z), ray through the virtual detector point
// P*u + xi*e_z on the plane through the rotation centre, so its direction is
// d = (P cos b + D sin b, P sin b - D cos b, xi).
//
// The reference walks the grid by comparing squared distances to the next
// t, s and z planes in FP64 and assigns each segment to the voxel holding its
// midpoint (:270-375).  Here the same segments are produced by an
// alpha-parameter Siddon walk: the entry and exit parameters and the entry /
// exit voxels come from an FP64 slab test (the only FP64 step: voxel
// assignment at the box boundary needs it), then the walk runs in FP32
// registers (siddon.cuh).  The walk is unrolled by four so four gathers are
// in flight per thread.
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {

namespace {

constexpr int FP_BX = 32;   // detector columns per block (one warp)
constexpr int FP_BY = 4;    // detector rows per block

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
    const float Pf = g.P[p], Xf = g.xi[x];
    const double Pd = (double)Pf;
    const double src[3] = {vs.src_t, vs.src_s, 0.5 * g.size[2]};
    const double d[3] = {fma(Pd, tr.y, vs.dsb), fma(Pd, tr.x, -vs.dcb), (double)Xf};
    const int n[3] = {g.nt, g.ns, g.nz};
    // FP32 slab test on FP32 inputs: picks the entry and exit faces
    const float srcf[3] = {(float)vs.src_t, (float)vs.src_s, (float)src[2]};
    const float df[3] = {fmaf(Pf, (float)tr.y, (float)vs.dsb), fmaf(Pf, (float)tr.x, -(float)vs.dcb), Xf};
    float tin[3], tout[3], idf[3];
    int ax_in = -1, ax_out = -1;
    float fin = -3.0e38f, fout = 3.0e38f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float hi = (float)(n[a] * g.res[a]);
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
        if (d[a] == 0.0) continue;
        const bool cand_in = (a == ax_in32) || (tin[a] > -3.0e38f && fabsf(tin[a] - fin) <= 1e-5f * fabsf(fin));
        const bool cand_out = (a == ax_out32) || (tout[a] < 3.0e38f && fabsf(tout[a] - fout) <= 1e-5f * fabsf(fout));
        if (!(cand_in || cand_out)) continue;
        const double inv = drcp1(d[a]);
        const double hi = n[a] * g.res[a];
        const bool pos = d[a] > 0.0;
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
    int vs0[3], cnt[3], sg[3];
    float a0[3], da[3];
    bool grazing = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        sg[a] = d[a] > 0.0 ? 1 : (d[a] < 0.0 ? -1 : 0);
        // entry coordinate in voxel units: exact on the entry face, FP64 elsewhere
        const double gin = (a == ax_in) ? (sg[a] > 0 ? 0.0 : (double)n[a]) : fma(a_in, d[a], src[a]) * g.ires[a];
        const float ginf = (float)gin;
        const float gstep = df[a] * (float)g.ires[a];               // voxel units per parameter unit
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

// MODE 0: proj = A vol.  MODE 1: out = (b - A vol) * scale, norms += (|r|^2, |b|^2).
// MODE 2: count segments into *norms (as double).
template <int MODE>
__global__ void __launch_bounds__(FP_BX * FP_BY)
cone_fp_kernel(const ConeGeom g, const float *__restrict__ vol, const float *__restrict__ volT,
               float *__restrict__ out, const float *__restrict__ b, const float *__restrict__ rowsum, float eps,
               double *__restrict__ norms, const GrazeList gl) {
    const int p = blockIdx.x * FP_BX + threadIdx.x;
    const int x = blockIdx.y * FP_BY + threadIdx.y;
    const int v = blockIdx.z;
    const bool active = p < g.np && x < g.nx;
    const int nmax = g.nt * g.ns * g.nz - 1;
    const long long o = ((long long)v * g.nx + x) * g.np + p;
    double r2 = 0.0, b2 = 0.0;
    if (active) {
        RayWalk w;
        // detector neighbours in P are offset along (cos b, sin b): read the copy
        // of the volume whose fastest axis is closest to that direction, so the
        // gathers of a warp fall on few sectors
        const double2 tr = g.trig[v];
        const bool use_t = volT && fabs(tr.x) > fabs(tr.y);
        const bool hit = ray_setup(g, v, p, x, use_t, w);
        if (MODE == 2) {
            r2 = hit ? (double)w.nseg : 0.0;
        } else {
            if (hit && w.grazing) {
                const int slot = atomicAdd(gl.count, 1);
                if (slot < gl.cap) gl.rays[slot] = (unsigned long long)o;
            }
            const float val = hit ? ray_integral(w, use_t ? volT : vol, nmax) : 0.0f;
            if (MODE == 0) {
                out[o] = val;
            } else {
                const float bb = b[o];
                const float r = bb - val;
                const float sc = rowsum ? 1.0f / (rowsum[o] + eps) : 1.0f;
                out[o] = r * sc;
                r2 = (hit && w.grazing) ? 0.0 : (double)r * r;   // grazing rays: added by the FP64 re-walk
                b2 = (double)bb * bb;
            }
        }
    }
    if (MODE == 1) {
        block_sum_atomic<FP_BX * FP_BY / 32>(r2, norms);
        block_sum_atomic<FP_BX * FP_BY / 32>(b2, norms + 1);
    } else if (MODE == 2) {
        block_sum_atomic<FP_BX * FP_BY / 32>(r2, norms);
    }
}

// [z][s][t] -> [z][t][s], 32x32 tiles through shared memory
__global__ void __launch_bounds__(256)
transpose_ts_kernel(const float *__restrict__ in, float *__restrict__ out, int nt, int ns) {
    __shared__ float tile[32][33];
    const int z = blockIdx.z;
    const int t0 = blockIdx.x * 32, s0 = blockIdx.y * 32;
    const float *src = in + (long long)z * nt * ns;
    float *dst = out + (long long)z * nt * ns;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int s = s0 + j, t = t0 + threadIdx.x;
        if (s < ns && t < nt) tile[j][threadIdx.x] = src[(long long)s * nt + t];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int t = t0 + j, s = s0 + threadIdx.x;
        if (s < ns && t < nt) dst[(long long)t * ns + s] = tile[threadIdx.x][j];
    }
}

}  // namespace

int cone_transpose_ts(const ConeGeom &g, const float *vol, float *volT, cudaStream_t st) {
    CT_REQUIRE(g.nz <= 65535, "transpose: at most 65535 slices");
    dim3 block(32, 8), grid((g.nt + 31) / 32, (g.ns + 31) / 32, g.nz);
    transpose_ts_kernel<<<grid, block, 0, st>>>(vol, volT, g.nt, g.ns);
    CT_LAUNCH_CHECK("transpose_ts_kernel");
    return CT_OK;
}

int cone_fp_launch(const ConeGeom &g, const float *vol, const float *volT, float *out, const float *b,
                   const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st) {
    dim3 block(FP_BX, FP_BY);
    dim3 grid((g.np + FP_BX - 1) / FP_BX, (g.nx + FP_BY - 1) / FP_BY, g.nb);
    CT_REQUIRE(g.nb <= 65535, "cone_fp: at most 65535 views per launch");
    if (mode != 2) CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(int), st), "graze list reset");
    if (mode == 0)
        cone_fp_kernel<0><<<grid, block, 0, st>>>(g, vol, volT, out, nullptr, nullptr, 0.0f, nullptr, gl);
    else if (mode == 1)
        cone_fp_kernel<1><<<grid, block, 0, st>>>(g, vol, volT, out, b, rowsum, eps, norms, gl);
    else
        cone_fp_kernel<2><<<grid, block, 0, st>>>(g, nullptr, nullptr, nullptr, nullptr, nullptr, 0.0f, norms, gl);
    CT_LAUNCH_CHECK("cone_fp_kernel");
    if (mode != 2) return cone_fixup_launch(g, vol, out, b, rowsum, eps, norms, mode, gl.rays, gl.count, gl.cap, st);
    return CT_OK;
}

}  // namespace ct
