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
// alpha-parameter Siddon walk in FP32 registers (siddon.cuh), unrolled by four
// so four gathers are in flight per thread.
//
// Set-up.  The rays of one detector column (view b, column P) share the source
// and the (t, s) part of d, so they cross the same t and s planes at the same
// parameters.  That in-plane part of the set-up (entry into the (t, s) square
// and voxel, first crossings, counts; FP64 where voxel assignment at the box
// boundary needs it) is a per-column table built once per geometry
// (cone_fp_columns).  The source sits at the volume's mid-height, so a ray is
// inside the z range where it enters the (t, s) square or never enters the
// volume; per ray only the z part remains: the entry z (FP64: one FMA and one
// multiply), the first z crossing and whether the ray leaves through the top
// or bottom before the (t, s) exit.  GB300 runs FP64 at a small fraction of its
// FP32 rate: the per-ray FP64 slab test this replaces held the FP64 pipe at
// ~87% in a set-up-only launch.
#include "cone_setup.cuh"
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {

namespace {

// Block 32 columns x 2 rows, 24 blocks (48 warps) per SM at 40 registers.
// Measured at 512^3 / 360 views: 32 x 4 at 16 / 12 / 10 blocks per SM 47.6 (spills
// at 32 registers) / 40.5 / 41.9 ms; 32 x 2 at 24 blocks 39.7 ms; 32 x 8 at 6
// blocks 43.1 ms; the walk unrolled by 2 / 8 instead of 4: 41.7 / 41.5 ms.
constexpr int FP_BX = 32;   // detector columns per block (one warp)
#ifndef CT_FP_BY
#define CT_FP_BY 2
#endif
constexpr int FP_BY = CT_FP_BY;   // detector rows per block
#ifndef CT_FP_MINB
#define CT_FP_MINB 24
#endif

enum { COL_GRAZE = 1, COL_TPOS = 2, COL_TNEG = 4, COL_SPOS = 8, COL_SNEG = 16 };

// The in-plane Siddon set-up of one detector column in FP64: entry and exit on
// the (t, s) square [0, nt rt] x [0, ns rs], entry voxel and coordinates,
// first crossings and crossing counts per axis.  The face and voxel rules of
// the per-ray set-up (cone_setup.cuh), restricted to t and s; the crossing
// parameters in FP32 as the walk uses them.
__global__ void __launch_bounds__(128)
fp_columns_kernel(const ConeGeom g, FpColumn *__restrict__ cols) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)g.nb * g.np) return;
    const int v = (int)(i / g.np), p = (int)(i % g.np);
    const ViewSrc vs = g.vsrc[v];
    const double2 tr = g.trig[v];
    const float4 vf = g.vsrcf[v];
    const float2 trf = g.trigf[v];
    const double Pd = g.Pd[p];
    const float Pf = g.P[p];
    const double src[2] = {vs.src_t, vs.src_s};
    const double d[2] = {fma(Pd, tr.y, vs.dsb), fma(Pd, tr.x, -vs.dcb)};
    const float df[2] = {fmaf(Pf, trf.y, vf.z), fmaf(Pf, trf.x, -vf.w)};
    const int n[2] = {g.nt, g.ns};
    FpColumn c{};
    c.dtf = df[0];
    c.dsf = df[1];
    double a_in = -1.0e300, a_out = 1.0e300;
    int ax_in = -1, ax_out = -1;
    bool miss = false;
    for (int a = 0; a < 2; ++a) {
        if (d[a] != 0.0) {
            const double t0 = (0.0 - src[a]) / d[a], t1 = (g.ext[a] - src[a]) / d[a];
            const double lo = fmin(t0, t1), hi = fmax(t0, t1);
            if (lo > a_in) { a_in = lo; ax_in = a; }
            if (hi < a_out) { a_out = hi; ax_out = a; }
        } else if (!(src[a] > 0.0 && src[a] < g.ext[a])) {
            miss = true;
        }
    }
    if (miss || ax_in < 0 || ax_out < 0 || !(a_out > a_in)) {
        c.cntt = -1;
        cols[i] = c;
        return;
    }
    int s0[2], cnt[2], sg[2];
    float a0[2], da[2], gf[2];
    bool grazing = false;
    for (int a = 0; a < 2; ++a) {
        sg[a] = d[a] > 0.0 ? 1 : (d[a] < 0.0 ? -1 : 0);
        const double gin = (a == ax_in) ? (sg[a] > 0 ? 0.0 : (double)n[a]) : fma(a_in, d[a], src[a]) * g.ires[a];
        const double gout = (a == ax_out) ? (sg[a] > 0 ? (double)n[a] : 0.0) : fma(a_out, d[a], src[a]) * g.ires[a];
        gf[a] = (float)gin;
        s0[a] = (a == ax_in) ? (sg[a] > 0 ? 0 : n[a] - 1) : (int)floor(gin);
        int e0 = (a == ax_out) ? (sg[a] > 0 ? n[a] - 1 : 0) : (int)floor(gout);
        s0[a] = min(max(s0[a], 0), n[a] - 1);
        e0 = min(max(e0, 0), n[a] - 1);
        cnt[a] = (sg[a] == 0) ? 0 : abs(e0 - s0[a]);
        if (sg[a] != 0) {
            const double glo = fmin(gin, gout), ghi = fmax(gin, gout);
            if (ghi - glo < 1e-3 && floor(ghi + 1e-6) != floor(glo - 1e-6)) grazing = true;
        }
        // first crossing and the step between crossings, in the walk's FP32
        // (as the per-ray set-up): kept for every moving axis, since a ray that
        // leaves through the top or bottom recounts its crossings
        if (sg[a] != 0) {
            const float stepf = fabsf(__frcp_rn(df[a] * g.iresf[a]));   // parameter per plane
            const int k1 = s0[a] + (sg[a] > 0 ? 1 : 0);
            a0[a] = (float)fabs((double)k1 - gin) * stepf;
            da[a] = stepf;
        } else {
            a0[a] = __int_as_float(0x7f800000);   // +inf: no crossing on this axis
            da[a] = 0.0f;
        }
    }
    c.a_in = a_in;
    c.a0t = a0[0];
    c.a0s = a0[1];
    c.dat = da[0];
    c.das = da[1];
    c.L = (float)(a_out - a_in);
    c.gint = gf[0];
    c.gins = gf[1];
    c.s0t = s0[0];
    c.s0s = s0[1];
    c.cntt = cnt[0];
    c.cnts = cnt[1];
    c.flags = (grazing ? COL_GRAZE : 0) | (sg[0] > 0 ? COL_TPOS : 0) | (sg[0] < 0 ? COL_TNEG : 0) |
              (sg[1] > 0 ? COL_SPOS : 0) | (sg[1] < 0 ? COL_SNEG : 0);
    cols[i] = c;
}

// Crossings along an in-plane axis up to parameter L when the ray leaves
// through the top or bottom first: the exit voxel from the FP32 exit
// coordinate, as the per-ray set-up takes it for an axis it does not leave by.
__device__ __forceinline__ int recount(float gin, float dfa, float iresf, float L, int s0, int n) {
    const float gout = fmaf(L, dfa * iresf, gin);
    const int e0 = min(max((int)floorf(gout), 0), n - 1);
    return abs(e0 - s0);
}

// Walk set-up of ray (column c, row x): false for rays that miss the volume.
__device__ __forceinline__ bool ray_setup_col(const ConeGeom &g, const FpColumn &c, int x, bool tr_layout,
                                              RayWalk &w, bool &grazing) {
    grazing = c.flags & COL_GRAZE;
    if (c.cntt < 0) return false;
    const int nz = g.nz;
    const double gz = fma(c.a_in, g.xid[x], g.srcz) * g.ires[2];   // entry z in voxel units
    const float xf = g.xi[x];
    const float gstz = xf * g.iresf[2];
    float L = c.L;
    if (xf != 0.0f) {
        // along a z plane to FP64 precision (tested before the range test, so that
        // rays along the top or bottom face also get the reference's FP64 walk)
        const float ginf = (float)gz, gout = fmaf(L, gstz, ginf);
        const float glo = fminf(ginf, gout), ghi = fmaxf(ginf, gout);
        if (ghi - glo < 1e-3f && floorf(ghi + 1e-6f) != floorf(glo - 1e-6f)) grazing = true;
    }
    if (!(gz >= 0.0 && gz < (double)nz)) return false;
    const int zi = (int)gz;
    int cntt = c.cntt, cnts = c.cnts, cntz = 0, sgz = 0;
    float a0z = __int_as_float(0x7f800000), daz = 0.0f;
    if (xf != 0.0f) {
        sgz = xf > 0.0f ? 1 : -1;
        const float stepz = fabsf(__frcp_rn(gstz));   // parameter per z plane
        a0z = (float)fabs((double)(zi + (sgz > 0 ? 1 : 0)) - gz) * stepz;
        daz = stepz;
        // parameter where the ray leaves through the top or bottom face
        const float lz = (float)fabs((double)(sgz > 0 ? nz : 0) - gz) * stepz;
        if (lz < L) {
            L = lz;
            cntz = sgz > 0 ? nz - 1 - zi : zi;
            if (c.flags & (COL_TPOS | COL_TNEG)) cntt = recount(c.gint, c.dtf, g.iresf[0], L, c.s0t, g.nt);
            if (c.flags & (COL_SPOS | COL_SNEG)) cnts = recount(c.gins, c.dsf, g.iresf[1], L, c.s0s, g.ns);
        } else {
            const int e0 = min(max((int)floorf(fmaf(L, gstz, (float)gz)), 0), nz - 1);
            cntz = abs(e0 - zi);
        }
    }
    const int sgt = (c.flags & COL_TPOS) ? 1 : ((c.flags & COL_TNEG) ? -1 : 0);
    const int sgs = (c.flags & COL_SPOS) ? 1 : ((c.flags & COL_SNEG) ? -1 : 0);
    w.a0 = cntt > 0 ? c.a0t : __int_as_float(0x7f800000);
    w.a1 = cnts > 0 ? c.a0s : __int_as_float(0x7f800000);
    w.a2 = cntz > 0 ? a0z : __int_as_float(0x7f800000);
    w.n0 = w.a0; w.n1 = w.a1; w.n2 = w.a2;
    w.d0 = cntt > 0 ? c.dat : 0.0f;
    w.d1 = cnts > 0 ? c.das : 0.0f;
    w.d2 = cntz > 0 ? daz : 0.0f;
    w.k0 = w.k1 = w.k2 = 0.0f;
    if (tr_layout) {   // [z][t][s]
        w.s0 = sgt * g.ns;
        w.s1 = sgs;
        w.s2 = sgz * g.nt * g.ns;
        w.idx = (zi * g.nt + c.s0t) * g.ns + c.s0s;
    } else {           // [z][s][t]
        w.s0 = sgt;
        w.s1 = sgs * g.nt;
        w.s2 = sgz * g.nt * g.ns;
        w.idx = (zi * g.ns + c.s0s) * g.nt + c.s0t;
    }
    w.nseg = 1 + cntt + cnts + cntz;
    w.grazing = grazing;
    w.L = L;
    w.scale = sqrtf(fmaf(c.dtf, c.dtf, fmaf(c.dsf, c.dsf, xf * xf)));
    return true;
}

// MODE 0: proj = A vol.  MODE 1: out = (b - A vol) * scale, norms += (|r|^2, |b|^2).
// Launch order (grid (P tiles, views, xi tiles)), views inner: a wave of
// resident blocks holds many views of the same few detector rows, whose rays
// cross a thin z-slab of the volume that stays in L2, instead of one whole
// view, whose rays sweep the whole volume (512 MiB at 512^3, above L2) once
// per view.  Measured at 512^3 / 360 views: 47.9 -> 43.7 ms.
template <int MODE>
__global__ void __launch_bounds__(FP_BX * FP_BY, CT_FP_MINB)
cone_fp_kernel(const ConeGeom g, int v0, const FpColumn *__restrict__ cols, const float *__restrict__ vol,
               const float *__restrict__ volT, float *__restrict__ out, const float *__restrict__ b,
               const float *__restrict__ rowsum, float eps, double *__restrict__ norms, const GrazeList gl) {
    const int p = blockIdx.x * FP_BX + threadIdx.x;
    const int x = blockIdx.z * FP_BY + threadIdx.y;
    const int v = g.vorder[v0 + blockIdx.y];
    const bool active = p < g.np && x < g.nx;
    const int nmax = g.nt * g.ns * g.nz - 1;
    const long long o = ((long long)v * g.nx + x) * g.np + p;
    float r2 = 0.0f, b2 = 0.0f;    // per-ray terms of the norms (FP32; block sums in FP64)
    if (active) {
        RayWalk w;
        bool grazing;
        // detector neighbours in P are offset along (cos b, sin b): read the copy
        // of the volume whose fastest axis is closest to that direction, so the
        // gathers of a warp fall on few sectors
        const float2 tr = g.trigf[v];
        const bool use_t = volT && fabsf(tr.x) > fabsf(tr.y);
        const FpColumn c = cols[(long long)v * g.np + p];
        const bool hit = ray_setup_col(g, c, x, use_t, w, grazing);
        if (grazing) graze_push(gl, (unsigned long long)o, (unsigned long long)o);
        const float val = hit ? ray_integral<false>(w, use_t ? volT : vol, nmax) : 0.0f;
        if (MODE == 0) {
            out[o] = val;
        } else {
            const float bb = b[o];
            const float r = bb - val;
            const float sc = rowsum ? 1.0f / (rowsum[o] + eps) : 1.0f;
            out[o] = r * sc;
            r2 = grazing ? 0.0f : r * r;   // grazing rays: added by the FP64 re-walk
            b2 = bb * bb;
        }
    }
    if (MODE == 1) {
        block_sum_atomic_f<FP_BX * FP_BY / 32>(r2, norms);
        block_sum_atomic_f<FP_BX * FP_BY / 32>(b2, norms + 1);
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

// Segment count with the per-ray set-up of cone_setup.cuh, one thread per ray.
__global__ void __launch_bounds__(128)
cone_count_kernel(const ConeGeom g, double *__restrict__ count) {
    const int p = blockIdx.x * 32 + threadIdx.x;
    const int x = blockIdx.z * 4 + threadIdx.y;
    const int v = blockIdx.y;
    float n = 0.0f;
    if (p < g.np && x < g.nx) {
        RayWalk w;
        if (ray_setup(g, v, p, x, false, w)) n = (float)w.nseg;   // exact: counts < 2^19
    }
    block_sum_atomic_f<4>(n, count);
}

}  // namespace

int cone_fp_columns(const ConeGeom &g, FpColumn *cols, cudaStream_t st) {
    const long long n = (long long)g.nb * g.np;
    CT_REQUIRE(n < (1LL << 31), "cone_fp: at most 2^31 detector columns");
    fp_columns_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(g, cols);
    CT_LAUNCH_CHECK("fp_columns_kernel");
    return CT_OK;
}

int cone_transpose_ts(const ConeGeom &g, const float *vol, float *volT, cudaStream_t st) {
    CT_REQUIRE(g.nz <= 65535, "transpose: at most 65535 slices");
    dim3 block(32, 8), grid((g.nt + 31) / 32, (g.ns + 31) / 32, g.nz);
    transpose_ts_kernel<<<grid, block, 0, st>>>(vol, volT, g.nt, g.ns);
    CT_LAUNCH_CHECK("transpose_ts_kernel");
    return CT_OK;
}

int cone_fp_launch(const ConeGeom &g, const FpColumn *cols, const float *vol, const float *volT, const float *volU,
                   float *out, const float *b, const float *rowsum, float eps, double *norms, int mode,
                   const GrazeList &gl, cudaStream_t st, int v0, int nv) {
    if (nv <= 0) nv = g.nb - v0;
    CT_REQUIRE(v0 >= 0 && v0 + nv <= g.nb, "cone_fp: view range out of bounds");
    CT_REQUIRE(mode == 0 || mode == 1, "cone_fp: mode must be 0 or 1");
    CT_REQUIRE(nv <= 65535, "cone_fp: at most 65535 views per launch");
    CT_REQUIRE((g.nx + FP_BY - 1) / FP_BY <= 65535, "cone_fp: at most 262140 detector rows");
    dim3 block(FP_BX, FP_BY);
    dim3 grid((g.np + FP_BX - 1) / FP_BX, nv, (g.nx + FP_BY - 1) / FP_BY);
    CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(*gl.count), st), "graze list reset");
    if (mode == 0)
        cone_fp_kernel<0><<<grid, block, 0, st>>>(g, v0, cols, vol, volT, out, nullptr, nullptr, 0.0f, nullptr, gl);
    else
        cone_fp_kernel<1><<<grid, block, 0, st>>>(g, v0, cols, vol, volT, out, b, rowsum, eps, norms, gl);
    CT_LAUNCH_CHECK("cone_fp_kernel");
    return cone_fixup_launch(g, volU, out, b, rowsum, eps, norms, mode, gl, st);
}

int cone_count_launch(const ConeGeom &g, double *count, cudaStream_t st) {
    CT_REQUIRE(g.nb <= 65535 && (g.nx + 3) / 4 <= 65535, "cone_count: grid too large");
    dim3 block(32, 4), grid((g.np + 31) / 32, g.nb, (g.nx + 3) / 4);
    cone_count_kernel<<<grid, block, 0, st>>>(g, count);
    CT_LAUNCH_CHECK("cone_count_kernel");
    return CT_OK;
}

}  // namespace ct
