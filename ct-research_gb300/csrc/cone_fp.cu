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
#include "cone_setup.cuh"
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {

namespace {

constexpr int FP_BX = 32;   // detector columns per block (one warp)
constexpr int FP_BY = 4;    // detector rows per block
// Launch order.  Views inner (grid (P tiles, views, xi tiles)): a wave of
// resident blocks holds many views of the same few detector rows, whose rays
// cross a thin z-slab of the volume that stays in L2, instead of one whole
// view, whose rays sweep the whole volume (512 MiB at 512^3, above L2) once
// per view.  Measured at 512^3 / 360 views: 47.9 -> 43.7 ms.
#ifndef CT_FP_VIEW_INNER
#define CT_FP_VIEW_INNER 1
#endif
#ifndef CT_FP_MINB
#define CT_FP_MINB 16       // full occupancy (64 warps per SM): 32 registers, a few setup values spilled
#endif

// MODE 0: proj = A vol.  MODE 1: out = (b - A vol) * scale, norms += (|r|^2, |b|^2).
// MODE 2: count segments into *norms (as double).
template <int MODE>
__global__ void __launch_bounds__(FP_BX * FP_BY, CT_FP_MINB)
cone_fp_kernel(const ConeGeom g, int v0, const float *__restrict__ vol, const float *__restrict__ volT,
               float *__restrict__ out, const float *__restrict__ b, const float *__restrict__ rowsum, float eps,
               double *__restrict__ norms, const GrazeList gl) {
    const int p = blockIdx.x * FP_BX + threadIdx.x;
#if CT_FP_VIEW_INNER
    const int x = blockIdx.z * FP_BY + threadIdx.y;
    const int v = g.vorder[v0 + blockIdx.y];
#else
    const int x = blockIdx.y * FP_BY + threadIdx.y;
    const int v = v0 + blockIdx.z;
#endif
    const bool active = p < g.np && x < g.nx;
    const int nmax = g.nt * g.ns * g.nz - 1;
    const long long o = ((long long)v * g.nx + x) * g.np + p;
    float r2 = 0.0f, b2 = 0.0f;    // per-ray terms of the norms (FP32; block sums in FP64)
    if (active) {
        RayWalk w;
        // detector neighbours in P are offset along (cos b, sin b): read the copy
        // of the volume whose fastest axis is closest to that direction, so the
        // gathers of a warp fall on few sectors
        const float2 tr = g.trigf[v];
        const bool use_t = volT && fabsf(tr.x) > fabsf(tr.y);
        const bool hit = ray_setup(g, v, p, x, use_t, w);
        if (MODE == 2) {
            r2 = hit ? (float)w.nseg : 0.0f;   // exact: counts < 2^19
        } else {
            if (hit && w.grazing) graze_push(gl, (unsigned long long)o, (unsigned long long)o);
            const float val = hit ? ray_integral<false>(w, use_t ? volT : vol, nmax) : 0.0f;
            if (MODE == 0) {
                out[o] = val;
            } else {
                const float bb = b[o];
                const float r = bb - val;
                const float sc = rowsum ? 1.0f / (rowsum[o] + eps) : 1.0f;
                out[o] = r * sc;
                r2 = (hit && w.grazing) ? 0.0f : r * r;   // grazing rays: added by the FP64 re-walk
                b2 = bb * bb;
            }
        }
    }
    if (MODE == 1) {
        block_sum_atomic_f<FP_BX * FP_BY / 32>(r2, norms);
        block_sum_atomic_f<FP_BX * FP_BY / 32>(b2, norms + 1);
    } else if (MODE == 2) {
        block_sum_atomic_f<FP_BX * FP_BY / 32>(r2, norms);
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

int cone_fp_launch(const ConeGeom &g, const float *vol, const float *volT, const float *volU, float *out,
                   const float *b, const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl,
                   cudaStream_t st, int v0, int nv) {
    if (nv <= 0) nv = g.nb - v0;
    CT_REQUIRE(v0 >= 0 && v0 + nv <= g.nb, "cone_fp: view range out of bounds");
    dim3 block(FP_BX, FP_BY);
#if CT_FP_VIEW_INNER
    dim3 grid((g.np + FP_BX - 1) / FP_BX, nv, (g.nx + FP_BY - 1) / FP_BY);
#else
    dim3 grid((g.np + FP_BX - 1) / FP_BX, (g.nx + FP_BY - 1) / FP_BY, nv);
#endif
    CT_REQUIRE(nv <= 65535, "cone_fp: at most 65535 views per launch");
    CT_REQUIRE((g.nx + FP_BY - 1) / FP_BY <= 65535, "cone_fp: at most 262140 detector rows");
    if (mode != 2) CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(*gl.count), st), "graze list reset");
    if (mode == 0)
        cone_fp_kernel<0><<<grid, block, 0, st>>>(g, v0, vol, volT, out, nullptr, nullptr, 0.0f, nullptr, gl);
    else if (mode == 1)
        cone_fp_kernel<1><<<grid, block, 0, st>>>(g, v0, vol, volT, out, b, rowsum, eps, norms, gl);
    else
        cone_fp_kernel<2><<<grid, block, 0, st>>>(g, v0, nullptr, nullptr, nullptr, nullptr, nullptr, 0.0f, norms, gl);
    CT_LAUNCH_CHECK("cone_fp_kernel");
    if (mode != 2) return cone_fixup_launch(g, volU, out, b, rowsum, eps, norms, mode, gl, st);
    return CT_OK;
}

}  // namespace ct
