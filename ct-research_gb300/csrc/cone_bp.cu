// cone_bp.cu -- voxel-driven cone-beam backprojection for sm_103a.
//
// Two weightings of the same bilinear detector interpolation:
//  * CHORD (Backprojection3D.cu:8-291): each voxel-view adds
//      bilinear(R) * 2 * |entry - centre|, the chord of the source->voxel-centre
//      line through the voxel.  For a line through the centre the chord is
//      2 * min_a(h_a / |d_a|) * |d| (h = half voxel, d = centre - source),
//      which equals the reference's low-face construction.
//  * FDK (FDK.cu:50-126): bilinear(filtered R) * LR^2 * dbeta, where
//      LR = D / (D - dect_s); in STICKY mode a voxel whose projection leaves
//      the detector re-adds the last in-range value of its column, as the
//      reference does because it never resets Display_pBeta (:73, :100-123).
//
// Layout: each view's projection is first repacked into 2x2 quads,
//   Q[v][x][p] = (R[x][p], R[x][p+1], R[x+1][p], R[x+1][p+1]),
// so the four bilinear taps of a voxel-view are one aligned 16-byte load.
// This trades HBM capacity (4x the sinogram, 2.3 GB at 360x512x768) for a
// quarter of the load instructions on a load-issue-bound kernel.
//
// Threads own one (t, s) column and ZC consecutive z; the view loop runs
// inside the thread with the ZC sums in registers, and each voxel is written
// once at the end (no atomics, deterministic).  The fused SIRT variant writes
// clamp(x + lambda * bp / (colsum + eps), lo, hi) instead of bp.
#include "cone_geom.cuh"

namespace ct {

namespace {

constexpr int BP_BX = 32;   // t per block
constexpr int BP_BY = 4;    // s per block
constexpr int BP_ZC = 16;   // z per thread

__global__ void __launch_bounds__(256)
pack_quads_kernel(const float *__restrict__ R, float4 *__restrict__ Q, int nb, int nx, int np) {
    const long long n = (long long)nb * nx * np;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(i % np);
        const long long rv = i / np;
        const int x = (int)(rv % nx);
        const bool pr = p + 1 < np, xr = x + 1 < nx;
        float4 q;
        q.x = R[i];
        q.y = pr ? R[i + 1] : 0.0f;
        q.z = xr ? R[i + np] : 0.0f;
        q.w = (pr && xr) ? R[i + np + 1] : 0.0f;
        Q[i] = q;
    }
}

enum { W_CHORD = 0, W_FDK_ZERO = 1, W_FDK_STICKY = 2 };

template <int WMODE, bool UPDATE>
__global__ void __launch_bounds__(BP_BX * BP_BY)
cone_bp_kernel(const ConeGeom g, const float4 *__restrict__ Q, float *__restrict__ vol,
               const float *__restrict__ colsum, float eps, float lambda, float lo, float hi) {
    const int ti = blockIdx.x * BP_BX + threadIdx.x;
    const int si = blockIdx.y * BP_BY + threadIdx.y;
    const int z0 = blockIdx.z * BP_ZC;
    if (ti >= g.nt || si >= g.ns) return;

    const float rt = (float)g.res[0], rs = (float)g.res[1], rz = (float)g.res[2];
    const float ct_ = (float)(0.5 * g.size[0]), cs_ = (float)(0.5 * g.size[1]), cz_ = (float)(0.5 * g.size[2]);
    const float it = (float)((ti + 0.5) * g.res[0] - 0.5 * g.size[0]);
    const float is = (float)((si + 0.5) * g.res[1] - 0.5 * g.size[1]);
    const float D = (float)g.D;
    const float ipint = 1.0f / g.pint, ixint = 1.0f / g.xint;
    (void)ct_; (void)cs_; (void)rt; (void)rs;

    float acc[BP_ZC];
    float zg[BP_ZC], zq[BP_ZC];   // per z: h_z / |iz| and iz^2 (chord weight)
#pragma unroll
    for (int k = 0; k < BP_ZC; ++k) {
        acc[k] = 0.0f;
        const float iz = (float)((z0 + k + 0.5) * g.res[2] - 0.5 * g.size[2]);
        zg[k] = 0.5f * rz / fabsf(iz);
        zq[k] = iz * iz;
    }
    const float ht = 0.5f * (float)g.res[0], hs = 0.5f * (float)g.res[1];
    const float x_base = (float)(0.5 * g.res[2] - 0.5 * g.size[2]);   // iz at z = 0
    const long long vstride = (long long)g.nx * g.np;

    for (int v = 0; v < g.nb; ++v) {
        const double2 tr = g.trig[v];
        const float sb = (float)tr.x, cb = (float)tr.y;
        const float dect_t = fmaf(it, cb, is * sb);
        const float dect_s = fmaf(is, cb, -it * sb);
        const float lr = D / (D - dect_s);
        const float P = dect_t * lr;
        if (!(P >= g.minp && P < g.maxp)) continue;   // whole column off the detector
        // detector column and its interpolation weight
        const float pf = (P - g.p0) * g.psgn * ipint;
        int p1 = __float2int_rd(pf);
        p1 = min(max(p1, 0), g.np - 2);
        const float fp = pf - (float)p1;
        // xi(z) = (x_base + z rz) * lr; detector rows in range for z in [zlo, zhi]
        const float xslope = rz * lr, xoff = x_base * lr;
        const float zlo_f = (g.minx - xoff) / xslope, zhi_f = (g.maxx - xoff) / xslope;
        int zlo = (int)ceilf(zlo_f);             // first z with xi >= minx
        int zhi = (int)ceilf(zhi_f) - 1;         // last z with xi < maxx
        // fractional row index as a linear function of z
        const float B = xslope * g.xsgn * ixint;
        const float A = (xoff - g.x0) * g.xsgn * ixint;
        const float4 *Qv = Q + (long long)v * vstride + p1;

        float wv = 1.0f, mts = 0.0f, qq = 0.0f;
        if (WMODE == W_CHORD) {
            const float dt = it + D * sb, ds = is - D * cb;
            mts = fminf(ht / fabsf(dt), hs / fabsf(ds));
            qq = fmaf(dt, dt, ds * ds);
        } else {
            wv = lr * lr * g.bint;
        }
        if (WMODE == W_FDK_STICKY) {
            if (zhi < zlo) continue;
        }
#pragma unroll
        for (int k = 0; k < BP_ZC; ++k) {
            int z = z0 + k;
            bool in = (z >= zlo) && (z <= zhi);
            if (WMODE == W_FDK_STICKY) {
                in = z >= zlo;
                z = min(z, zhi);
            }
            const float xf = fmaf((float)z, B, A);
            int x1 = __float2int_rd(xf);
            x1 = min(max(x1, 0), g.nx - 2);
            const float fr = xf - (float)x1;
            const float4 q = __ldg(Qv + (long long)x1 * g.np);
            const float top = fmaf(fp, q.y - q.x, q.x);
            const float bot = fmaf(fp, q.w - q.z, q.z);
            const float val = fmaf(fr, bot - top, top);
            float w;
            if (WMODE == W_CHORD) {
                w = 2.0f * fminf(mts, zg[k]) * sqrtf(qq + zq[k]);
            } else {
                w = wv;
            }
            acc[k] = in ? fmaf(val, w, acc[k]) : acc[k];
        }
    }
#pragma unroll
    for (int k = 0; k < BP_ZC; ++k) {
        const int z = z0 + k;
        if (z < g.nz) {
            const long long o = ((long long)z * g.ns + si) * g.nt + ti;
            if (UPDATE) {
                const float x = vol[o] + lambda * acc[k] / (colsum[o] + eps);
                vol[o] = fminf(fmaxf(x, lo), hi);
            } else {
                vol[o] = acc[k];
            }
        }
    }
}

}  // namespace

size_t cone_quads_bytes(const ConeGeom &g) { return sizeof(float4) * (size_t)g.nb * g.nx * g.np; }

int cone_pack_quads(const ConeGeom &g, const float *R, float4 *Q, cudaStream_t st) {
    const long long n = (long long)g.nb * g.nx * g.np;
    int blocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 16);
    pack_quads_kernel<<<blocks, 256, 0, st>>>(R, Q, g.nb, g.nx, g.np);
    CT_LAUNCH_CHECK("pack_quads_kernel");
    return CT_OK;
}

// weighting: 0 chord, 1 FDK (off-detector adds 0), 2 FDK sticky
int cone_bp_launch(const ConeGeom &g, const float4 *Q, float *vol, int weighting, const float *colsum,
                   float eps, float lambda, float lo, float hi, bool update, cudaStream_t st) {
    CT_REQUIRE(g.np >= 2 && g.nx >= 2, "cone_bp: detector needs at least 2x2 samples");
    dim3 block(BP_BX, BP_BY);
    dim3 grid((g.nt + BP_BX - 1) / BP_BX, (g.ns + BP_BY - 1) / BP_BY, (g.nz + BP_ZC - 1) / BP_ZC);
#define CT_BP_CASE(W, U)                                                                     \
    cone_bp_kernel<W, U><<<grid, block, 0, st>>>(g, Q, vol, colsum, eps, lambda, lo, hi)
    if (update) {
        if (weighting == W_CHORD) CT_BP_CASE(W_CHORD, true);
        else if (weighting == W_FDK_ZERO) CT_BP_CASE(W_FDK_ZERO, true);
        else CT_BP_CASE(W_FDK_STICKY, true);
    } else {
        if (weighting == W_CHORD) CT_BP_CASE(W_CHORD, false);
        else if (weighting == W_FDK_ZERO) CT_BP_CASE(W_FDK_ZERO, false);
        else CT_BP_CASE(W_FDK_STICKY, false);
    }
#undef CT_BP_CASE
    CT_LAUNCH_CHECK("cone_bp_kernel");
    return CT_OK;
}

}  // namespace ct
