// fan2d.cu -- 2D fan- and parallel-beam projectors and backprojectors.
//
// Forward projectors: one thread per ray, the Siddon walk of siddon.cuh on a
// one-slice volume (n[2] = 1, no z crossings).
//  * fan (ProjectionFan_2D.cu:19-216): source (C_t - D sin b, C_s + D cos b),
//    ray through the point P on the line through the centre perpendicular to
//    the central ray: d = (P cos b + D sin b, P sin b - D cos b).
//  * parallel (ProjectionParallel_2D.cu:23-243): ray of offset t at angle th,
//    direction (-sin th, cos th) in (x, y) = (width, height) coordinates,
//    through (C_x + t cos th, C_y + t sin th).
// Backprojectors: one thread per pixel with the view loop inside and the sum in
// a register; written once (no atomics).
//  * BACKPROJ (BackprojectionFan2D.cu:7-116): linear interpolation of R at the
//    pixel's detector position P/U times the reference's weight
//    2 * |T1S1 - End|: End is the far point 2*Rscan along the source->pixel
//    line and T1S1 its crossing with the pixel's low t edge (accepted when the
//    crossing's s lies in [0, s_high], as the reference tests) or else its low
//    s edge (t in [0, t_high]); pixel-views with neither add nothing.
//  * FBPFAN (FBPfan.cu:45-96): filtered R interpolated, times dbeta / U^2.
//  * FBPPAR (FBPparallel.cu:41-89): filtered R at t = x cos th + y sin th, times dth.
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {


namespace {

constexpr int F2_BLOCK = 128;

template <typename OutT, int MODE>
__global__ void __launch_bounds__(F2_BLOCK)
fan_fp_kernel(const FanGeom g, const float *__restrict__ img, OutT *__restrict__ out,
              const float *__restrict__ b, const float *__restrict__ rowsum, float eps,
              double *__restrict__ norms, const GrazeList gl) {
    const long long r = (long long)blockIdx.x * F2_BLOCK + threadIdx.x;
    const bool active = r < (long long)g.nb * g.np;
    double r2 = 0.0, b2 = 0.0;
    if (active) {
        const int p = (int)(r % g.np), v = (int)(r / g.np);
        const double2 tr = g.trig_d[v];
        const double sb = tr.x, cb = tr.y;
        const double P = g.Pd[p];
        double src[3], d[3];
        const int n[3] = {g.nt, g.ns, 1};
        double res[3] = {g.res[0], g.res[1], 1.0};
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
        RayWalk w;
        float val = 0.0f;
        if (siddon_setup(src, d, n, res, w)) {
            val = ray_integral(w, img, g.nt * g.ns - 1);
            if (w.grazing) {
                const int slot = atomicAdd(gl.count, 1);
                if (slot < gl.cap) gl.rays[slot] = (unsigned long long)r;
            }
        }
        if (MODE == 0) {
            out[r] = (OutT)val;
        } else {
            const float bb = b[r];
            const float rr = bb - val;
            const float sc = rowsum ? 1.0f / (rowsum[r] + eps) : 1.0f;
            out[r] = (OutT)(rr * sc);
            r2 = (double)rr * rr;
            b2 = (double)bb * bb;
        }
    }
    if (MODE == 1) {
        block_sum_atomic<F2_BLOCK / 32>(r2, norms);
        block_sum_atomic<F2_BLOCK / 32>(b2, norms + 1);
    }
}

enum { BP2_BACKPROJ = 0, BP2_FBPFAN = 1, BP2_FBPPAR = 2 };

template <int WMODE, bool UPDATE>
__global__ void __launch_bounds__(F2_BLOCK)
fan_bp_kernel(const FanGeom g, const float *__restrict__ R, float *__restrict__ img,
              const float *__restrict__ colsum, float eps, float lambda, float lo, float hi) {
    const int i = blockIdx.x * F2_BLOCK + threadIdx.x;
    if (i >= g.nt * g.ns) return;
    const int ti = i % g.nt, si = i / g.nt;
    const float it = (float)((ti + 0.5) * g.res[0] - 0.5 * g.size[0]);
    const float is = (float)((si + 0.5) * g.res[1] - 0.5 * g.size[1]);
    const float Rs = (float)g.D;
    const float ipint = 1.0f / g.pint;
    // pixel edges and centre in world coordinates (BackprojectionFan2D.cu:82)
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
            // index floor(|P - P0| / PInt), weights from the domain values
            // (BackprojectionFan2D.cu:44-53)
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
    if (UPDATE) {
        const float x = img[i] + lambda * acc / (colsum[i] + eps);
        img[i] = fminf(fmaxf(x, lo), hi);
    } else {
        img[i] = acc;
    }
}

}  // namespace

// mode 0: forward projection (float); 1: residual (float); 3: forward projection into double
int fan_fp_launch(const FanGeom &g, const float *img, void *out, const float *b, const float *rowsum,
                  float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st) {
    const long long nray = (long long)g.nb * g.np;
    const unsigned blocks = (unsigned)((nray + F2_BLOCK - 1) / F2_BLOCK);
    CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(int), st), "graze list reset");
    if (mode == 0)
        fan_fp_kernel<float, 0><<<blocks, F2_BLOCK, 0, st>>>(g, img, (float *)out, nullptr, nullptr, 0.f, nullptr, gl);
    else if (mode == 1)
        fan_fp_kernel<float, 1><<<blocks, F2_BLOCK, 0, st>>>(g, img, (float *)out, b, rowsum, eps, norms, gl);
    else
        fan_fp_kernel<double, 0><<<blocks, F2_BLOCK, 0, st>>>(g, img, (double *)out, nullptr, nullptr, 0.f, nullptr, gl);
    CT_LAUNCH_CHECK("fan_fp_kernel");
    return fan_fixup_launch(g, img, out, mode == 3, b, rowsum, eps, norms, mode == 1 ? 1 : 0, gl.rays, gl.count,
                            gl.cap, st);
}

// wmode: 0 BackprojectionFan2D weight, 1 FBPfan, 2 FBPpara
int fan_bp_launch(const FanGeom &g, const float *R, float *img, int wmode, const float *colsum, float eps,
                  float lambda, float lo, float hi, bool update, cudaStream_t st) {
    CT_REQUIRE(g.np >= 2, "fan_bp: at least 2 detector bins");
    const unsigned blocks = (unsigned)((g.nt * g.ns + F2_BLOCK - 1) / F2_BLOCK);
#define CT_F2_CASE(W, U) fan_bp_kernel<W, U><<<blocks, F2_BLOCK, 0, st>>>(g, R, img, colsum, eps, lambda, lo, hi)
    if (update) {
        if (wmode == 0) CT_F2_CASE(BP2_BACKPROJ, true);
        else if (wmode == 1) CT_F2_CASE(BP2_FBPFAN, true);
        else CT_F2_CASE(BP2_FBPPAR, true);
    } else {
        if (wmode == 0) CT_F2_CASE(BP2_BACKPROJ, false);
        else if (wmode == 1) CT_F2_CASE(BP2_FBPFAN, false);
        else CT_F2_CASE(BP2_FBPPAR, false);
    }
#undef CT_F2_CASE
    CT_LAUNCH_CHECK("fan_bp_kernel");
    return CT_OK;
}

}  // namespace ct
