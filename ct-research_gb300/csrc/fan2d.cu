// fan2d.cu -- single-slice 2D fan- and parallel-beam projectors and
// backprojectors (device code in fan2d_dev.cuh).  One thread per ray for the
// forward projectors, one thread per pixel (all views, sum in a register,
// written once) for the backprojectors.
#include "fan2d_dev.cuh"

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
    float r2 = 0.0f, b2 = 0.0f;
    if (active) {
        bool grazing;
        const float val = fan_ray_value(g, img, r, grazing);
        if (grazing) graze_push(gl, (unsigned long long)r, (unsigned long long)r);
        if (MODE == 0) {
            out[r] = (OutT)val;
        } else {
            const float bb = b[r];
            const float rr = bb - val;
            const float sc = rowsum ? 1.0f / (rowsum[r] + eps) : 1.0f;
            out[r] = (OutT)(rr * sc);
            r2 = grazing ? 0.0f : rr * rr;   // grazing rays: added by the FP64 re-walk
            b2 = bb * bb;
        }
    }
    if (MODE == 1) {
        block_sum_atomic_f<F2_BLOCK / 32>(r2, norms);
        block_sum_atomic_f<F2_BLOCK / 32>(b2, norms + 1);
    }
}

template <int WMODE, bool UPDATE>
__global__ void __launch_bounds__(F2_BLOCK)
fan_bp_kernel(const FanGeom g, const float *__restrict__ R, float *__restrict__ img,
              const float *__restrict__ colsum, float eps, float lambda, float lo, float hi) {
    const int i = blockIdx.x * F2_BLOCK + threadIdx.x;
    if (i >= g.nt * g.ns) return;
    const float acc = fan_pixel_sum<WMODE>(g, R, i);
    if (UPDATE) {
        const float x = img[i] + lambda * acc / (colsum[i] + eps);
        img[i] = fminf(fmaxf(x, lo), hi);
    } else {
        img[i] = acc;
    }
}

}  // namespace

// The set-up table: ray r's walk set-up as fan_ray_setup_compute makes it.
__global__ void __launch_bounds__(256)
fan_ray_table_kernel(const FanGeom g, FanRay *__restrict__ tab) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= (long long)g.nb * g.np) return;
    RayWalk w;
    const bool hit = fan_ray_setup_compute(g, r, w);
    FanRay t;
    t.a0t = w.a0; t.a0s = w.a1; t.dat = w.d0; t.das = w.d1;
    t.L = w.L; t.scale = w.scale;
    t.idx = w.idx; t.nseg = w.nseg;
    t.st = w.s0; t.ss = w.s1;
    t.flags = (hit ? 1 : 0) | (w.grazing ? 2 : 0);
    t.pad_ = 0;
    tab[r] = t;
}

int fan_ray_table_launch(const FanGeom &g0, FanRay *tab, cudaStream_t st) {
    FanGeom g = g0;
    fan_geom_derive(g);
    g.ray_tab = nullptr;
    const long long n = (long long)g.nb * g.np;
    fan_ray_table_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, tab);
    CT_LAUNCH_CHECK("fan_ray_table_kernel");
    return CT_OK;
}

// mode 0: forward projection (float); 1: residual (float); 3: forward projection into double
int fan_fp_launch(const FanGeom &g0, const float *img, void *out, const float *b, const float *rowsum,
                  float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st) {
    FanGeom g = g0;
    fan_geom_derive(g);
    const long long nray = (long long)g.nb * g.np;
    const unsigned blocks = (unsigned)((nray + F2_BLOCK - 1) / F2_BLOCK);
    CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(*gl.count), st), "graze list reset");
    if (mode == 0)
        fan_fp_kernel<float, 0><<<blocks, F2_BLOCK, 0, st>>>(g, img, (float *)out, nullptr, nullptr, 0.f, nullptr, gl);
    else if (mode == 1)
        fan_fp_kernel<float, 1><<<blocks, F2_BLOCK, 0, st>>>(g, img, (float *)out, b, rowsum, eps, norms, gl);
    else
        fan_fp_kernel<double, 0><<<blocks, F2_BLOCK, 0, st>>>(g, img, (double *)out, nullptr, nullptr, 0.f, nullptr, gl);
    CT_LAUNCH_CHECK("fan_fp_kernel");
    return fan_fixup_launch(g, img, out, mode == 3, b, rowsum, eps, norms, mode == 1 ? 1 : 0, gl, st);
}

// wmode: 0 BackprojectionFan2D weight, 1 FBPfan, 2 FBPpara
int fan_bp_launch(const FanGeom &g0, const float *R, float *img, int wmode, const float *colsum, float eps,
                  float lambda, float lo, float hi, bool update, cudaStream_t st) {
    FanGeom g = g0;
    fan_geom_derive(g);
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
