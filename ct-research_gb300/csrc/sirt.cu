// sirt.cu -- regulariser and reduction kernels of the SIRT(-TV) loops.
//
// TV step.  The reference has no SIRT+TV driver; its TV building block is
// the TV-flow update of tv.m (Exterior_toolbox/Code_ProLu_OptDenoise/tv.m:
// 30-44: I <- I + dt * curvature, epsilon-regularised gradient).  This file
// runs the same flow in 3D with forward differences and Neumann boundaries:
//   TV_eps(x) = sum_v sqrt(|D+ x|_v^2 + eps^2),  g = dTV_eps/dx,
//   g_v = -(dx_v + dy_v + dz_v)/n_v + dx_{v-ex}/n_{v-ex} + dy_{v-ey}/n_{v-ey} + dz_{v-ez}/n_{v-ez},
// and each sub-iteration moves x <- max(x - step * g / rms(g), lo), i.e. a
// normalised gradient step whose RMS size is `step` (ASD-POCS style).
// Two passes per sub-iteration: gradient + sum(g^2) (block reduction, one
// double atomic per block), then the update.
#include "kernels.cuh"

namespace ct {

namespace {

constexpr int TV_BX = 32, TV_BY = 4, TV_BZ = 2;

__device__ __forceinline__ float ld(const float *__restrict__ x, int i) { return __ldg(x + i); }

// forward differences and the smoothed norm at (i, j, k); zero difference
// across the last plane of each axis (Neumann)
__device__ __forceinline__ void fdiff(const float *__restrict__ x, int nx, int ny, int nz, int i, int j, int k,
                                      float eps2, float &dx, float &dy, float &dz, float &inv_n) {
    const int o = (k * ny + j) * nx + i;
    const float c = ld(x, o);
    dx = (i + 1 < nx) ? ld(x, o + 1) - c : 0.0f;
    dy = (j + 1 < ny) ? ld(x, o + nx) - c : 0.0f;
    dz = (k + 1 < nz) ? ld(x, o + nx * ny) - c : 0.0f;
    inv_n = rsqrtf(dx * dx + dy * dy + dz * dz + eps2);
}

__global__ void __launch_bounds__(TV_BX * TV_BY * TV_BZ)
tv_grad_kernel(const float *__restrict__ x, float *__restrict__ g, int nx, int ny, int nz, float eps2,
               double *__restrict__ sumsq) {
    const int i = blockIdx.x * TV_BX + threadIdx.x;
    const int j = blockIdx.y * TV_BY + threadIdx.y;
    double s = 0.0;
    // each thread walks z with the grid's z stride, so one launch adds a few
    // thousand block sums to *sumsq instead of one per 256 voxels; unrolled so
    // that several planes' loads are in flight per thread
#pragma unroll 4
    for (int k = blockIdx.z * TV_BZ + threadIdx.z; i < nx && j < ny && k < nz; k += gridDim.z * TV_BZ) {
        float dx, dy, dz, in;
        fdiff(x, nx, ny, nz, i, j, k, eps2, dx, dy, dz, in);
        float gv = -(dx + dy + dz) * in;
        if (i > 0) {
            float ax, ay, az, an;
            fdiff(x, nx, ny, nz, i - 1, j, k, eps2, ax, ay, az, an);
            gv += ax * an;
        }
        if (j > 0) {
            float ax, ay, az, an;
            fdiff(x, nx, ny, nz, i, j - 1, k, eps2, ax, ay, az, an);
            gv += ay * an;
        }
        if (k > 0) {
            float ax, ay, az, an;
            fdiff(x, nx, ny, nz, i, j, k - 1, eps2, ax, ay, az, an);
            gv += az * an;
        }
        g[(k * ny + j) * nx + i] = gv;
        s += (double)gv * gv;
    }
    block_sum_atomic<TV_BX * TV_BY * TV_BZ / 32>(s, sumsq);
}

__global__ void __launch_bounds__(256)
tv_apply_kernel(float *__restrict__ x, const float *__restrict__ g, long long n, float step, float lo,
                const double *__restrict__ sumsq) {
    const double ss = *sumsq;
    if (!(ss > 0.0)) return;
    const float scale = (float)(step * sqrt((double)n / ss));
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = fmaxf(fmaf(-scale, g[i], x[i]), lo);
}

// tv_apply_kernel with the ASD-POCS step on the device: state = (alpha, dp2, dg2)
// with dp2 the squared size of the data step, so the RMS move of the sub-step
// is alpha * sqrt(dp2 / n), i.e. scale = alpha * sqrt(dp2 / sum g^2).
__global__ void __launch_bounds__(256)
tv_apply_asd_kernel(float *__restrict__ x, const float *__restrict__ g, long long n, float lo,
                    const double *__restrict__ sumsq, const double *__restrict__ state) {
    const double ss = *sumsq, dp2 = state[1];
    if (!(ss > 0.0) || !(dp2 > 0.0)) return;
    const float scale = (float)(state[0] * sqrt(dp2 / ss));
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = fmaxf(fmaf(-scale, g[i], x[i]), lo);
}

// alpha <- alpha * alpha_red when the TV phase moved x more than r_max times the data step
__global__ void asd_alpha_kernel(double *state, float alpha_red, float r_max) {
    if (sqrt(state[2]) > (double)r_max * sqrt(state[1])) state[0] *= (double)alpha_red;
}

__global__ void __launch_bounds__(256)
sq_diff_kernel(const float *__restrict__ a, const float *__restrict__ b, long long n, double *__restrict__ out) {
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = a[i] - b[i];
        s += (double)d * d;
    }
    block_sum_atomic<8>(s, out);
}

// xy tiles of the volume, and z blocks up to ~16 blocks per SM in total
dim3 tv_grid(int nx, int ny, int nz) {
    const int gx = (nx + TV_BX - 1) / TV_BX, gy = (ny + TV_BY - 1) / TV_BY, zb = (nz + TV_BZ - 1) / TV_BZ;
    const long long want = 16LL * sm_count();
    const int gz = (int)std::max<long long>(1, std::min<long long>(zb, want / ((long long)gx * gy)));
    return dim3(gx, gy, gz);
}

}  // namespace

int tv_flow_launch(float *x, float *work, double *scratch, int nx, int ny, int nz, int iters, float step, float eps,
                   float lo, cudaStream_t st) {
    CT_REQUIRE(nx > 0 && ny > 0 && nz > 0, "tv: sizes must be positive");
    CT_REQUIRE((long long)nx * ny * nz < (1LL << 31), "tv: volume too large");
    const long long n = (long long)nx * ny * nz;
    dim3 block(TV_BX, TV_BY, TV_BZ);
    const dim3 grid = tv_grid(nx, ny, nz);
    const int ablocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
    for (int it = 0; it < iters; ++it) {
        CT_CUDA(cudaMemsetAsync(scratch, 0, sizeof(double), st), "tv memset");
        tv_grad_kernel<<<grid, block, 0, st>>>(x, work, nx, ny, nz, eps * eps, scratch);
        CT_LAUNCH_CHECK("tv_grad_kernel");
        tv_apply_kernel<<<ablocks, 256, 0, st>>>(x, work, n, step, lo, scratch);
        CT_LAUNCH_CHECK("tv_apply_kernel");
    }
    return CT_OK;
}

int tv_flow_asd_launch(float *x, float *prev, float *work, double *scratch, double *state, int nx, int ny, int nz,
                       int iters, float eps, float lo, float alpha_red, float r_max, cudaStream_t st) {
    CT_REQUIRE(nx > 0 && ny > 0 && nz > 0, "tv: sizes must be positive");
    CT_REQUIRE((long long)nx * ny * nz < (1LL << 31), "tv: volume too large");
    const long long n = (long long)nx * ny * nz;
    dim3 block(TV_BX, TV_BY, TV_BZ);
    const dim3 grid = tv_grid(nx, ny, nz);
    const int ablocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
    CT_CUDA(cudaMemsetAsync(state + 1, 0, 2 * sizeof(double), st), "asd memset");
    if (int s = sq_diff_sum_launch(x, prev, n, state + 1, st)) return s;        // dp2
    CT_CUDA(cudaMemcpyAsync(prev, x, n * sizeof(float), cudaMemcpyDeviceToDevice, st), "asd copy");
    for (int it = 0; it < iters; ++it) {
        CT_CUDA(cudaMemsetAsync(scratch, 0, sizeof(double), st), "tv memset");
        tv_grad_kernel<<<grid, block, 0, st>>>(x, work, nx, ny, nz, eps * eps, scratch);
        CT_LAUNCH_CHECK("tv_grad_kernel");
        tv_apply_asd_kernel<<<ablocks, 256, 0, st>>>(x, work, n, lo, scratch, state);
        CT_LAUNCH_CHECK("tv_apply_asd_kernel");
    }
    if (int s = sq_diff_sum_launch(x, prev, n, state + 2, st)) return s;        // dg2
    asd_alpha_kernel<<<1, 1, 0, st>>>(state, alpha_red, r_max);
    CT_LAUNCH_CHECK("asd_alpha_kernel");
    return CT_OK;
}

int sq_diff_sum_launch(const float *a, const float *b, long long n, double *out, cudaStream_t st) {
    const int blocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
    if (blocks <= 0) return CT_OK;
    sq_diff_kernel<<<blocks, 256, 0, st>>>(a, b, n, out);
    CT_LAUNCH_CHECK("sq_diff_kernel");
    return CT_OK;
}

}  // namespace ct

extern "C" {

int ct_tv_flow(float *d_x, float *d_work, double *d_scratch, int nx, int ny, int nz, int iters, float step, float eps,
               float lo, void *stream) {
    CT_REQUIRE(d_x && d_work && d_scratch, "ct_tv_flow: null argument");
    CT_REQUIRE(iters >= 0, "ct_tv_flow: negative iteration count");
    return ct::tv_flow_launch(d_x, d_work, d_scratch, nx, ny, nz, iters, step, eps, lo, ct::as_stream(stream));
}

int ct_tv_flow_asd(float *d_x, float *d_prev, float *d_work, double *d_scratch, double *d_state, int nx, int ny,
                   int nz, int iters, float eps, float lo, float alpha_red, float r_max, void *stream) {
    CT_REQUIRE(d_x && d_prev && d_work && d_scratch && d_state, "ct_tv_flow_asd: null argument");
    CT_REQUIRE(iters >= 0, "ct_tv_flow_asd: negative iteration count");
    return ct::tv_flow_asd_launch(d_x, d_prev, d_work, d_scratch, d_state, nx, ny, nz, iters, eps, lo, alpha_red, r_max,
                                  ct::as_stream(stream));
}

int ct_sq_diff_sum(const float *d_a, const float *d_b, long long n, double *d_norm, void *stream) {
    CT_REQUIRE(d_a && d_b && d_norm && n >= 0, "ct_sq_diff_sum: bad argument");
    return ct::sq_diff_sum_launch(d_a, d_b, n, d_norm, ct::as_stream(stream));
}

}  // extern "C"
