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

constexpr int TV_BX = 32, TV_BY = 8;   // gradient block: 32 x 8 columns

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

// The gradient of one sub-step.  A block owns a 32 x 8 tile of columns and a
// run of kc planes; it keeps three planes of x (the tile plus a one-voxel halo
// on every side, 34 x 10) in shared memory, prefetching the plane after next
// into registers while it works on the current one.  Each voxel's forward
// differences and norm are evaluated once (as fdiff does, same operations)
// and shared through shared memory with the voxels whose backward terms need
// them; threads 0-39 also evaluate the 40 halo points (column i0 - 1, row
// j0 - 1) whose terms the tile's edge voxels need; the (i, j, k-1) term stays
// in a register from the previous plane.  One double atomic per block.
__global__ void __launch_bounds__(TV_BX * TV_BY)
tv_grad_kernel(const float *__restrict__ x, float *__restrict__ g, int nx, int ny, int nz, int kc, float eps2,
               double *__restrict__ sumsq) {
    constexpr int W = TV_BX + 2, H = TV_BY + 2, NT = TV_BX * TV_BY, PW = W * H;
    static_assert(PW <= 2 * NT && TV_BX + TV_BY <= NT, "tile and halo sizes");
    __shared__ float T[3 * PW];
    __shared__ float Px[H][W], Py[H][W];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TV_BX + tx;
    const int i0 = blockIdx.x * TV_BX, j0 = blockIdx.y * TV_BY;
    const int k0 = blockIdx.z * kc, k1 = min(k0 + kc, nz);
    const int plane = nx * ny;
    const int i = i0 + tx, j = j0 + ty;
    const bool in = i < nx && j < ny;
    // tile element e -> clamped global offset in a plane (halo outside the volume: never used)
    auto toff = [&](int e) {
        const int gi = min(max(i0 - 1 + e % W, 0), nx - 1), gj = min(max(j0 - 1 + e / W, 0), ny - 1);
        return gj * nx + gi;
    };
    const int e1 = tid + NT;
    const bool has1 = e1 < PW;
    const int o0 = toff(tid), o1 = has1 ? toff(e1) : 0;
    // halo point of this thread (tid < 40): column i0 - 1 for tid < 8, row j0 - 1 for 8 <= tid < 40
    const bool hcol = tid < TV_BY, hrow = tid >= TV_BY && tid < TV_BY + TV_BX;
    const int hr = hcol ? tid + 1 : 0, hc = hcol ? 0 : tid - TV_BY + 1;          // tile coordinates
    const int hgi = i0 - 1 + hc, hgj = j0 - 1 + hr;                                // global coordinates
    const bool hdo = (hcol && i0 > 0 && hgj < ny) || (hrow && j0 > 0 && hgi < nx);
    // plane buffers, rotated each plane: cur (k), nxt (k + 1), spare (k - 1, then k + 2)
    int cur = 0, nxt = PW, spare = 2 * PW;
    const int zk1 = min(k0 + 1, nz - 1);
    T[cur + tid] = __ldg(x + k0 * plane + o0);
    T[nxt + tid] = __ldg(x + zk1 * plane + o0);
    if (has1) {
        T[cur + e1] = __ldg(x + k0 * plane + o1);
        T[nxt + e1] = __ldg(x + zk1 * plane + o1);
    }
    float pz_prev = 0.0f;
    if (in && k0 > 0) {
        float ax, ay, az, an;
        fdiff(x, nx, ny, nz, i, j, k0 - 1, eps2, ax, ay, az, an);
        pz_prev = az * an;
    }
    __syncthreads();
    float s = 0.0f;                 // this thread's g^2 over its (at most 32) planes
    const float *px0 = x + o0, *px1 = x + o1;
    for (int k = k0; k < k1; ++k) {
        const bool more = k + 1 < k1;                        // the next plane needs plane k + 2
        float r0 = 0.0f, r1 = 0.0f;
        if (more) {
            const int zp = min(k + 2, nz - 1) * plane;
            r0 = __ldg(px0 + zp);
            if (has1) r1 = __ldg(px1 + zp);
        }
        const bool zf = k + 1 < nz;
        // forward differences and norm at tile point (r, c) = global (gi, gj, k), as fdiff
        auto fd = [&](int r, int c, int gi, int gj, float &dx, float &dy, float &dz, float &inv_n) {
            const int e = r * W + c;
            const float v = T[cur + e];
            dx = (gi + 1 < nx) ? T[cur + e + 1] - v : 0.0f;
            dy = (gj + 1 < ny) ? T[cur + e + W] - v : 0.0f;
            dz = zf ? T[nxt + e] - v : 0.0f;
            inv_n = rsqrtf(dx * dx + dy * dy + dz * dz + eps2);
        };
        float dx, dy, dz, inv_n;
        fd(ty + 1, tx + 1, i, j, dx, dy, dz, inv_n);
        Px[ty + 1][tx + 1] = dx * inv_n;
        Py[ty + 1][tx + 1] = dy * inv_n;
        if (hdo) {
            float ax, ay, az, an;
            fd(hr, hc, hgi, hgj, ax, ay, az, an);
            if (hcol) Px[hr][0] = ax * an;
            else Py[0][hc] = ay * an;
        }
        __syncthreads();
        float gv = -(dx + dy + dz) * inv_n;
        if (i > 0) gv += Px[ty + 1][tx];
        if (j > 0) gv += Py[ty][tx + 1];
        if (k > 0) gv += pz_prev;
        pz_prev = dz * inv_n;
        if (in) {
            g[k * plane + j * nx + i] = gv;
            s = fmaf(gv, gv, s);
        }
        if (more) {                                          // plane k + 2 replaces plane k - 1
            T[spare + tid] = r0;
            if (has1) T[spare + e1] = r1;
        }
        const int t = cur;
        cur = nxt;
        nxt = spare;
        spare = t;
        __syncthreads();
    }
    block_sum_atomic_f<TV_BX * TV_BY / 32>(s, sumsq);
}

__global__ void __launch_bounds__(256)
tv_apply_kernel(float *__restrict__ x, const float *__restrict__ g, long long n, float step, float lo,
                const double *__restrict__ sumsq) {
    const double ss = *sumsq;
    if (!(ss > 0.0)) return;
    const float scale = (float)(step * sqrt((double)n / ss));
#pragma unroll 4
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
#pragma unroll 4
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = fmaxf(fmaf(-scale, g[i], x[i]), lo);
}

// alpha <- alpha * alpha_red when the TV phase moved x more than r_max times the data step
__global__ void asd_alpha_kernel(double *state, float alpha_red, float r_max) {
    if (sqrt(state[2]) > (double)r_max * sqrt(state[1])) state[0] *= (double)alpha_red;
}

__global__ void __launch_bounds__(256)
sq_diff_kernel(const float *__restrict__ a, const float *__restrict__ b, long long n, double *__restrict__ out) {
    // FP32 partial sums of 16 terms, flushed into an FP64 sum (FP64 per
    // element would bound this kernel on GB300)
    double s = 0.0;
    float f = 0.0f;
    int c = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = a[i] - b[i];
        f = fmaf(d, d, f);
        if (++c == 16) {
            s += (double)f;
            f = 0.0f;
            c = 0;
        }
    }
    s += (double)f;
    block_sum_atomic<8>(s, out);
}

// 32 x 8 column tiles, and runs of kc planes: up to 32, fewer when that leaves
// under ~8 blocks per SM
dim3 tv_grid(int nx, int ny, int nz, int &kc) {
    const long long gx = (nx + TV_BX - 1) / TV_BX, gy = (ny + TV_BY - 1) / TV_BY;
    const long long fill = gx * gy * nz / (8LL * sm_count());
    kc = (int)std::min<long long>(nz, std::max<long long>(2, std::min<long long>(32, fill)));
    return dim3((unsigned)gx, (unsigned)gy, (unsigned)((nz + kc - 1) / kc));
}

}  // namespace

int tv_flow_launch(float *x, float *work, double *scratch, int nx, int ny, int nz, int iters, float step, float eps,
                   float lo, cudaStream_t st) {
    CT_REQUIRE(nx > 0 && ny > 0 && nz > 0, "tv: sizes must be positive");
    CT_REQUIRE((long long)nx * ny * nz < (1LL << 31), "tv: volume too large");
    const long long n = (long long)nx * ny * nz;
    dim3 block(TV_BX, TV_BY);
    int kc = 1;
    const dim3 grid = tv_grid(nx, ny, nz, kc);
    const int ablocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
    for (int it = 0; it < iters; ++it) {
        CT_CUDA(cudaMemsetAsync(scratch, 0, sizeof(double), st), "tv memset");
        tv_grad_kernel<<<grid, block, 0, st>>>(x, work, nx, ny, nz, kc, eps * eps, scratch);
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
    dim3 block(TV_BX, TV_BY);
    int kc = 1;
    const dim3 grid = tv_grid(nx, ny, nz, kc);
    const int ablocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 8);
    CT_CUDA(cudaMemsetAsync(state + 1, 0, 2 * sizeof(double), st), "asd memset");
    if (int s = sq_diff_sum_launch(x, prev, n, state + 1, st)) return s;        // dp2
    CT_CUDA(cudaMemcpyAsync(prev, x, n * sizeof(float), cudaMemcpyDeviceToDevice, st), "asd copy");
    for (int it = 0; it < iters; ++it) {
        CT_CUDA(cudaMemsetAsync(scratch, 0, sizeof(double), st), "tv memset");
        tv_grad_kernel<<<grid, block, 0, st>>>(x, work, nx, ny, nz, kc, eps * eps, scratch);
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
