// unet_ops.cu -- the memory-bound pieces of the warm-start U-Net around the
// tensor-core convolutions (unet_conv.cu): the 27-tap gather of the one-channel
// input, 2x max pooling and nearest upsampling with their gradients, the
// channel-major x-shifted copies read by the weight-gradient kernel, the 1x1
// output head with the residual link to the input volume, and bias gradients.
// Activations are bf16 channels-last [n][z][y][x][c]; sums are FP32.
#include <cuda_bf16.h>

#include "ct_common.cuh"

namespace ct {

namespace {

using bf16 = __nv_bfloat16;

// out[v][k] = vol[v + offset(k)] for the 27 taps (z, y, x order, zero outside), 0 for k >= 27
__global__ void im2col27_kernel(const float *__restrict__ vol, bf16 *__restrict__ out, int nx, int ny, int nz,
                                long long nvox) {
    const long long v = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (v >= nvox) return;
    const int x = static_cast<int>(v % nx);
    const int y = static_cast<int>((v / nx) % ny);
    const int z = static_cast<int>((v / ((long long)nx * ny)) % nz);
    const long long base = v - x - (long long)y * nx - (long long)z * nx * ny;
    float val[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) {
        val[k] = 0.0f;
        if (k < 27) {
            const int zz = z + k / 9 - 1, yy = y + (k / 3) % 3 - 1, xx = x + k % 3 - 1;
            if (zz >= 0 && zz < nz && yy >= 0 && yy < ny && xx >= 0 && xx < nx)
                val[k] = __ldg(vol + base + ((long long)zz * ny + yy) * nx + xx);
        }
    }
    uint4 *o = reinterpret_cast<uint4 *>(out + v * 32);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint4 w;
        uint32_t *p = reinterpret_cast<uint32_t *>(&w);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(val[q * 8 + 2 * j], val[q * 8 + 2 * j + 1]);
            p[j] = *reinterpret_cast<const uint32_t *>(&h);
        }
        o[q] = w;
    }
}

__device__ __forceinline__ void unpack8(const uint4 &q, float (&f)[8]) {
    const bf16 *h = reinterpret_cast<const bf16 *>(&q);
#pragma unroll
    for (int j = 0; j < 8; ++j) f[j] = __bfloat162float(h[j]);
}

__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    uint4 w;
    uint32_t *p = reinterpret_cast<uint32_t *>(&w);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
        p[j] = *reinterpret_cast<const uint32_t *>(&h);
    }
    return w;
}

// coarse voxel index -> the 8 fine voxels (2x in every axis), child order z, y, x
__device__ __forceinline__ void children(long long cv, int cx, int cy, int cz, long long (&ch)[8]) {
    const int x = static_cast<int>(cv % cx);
    const int y = static_cast<int>((cv / cx) % cy);
    const long long zn = cv / ((long long)cx * cy);   // n * cz + z
    const int z = static_cast<int>(zn % cz);
    const long long n = zn / cz;
    const int fx = 2 * cx, fy = 2 * cy, fz = 2 * cz;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        ch[k] = ((n * fz + 2 * z + (k >> 2)) * fy + 2 * y + ((k >> 1) & 1)) * fx + 2 * x + (k & 1);
}

// one thread per (coarse voxel, 8 channels)
__global__ void pool2_kernel(const bf16 *__restrict__ in, bf16 *__restrict__ out, int c8, int cx, int cy, int cz,
                             long long n) {
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const long long cv = i / c8;
    const int g = static_cast<int>(i % c8);
    long long ch[8];
    children(cv, cx, cy, cz, ch);
    float m[8], f[8];
    unpack8(__ldg(reinterpret_cast<const uint4 *>(in) + ch[0] * c8 + g), m);
#pragma unroll
    for (int k = 1; k < 8; ++k) {
        unpack8(__ldg(reinterpret_cast<const uint4 *>(in) + ch[k] * c8 + g), f);
#pragma unroll
        for (int j = 0; j < 8; ++j) m[j] = fmaxf(m[j], f[j]);
    }
    reinterpret_cast<uint4 *>(out)[i] = pack8(m);
}

// dx[child] = dy where the child is the first maximum of its window and that
// maximum is > 0, else 0: the pooled activations are ReLU outputs, so this is
// also the ReLU derivative of the pooling path
__global__ void pool2_bwd_kernel(const bf16 *__restrict__ x, const bf16 *__restrict__ y, const bf16 *__restrict__ dy,
                                 bf16 *__restrict__ dx, int c8, int cx, int cy, int cz, long long n) {
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const long long cv = i / c8;
    const int g = static_cast<int>(i % c8);
    long long ch[8];
    children(cv, cx, cy, cz, ch);
    float m[8], d[8], f[8], o[8];
    unpack8(__ldg(reinterpret_cast<const uint4 *>(y) + i), m);
    unpack8(__ldg(reinterpret_cast<const uint4 *>(dy) + i), d);
    bool taken[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) taken[j] = false;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        unpack8(__ldg(reinterpret_cast<const uint4 *>(x) + ch[k] * c8 + g), f);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const bool hit = !taken[j] && f[j] == m[j];
            o[j] = (hit && m[j] > 0.0f) ? d[j] : 0.0f;
            taken[j] = taken[j] || hit;
        }
        reinterpret_cast<uint4 *>(dx)[ch[k] * c8 + g] = pack8(o);
    }
}

// fine voxel = its coarse parent
__global__ void up2_kernel(const bf16 *__restrict__ in, bf16 *__restrict__ out, int c8, int cx, int cy, int cz,
                           long long n) {
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const long long cv = i / c8;
    const int g = static_cast<int>(i % c8);
    long long ch[8];
    children(cv, cx, cy, cz, ch);
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(in) + i);
#pragma unroll
    for (int k = 0; k < 8; ++k) reinterpret_cast<uint4 *>(out)[ch[k] * c8 + g] = q;
}

// coarse gradient = sum of the 8 fine gradients
__global__ void up2_bwd_kernel(const bf16 *__restrict__ dout, bf16 *__restrict__ din, int c8, int cx, int cy, int cz,
                               long long n) {
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const long long cv = i / c8;
    const int g = static_cast<int>(i % c8);
    long long ch[8];
    children(cv, cx, cy, cz, ch);
    float s[8], f[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) s[j] = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        unpack8(__ldg(reinterpret_cast<const uint4 *>(dout) + ch[k] * c8 + g), f);
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] += f[j];
    }
    reinterpret_cast<uint4 *>(din)[i] = pack8(s);
}

// [n][z][y][x][c] -> three channel-major copies [n][ctot][z][y][x] at channel
// offset coff, shifted along x by -1, 0, +1 (zero outside); a null output is skipped.
// Block: 32 x 8 threads, tile of 32 x positions x 32 channels of one (n, z, y)
// row; grid (rows, x tiles, channel tiles), rows in x (up to 2^31 - 1).
__global__ void __launch_bounds__(256)
shift_t_kernel(const bf16 *__restrict__ in, bf16 *__restrict__ om, bf16 *__restrict__ o0, bf16 *__restrict__ op,
               int c, int ctot, int coff, int nx, int ny, int nz) {
    __shared__ float tile[34][33];
    const int x0 = blockIdx.y * 32, c0 = blockIdx.z * 32;
    const long long row = blockIdx.x;   // (n * nz + z) * ny + y
    const long long nzy = (long long)nz * ny;
    const long long n = row / nzy, zy = row % nzy;
    const bf16 *src = in + row * nx * c;
    for (int e = threadIdx.y * 32 + threadIdx.x; e < 34 * 32; e += 256) {
        const int xi = e / 32, cc = e % 32;
        const int x = x0 - 1 + xi, ch = c0 + cc;
        tile[xi][cc] = (x >= 0 && x < nx && ch < c) ? __bfloat162float(src[(long long)x * c + ch]) : 0.0f;
    }
    __syncthreads();
    const long long plane = nzy * nx;   // voxels of one channel
    for (int cc = threadIdx.y; cc < 32; cc += 8) {
        const int ch = c0 + cc, x = x0 + threadIdx.x;
        if (ch >= c || x >= nx) continue;
        const long long o = (n * ctot + coff + ch) * plane + zy * nx + x;
        if (om) om[o] = __float2bfloat16(tile[threadIdx.x][cc]);        // value at x - 1
        if (o0) o0[o] = __float2bfloat16(tile[threadIdx.x + 1][cc]);
        if (op) op[o] = __float2bfloat16(tile[threadIdx.x + 2][cc]);    // value at x + 1
    }
}

// out[v] = base[v] + b + sum_c w[c] f[v][c]   (32 channels)
__global__ void head_kernel(const bf16 *__restrict__ f, const float *__restrict__ w, const float *__restrict__ b,
                            const float *__restrict__ base, float *__restrict__ out, long long nvox) {
    const long long v = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (v >= nvox) return;
    float s = __ldg(b) + (base ? __ldg(base + v) : 0.0f);
    const uint4 *p = reinterpret_cast<const uint4 *>(f + v * 32);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float g[8];
        unpack8(__ldg(p + q), g);
#pragma unroll
        for (int j = 0; j < 8; ++j) s = fmaf(__ldg(w + q * 8 + j), g[j], s);
    }
    out[v] = s;
}

// df[v][c] = w[c] dout[v] (f[v][c] > 0); dw[c] += sum_v dout f; db += sum_v dout
__global__ void __launch_bounds__(256)
head_bwd_kernel(const float *__restrict__ dout, const bf16 *__restrict__ f, const float *__restrict__ w,
                bf16 *__restrict__ df, float *__restrict__ dw, float *__restrict__ db, long long nvox) {
    float acc[33];
#pragma unroll
    for (int j = 0; j < 33; ++j) acc[j] = 0.0f;
    float wr[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) wr[j] = __ldg(w + j);
    for (long long v = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; v < nvox;
         v += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float d = __ldg(dout + v);
        acc[32] += d;
        const uint4 *p = reinterpret_cast<const uint4 *>(f + v * 32);
        uint4 *o = reinterpret_cast<uint4 *>(df + v * 32);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float g[8], r[8];
            unpack8(__ldg(p + q), g);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                acc[q * 8 + j] = fmaf(d, g[j], acc[q * 8 + j]);
                r[j] = g[j] > 0.0f ? wr[q * 8 + j] * d : 0.0f;
            }
            o[q] = pack8(r);
        }
    }
    __shared__ float red[8][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 33; ++j) {
        const float s = warp_sum(acc[j]);
        if (lane == 0) red[warp][j] = s;
    }
    __syncthreads();
    if (threadIdx.x < 33) {
        float s = 0.0f;
        for (int k = 0; k < 8; ++k) s += red[k][threadIdx.x];
        atomicAdd(threadIdx.x < 32 ? dw + threadIdx.x : db, s);
    }
}

// db[c] += sum_v dy[v][c]; block of 256 threads = 256 / c voxel lanes x c channels
__global__ void __launch_bounds__(256)
colsum_kernel(const bf16 *__restrict__ dy, float *__restrict__ db, int c, long long nvox) {
    const int lanes = 256 / c;
    const int ch = threadIdx.x % c, l = threadIdx.x / c;
    float s = 0.0f;
    for (long long v = blockIdx.x * static_cast<long long>(lanes) + l; v < nvox;
         v += static_cast<long long>(gridDim.x) * lanes)
        s += __bfloat162float(dy[v * c + ch]);
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    if (l == 0) {
        for (int k = 1; k < lanes; ++k) s += red[k * c + ch];
        atomicAdd(db + ch, s);
    }
}

unsigned blocks_for(long long n, int threads) { return static_cast<unsigned>((n + threads - 1) / threads); }

bool al16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

}  // namespace ct

using namespace ct;

extern "C" {

int ct_unet_im2col27(const float *vol, int nb, int nz, int ny, int nx, void *out, void *stream) {
    CT_REQUIRE(vol && out && al16(out), "im2col27: null or unaligned pointer");
    CT_REQUIRE(nb > 0 && nz > 0 && ny > 0 && nx > 0, "im2col27: empty volume");
    const long long n = (long long)nb * nz * ny * nx;
    CT_REQUIRE(blocks_for(n, 256) < (1u << 31), "im2col27: volume too large");
    im2col27_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(vol, static_cast<bf16 *>(out), nx, ny, nz, n);
    CT_LAUNCH_CHECK("im2col27_kernel");
    return CT_OK;
}

static int pool_args(const void *a, const void *b, int c, int nb, int nz, int ny, int nx, long long &n) {
    CT_REQUIRE(a && b && al16(a) && al16(b), "pool/up: null or unaligned pointer");
    CT_REQUIRE(c > 0 && c % 8 == 0, "pool/up: channels must be a positive multiple of 8");
    CT_REQUIRE(nb > 0 && nz > 0 && ny > 0 && nx > 0, "pool/up: empty coarse volume");
    n = (long long)nb * nz * ny * nx * (c / 8);
    CT_REQUIRE(blocks_for(n, 256) < (1u << 31), "pool/up: volume too large");
    return CT_OK;
}

// Sizes are those of the coarse volume (nz, ny, nx); the fine one is twice each.
int ct_unet_pool2(const void *in, void *out, int c, int nb, int nz, int ny, int nx, void *stream) {
    long long n;
    if (int s = pool_args(in, out, c, nb, nz, ny, nx, n)) return s;
    pool2_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(static_cast<const bf16 *>(in),
                                                                     static_cast<bf16 *>(out), c / 8, nx, ny, nz * nb, n);
    CT_LAUNCH_CHECK("pool2_kernel");
    return CT_OK;
}

int ct_unet_pool2_bwd(const void *x, const void *y, const void *dy, void *dx, int c, int nb, int nz, int ny, int nx,
                      void *stream) {
    long long n;
    if (int s = pool_args(x, dx, c, nb, nz, ny, nx, n)) return s;
    CT_REQUIRE(y && dy && al16(y) && al16(dy), "pool2_bwd: null or unaligned pointer");
    pool2_bwd_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(
        static_cast<const bf16 *>(x), static_cast<const bf16 *>(y), static_cast<const bf16 *>(dy),
        static_cast<bf16 *>(dx), c / 8, nx, ny, nz * nb, n);
    CT_LAUNCH_CHECK("pool2_bwd_kernel");
    return CT_OK;
}

int ct_unet_up2(const void *in, void *out, int c, int nb, int nz, int ny, int nx, void *stream) {
    long long n;
    if (int s = pool_args(in, out, c, nb, nz, ny, nx, n)) return s;
    up2_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(static_cast<const bf16 *>(in),
                                                                   static_cast<bf16 *>(out), c / 8, nx, ny, nz * nb, n);
    CT_LAUNCH_CHECK("up2_kernel");
    return CT_OK;
}

int ct_unet_up2_bwd(const void *dout, void *din, int c, int nb, int nz, int ny, int nx, void *stream) {
    long long n;
    if (int s = pool_args(dout, din, c, nb, nz, ny, nx, n)) return s;
    up2_bwd_kernel<<<blocks_for(n, 256), 256, 0, as_stream(stream)>>>(
        static_cast<const bf16 *>(dout), static_cast<bf16 *>(din), c / 8, nx, ny, nz * nb, n);
    CT_LAUNCH_CHECK("up2_bwd_kernel");
    return CT_OK;
}

int ct_unet_shift_t(const void *in, int c, int nb, int nz, int ny, int nx, void *om, void *o0, void *op, int ctot,
                    int coff, void *stream) {
    CT_REQUIRE(in && (om || o0 || op), "shift_t: null pointer");
    CT_REQUIRE(c > 0 && coff >= 0 && coff + c <= ctot, "shift_t: channel range outside the output");
    CT_REQUIRE(nb > 0 && nz > 0 && ny > 0 && nx > 0, "shift_t: empty volume");
    const long long rows = (long long)nb * nz * ny;
    CT_REQUIRE(rows < (1ll << 31), "shift_t: volume too large");
    dim3 grid(static_cast<unsigned>(rows), (nx + 31) / 32, (c + 31) / 32);
    CT_REQUIRE(grid.y <= 65535 && grid.z <= 65535, "shift_t: x or channel count too large");
    shift_t_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(
        static_cast<const bf16 *>(in), static_cast<bf16 *>(om), static_cast<bf16 *>(o0), static_cast<bf16 *>(op), c,
        ctot, coff, nx, ny, nz);
    CT_LAUNCH_CHECK("shift_t_kernel");
    return CT_OK;
}

int ct_unet_head(const void *f, const float *w, const float *b, const float *base, float *out, long long nvox,
                 void *stream) {
    CT_REQUIRE(f && w && b && out && al16(f), "head: null or unaligned pointer");
    CT_REQUIRE(nvox > 0 && blocks_for(nvox, 256) < (1u << 31), "head: bad voxel count");
    head_kernel<<<blocks_for(nvox, 256), 256, 0, as_stream(stream)>>>(static_cast<const bf16 *>(f), w, b, base, out,
                                                                       nvox);
    CT_LAUNCH_CHECK("head_kernel");
    return CT_OK;
}

int ct_unet_head_bwd(const float *dout, const void *f, const float *w, void *df, float *dw, float *db, long long nvox,
                     void *stream) {
    CT_REQUIRE(dout && f && w && df && dw && db && al16(f) && al16(df), "head_bwd: null or unaligned pointer");
    CT_REQUIRE(nvox > 0, "head_bwd: bad voxel count");
    const unsigned grid = static_cast<unsigned>(std::min<long long>(blocks_for(nvox, 256), 4LL * sm_count()));
    head_bwd_kernel<<<grid, 256, 0, as_stream(stream)>>>(dout, static_cast<const bf16 *>(f), w, static_cast<bf16 *>(df),
                                                         dw, db, nvox);
    CT_LAUNCH_CHECK("head_bwd_kernel");
    return CT_OK;
}

int ct_unet_colsum(const void *dy, int c, long long nvox, float *db, void *stream) {
    CT_REQUIRE(dy && db, "colsum: null pointer");
    CT_REQUIRE(c > 0 && c <= 256 && 256 % c == 0, "colsum: channels must divide 256");
    CT_REQUIRE(nvox > 0, "colsum: bad voxel count");
    const long long lanes = 256 / c;
    const unsigned grid = static_cast<unsigned>(std::min<long long>((nvox + lanes - 1) / lanes, 8LL * sm_count()));
    colsum_kernel<<<grid, 256, 0, as_stream(stream)>>>(static_cast<const bf16 *>(dy), db, c, nvox);
    CT_LAUNCH_CHECK("colsum_kernel");
    return CT_OK;
}

}  // extern "C"
