// noalloc.cu -- 2D fan FBP that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc / cudaFree while they
// run -- services that reserve all device memory once at start-up and forbid
// later allocation, and hosts whose framework owns the device memory (a
// caching pool) so that a raw cudaMalloc would bypass its accounting and
// cudaFree would synchronise the whole device under their streams.  They pass
// the sinogram and the image as device buffers they already own.
//
// Everything else the FBP needs -- the per-view (sin, cos) table, the
// detector coordinates, the filter taps, the cosine pre-weights and the
// filtered sinogram -- lives in g_fbp_scratch, a file-scope device array of
// kNoAllocScratchBytes (8 MiB).  Every GPU that loads the library holds this
// array until the process exits.  Sizes whose tables and filtered sinogram do
// not fit are rejected with CT_ERR_ARG.  The caller's angle and detector
// arrays are copied into the array with cudaMemcpyAsync (a copy, not an
// allocation) and a small kernel derives the tables from them there.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress, with that device current; make that first call
// before any stream capture.  Under CUDA's lazy module loading (the default)
// the array's memory is committed when this file's code is first used on a
// device, i.e. by that first call: a caller that reserves the rest of device
// memory afterwards should make one call first (or load modules eagerly,
// CUDA_MODULE_LOADING=EAGER).  Every call shares the one array and leaves its
// contents behind (the filter kernel zeroes the rows it accumulates into, the
// table kernel rewrites every table), so calls whose GPU work overlaps -- on
// different streams, or from different host threads -- race on it: serialise
// them.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "kernels.cuh"

namespace ct {

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;   // 8 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_fbp_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// The FBP tables from the caller's float angles and bins (already in the
// scratch array): (sin, cos) of each angle as the float of the double sine
// and cosine (a correctly rounded sinf / cosf but for astronomically rare
// ties); the Shepp-Logan taps of GFunction (FBPfan.cu:6-19) and the weights
// Rscan / sqrt(Rscan^2 + P^2) (FBPfan.cu:32), in double with the products and
// sums rounded one by one as the host tables of the allocating path are.
__global__ void __launch_bounds__(256)
fbp_tables_kernel(const float *__restrict__ beta, int nb, const float *__restrict__ P, int np, float pint,
                  double rscan, float2 *__restrict__ trig, float *__restrict__ G, double *__restrict__ w) {
    const double x = __dmul_rn((double)pint, 3.141592653589793);
    const double a = __dmul_rn(x, x);
    const int n_all = max(nb, 2 * np - 1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_all; i += gridDim.x * blockDim.x) {
        if (i < nb) {
            const double b = (double)beta[i];
            trig[i] = make_float2((float)sin(b), (float)cos(b));
        }
        if (i < 2 * np - 1) {
            const int n = abs(i - (np - 1));
            const double den = __dadd_rn(__dmul_rn(4.0, __dmul_rn((double)n, (double)n)), -1.0);
            G[i] = n == 0 ? (float)__ddiv_rn(1.0, a) : (float)__ddiv_rn(__ddiv_rn(-1.0, a), den);
        }
        if (i < np) {
            const double p = (double)P[i];
            w[i] = __ddiv_rn(rscan, __dsqrt_rn(__dadd_rn(__dmul_rn(rscan, rscan), __dmul_rn(p, p))));
        }
    }
}

// Device address of g_fbp_scratch on the current device (looked up once per device).
int scratch_address(void **out) {
    int dev = 0;
    CT_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    CT_REQUIRE(dev >= 0 && dev < kMaxDevices, "ct_FBPfan_noalloc: device index out of range");
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        CT_CUDA(cudaGetSymbolAddress(&p, g_fbp_scratch), "cudaGetSymbolAddress(g_fbp_scratch)");
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return CT_OK;
}

}  // namespace

}  // namespace ct

using namespace ct;

extern "C" int ct_FBPfan_noalloc(float *d_Display, const float *d_R, const float *Pdomain,
                                 const float *BetaScanRange, int LBeta, int LP, const double *Size, int t_length,
                                 int s_length, double Rscan, void *stream) {
    CT_REQUIRE(d_Display && d_R && Pdomain && BetaScanRange && Size, "ct_FBPfan_noalloc: null argument");
    CT_REQUIRE(LBeta > 0 && LP >= 2 && t_length > 0 && s_length > 0, "ct_FBPfan_noalloc: sizes must be positive");
    CT_REQUIRE((long long)t_length * s_length < (1LL << 31), "ct_FBPfan_noalloc: image larger than 2^31 pixels");
    CT_REQUIRE(Size[0] > 0 && Size[1] > 0, "ct_FBPfan_noalloc: Size must be positive");
    CT_REQUIRE(Rscan > 0.5 * std::sqrt(Size[0] * Size[0] + Size[1] * Size[1]),
               "ct_FBPfan_noalloc: Rscan must exceed the half diagonal of the image");
    // scratch layout: [angles (float)][P (float)][trig (float2 per view)][taps (2LP-1 float)][weights (double)]
    // [filtered sinogram]
    const size_t o_b = 0;
    const size_t o_p = align256(o_b + sizeof(float) * (size_t)LBeta);
    const size_t o_trig = align256(o_p + sizeof(float) * (size_t)LP);
    const size_t o_g = align256(o_trig + sizeof(float2) * (size_t)LBeta);
    const size_t o_w = align256(o_g + sizeof(float) * (2 * (size_t)LP - 1));
    const size_t o_rc = align256(o_w + sizeof(double) * (size_t)LP);
    const size_t total = o_rc + sizeof(float) * (size_t)LBeta * LP;
    if (total > kNoAllocScratchBytes) {
        set_error("ct_FBPfan_noalloc: LBeta * LP too large for the 8 MiB scratch array (needs " +
                  std::to_string(total) + " bytes)");
        return CT_ERR_ARG;
    }
    for (int i = 0; i < LBeta; ++i) CT_REQUIRE(std::isfinite(BetaScanRange[i]), "ct_FBPfan_noalloc: non-finite angle");
    for (int i = 0; i < LP; ++i) CT_REQUIRE(std::isfinite(Pdomain[i]), "ct_FBPfan_noalloc: non-finite bin");

    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    void *base = nullptr;
    int s = scratch_address(&base);
    if (s) return s;
    unsigned char *dev = static_cast<unsigned char *>(base);
    cudaStream_t st = as_stream(stream);

    // geometry as FBPfan derives it (FBPfan.cu:109-113): float spacing and range
    FanGeom g{};
    g.nt = t_length;
    g.ns = s_length;
    g.nb = LBeta;
    g.np = LP;
    g.size[0] = Size[0];
    g.size[1] = Size[1];
    g.res[0] = 1.0 * Size[0] / t_length;
    g.res[1] = 1.0 * Size[1] / s_length;
    g.D = Rscan;
    g.parallel = 0;
    g.pint = std::fabs(Pdomain[1] - Pdomain[0]);
    g.bint = LBeta > 1 ? std::fabs(BetaScanRange[1] - BetaScanRange[0]) : 0.0f;
    g.maxp = std::max(Pdomain[0], Pdomain[LP - 1]);
    g.minp = std::min(Pdomain[0], Pdomain[LP - 1]);
    g.p0 = Pdomain[0];
    g.psgn = Pdomain[LP - 1] < Pdomain[0] ? -1.0f : 1.0f;

    // the caller's angles and bins into the array, then the tables from them
    CT_CUDA(cudaMemcpyAsync(dev + o_b, BetaScanRange, sizeof(float) * (size_t)LBeta, cudaMemcpyHostToDevice, st),
            "ct_FBPfan_noalloc: angle upload");
    CT_CUDA(cudaMemcpyAsync(dev + o_p, Pdomain, sizeof(float) * (size_t)LP, cudaMemcpyHostToDevice, st),
            "ct_FBPfan_noalloc: bin upload");
    const int n_all = std::max(LBeta, 2 * LP - 1);
    fbp_tables_kernel<<<(n_all + 255) / 256, 256, 0, st>>>(
        reinterpret_cast<const float *>(dev + o_b), LBeta, reinterpret_cast<const float *>(dev + o_p), LP, g.pint,
        Rscan, reinterpret_cast<float2 *>(dev + o_trig), reinterpret_cast<float *>(dev + o_g),
        reinterpret_cast<double *>(dev + o_w));
    CT_LAUNCH_CHECK("fbp_tables_kernel");

    g.trig_f = reinterpret_cast<const float2 *>(dev + o_trig);
    g.Pf = reinterpret_cast<const float *>(dev + o_p);
    float *filtered = reinterpret_cast<float *>(dev + o_rc);

    RowFilter f{};
    f.nrow = LBeta;
    f.np = LP;
    f.pint = g.pint;
    f.G = reinterpret_cast<const float *>(dev + o_g);
    f.w = reinterpret_cast<const double *>(dev + o_w);
    f.wrows = 1;
    f.launch_order = 1;   // the reference's in-place weight as launched (FBPfan.cu:286-420)
    f.tile = 128;
    f.limit = 1024;
    f.row_block = 128;
    f.rowmod = LBeta;
    if ((s = row_filter_launch(f, d_R, filtered, st))) return s;
    return fan_bp_launch(g, filtered, d_Display, 1, nullptr, 0.f, 0.f, 0.f, 0.f, false, st);
}
