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
// not fit are rejected with CT_ERR_ARG.  The small tables are computed on the
// host into a static host buffer and copied in with cudaMemcpyAsync (a copy,
// not an allocation).
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress, with that device current; make that first call
// before any stream capture.  Every call shares the one array and leaves its
// contents behind (the filter kernel zeroes the rows it accumulates into), so
// calls whose GPU work overlaps -- on different streams, or from different
// host threads -- race on it: serialise them.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "kernels.cuh"

namespace ct {

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;   // 8 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_fbp_scratch[kNoAllocScratchBytes];

// host staging of the small tables (static: no host allocation per call either)
alignas(256) unsigned char g_host_stage[size_t(1) << 20];
std::mutex g_noalloc_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

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
    CT_REQUIRE(Size[0] > 0 && Size[1] > 0, "ct_FBPfan_noalloc: Size must be positive");
    CT_REQUIRE(Rscan > 0.5 * std::sqrt(Size[0] * Size[0] + Size[1] * Size[1]),
               "ct_FBPfan_noalloc: Rscan must exceed the half diagonal of the image");
    // scratch layout: [trig (float2 per view)][P (float)][taps (2LP-1 float)][weights (double)][filtered]
    const size_t o_trig = 0;
    const size_t o_p = align256(o_trig + sizeof(float2) * (size_t)LBeta);
    const size_t o_g = align256(o_p + sizeof(float) * (size_t)LP);
    const size_t o_w = align256(o_g + sizeof(float) * (2 * (size_t)LP - 1));
    const size_t o_rc = align256(o_w + sizeof(double) * (size_t)LP);
    const size_t total = o_rc + sizeof(float) * (size_t)LBeta * LP;
    if (total > kNoAllocScratchBytes || o_rc > sizeof(g_host_stage)) {
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

    // tables on the host: sinf/cosf of the float angles, taps of GFunction
    // (FBPfan.cu:6-19) and the weights Rscan / sqrt(Rscan^2 + P^2) (FBPfan.cu:32)
    unsigned char *h = g_host_stage;
    std::memset(h, 0, o_rc);
    float2 *trig = reinterpret_cast<float2 *>(h + o_trig);
    for (int v = 0; v < LBeta; ++v) trig[v] = make_float2(sinf(BetaScanRange[v]), cosf(BetaScanRange[v]));
    std::memcpy(h + o_p, Pdomain, sizeof(float) * (size_t)LP);
    float *G = reinterpret_cast<float *>(h + o_g);
    const double PI = 3.141592653589793;
    for (int n = 0; n < LP; ++n) {
        const double a = 1.0 * ((double)g.pint * PI) * ((double)g.pint * PI);
        if (n == 0) G[LP - 1] = (float)(1.0 / a);
        else G[LP - 1 - n] = G[LP - 1 + n] = (float)(-1.0 / a / (4 * (1.0 * n * n) - 1));
    }
    double *w = reinterpret_cast<double *>(h + o_w);
    for (int p = 0; p < LP; ++p) w[p] = Rscan / std::sqrt(1.0 * Rscan * Rscan + 1.0 * Pdomain[p] * Pdomain[p]);
    CT_CUDA(cudaMemcpyAsync(dev, h, o_rc, cudaMemcpyHostToDevice, st), "ct_FBPfan_noalloc: table upload");

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
