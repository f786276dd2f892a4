// abi.cu -- the C ABI of libctgb.so (declared in include/ctgb.h).
//
// Plans hold the geometry in HBM (per-view trig tables, detector domains,
// filter taps, pre-weight tables) and lazily grown workspaces.  The drop-in
// host-pointer entry points keep the argument lists of the reference host
// helpers; they stage host data through device buffers that persist between
// calls (the reference allocates, copies and resets the device on every call,
// ProjectionCone_3D.cu:433-520 and ProjectionCone_3D.cpp:53).
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "devbuf.cuh"
#include "kernels.cuh"

namespace ct {



static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_status(cudaError_t e, const char *what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? CT_ERR_OOM : CT_ERR_CUDA;
}

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// Grazing rays for the FP64 re-walk (ref_walk.cu), in one buffer allocated on
// first use: the list of `cap` entries, the count, and, for launches of
// `nrays` rays, the overflow bitmap (one bit per ray; 17.7 MB at 360 x 512 x
// 768).  The buffer is zeroed whenever its layout changes, and the re-walk
// clears every bit it drains, so the bitmap is all zeros between launches.
// With nrays = 0 there is no bitmap and an overflow is only counted.
constexpr int kGrazeCap = 1 << 16;
static int g_graze_cap = kGrazeCap;   // list entries of later allocations (ct_set_graze_list_capacity)

struct GrazeBuf {
    DevBuf buf;
    int cap = 0;
    long long words = -1;
    void release() { buf.release(); cap = 0; words = -1; }
};

static int graze_list(GrazeBuf &b, GrazeList &gl, long long nrays, cudaStream_t st, int cap = 0) {
    if (cap <= 0) cap = g_graze_cap;
    const long long words = (nrays + 31) / 32;
    const size_t need = sizeof(unsigned long long) * ((size_t)cap + 2) + sizeof(unsigned int) * (size_t)words;
    if (need > b.buf.bytes || cap != b.cap || words != b.words) {
        int s = b.buf.ensure(need);
        if (s) return s;
        CT_CUDA(cudaMemsetAsync(b.buf.ptr, 0, need, st), "graze list clear");
        b.cap = cap;
        b.words = words;
    }
    gl.rays = b.buf.as<unsigned long long>();
    gl.count = gl.rays + cap;
    gl.cap = cap;
    gl.bits = nrays > 0 ? reinterpret_cast<unsigned int *>(gl.rays + cap + 2) : nullptr;
    gl.nbits = nrays;
    return CT_OK;
}

// Number of grazing rays of the buffer's last projection (a diagnostic; syncs the stream).
static int graze_count(const GrazeBuf &b, long long *n, cudaStream_t st) {
    CT_REQUIRE(n, "null count pointer");
    *n = 0;
    if (!b.buf.ptr) return CT_OK;
    unsigned long long h = 0;
    CT_CUDA(cudaMemcpyAsync(&h, b.buf.as<unsigned long long>() + b.cap, sizeof(h), cudaMemcpyDeviceToHost, st),
            "graze count");
    CT_CUDA(cudaStreamSynchronize(st), "graze count sync");
    *n = (long long)h;
    return CT_OK;
}

constexpr double kPi = 3.141592653589793;

// Ramp filter taps (2*np-1, centre np-1), computed in double, stored as float.
//  CT_FILTER_SHEPP_LOGAN: exactly as GFunction computes them (FDK.cu:6-19).
//  CT_FILTER_RAM_LAK: the kernel of FBP_parallel.m:241-251 (h[0] = 1/(2 dP)^2,
//    0 at even n, -1/(n pi dP)^2 at odd n) times 1/2, the amplitude convention
//    of the Shepp-Logan taps (whose centre is half the textbook 2/(pi dP)^2),
//    so that switching the filter keeps the image scale.
static std::vector<float> ramp_taps(int kind, float pint, int np) {
    std::vector<float> g(2 * (size_t)np - 1);
    for (int n = 0; n < np; ++n) {
        double v;
        if (kind == CT_FILTER_RAM_LAK) {
            if (n == 0) {
                v = 0.5 / ((2.0 * pint) * (2.0 * pint));
            } else if (n % 2 == 0) {
                v = 0.0;
            } else {
                const double a = (double)n * kPi * pint;
                v = -0.5 / (a * a);
            }
        } else if (n == 0) {
            v = 1.0 / (1.0 * (kPi * pint) * (kPi * pint));
        } else {
            const double a = 1.0 * ((double)pint * kPi) * ((double)pint * kPi);
            v = -1.0 / a / (4 * (1.0 * n * n) - 1);
        }
        g[np - 1 - n] = g[np - 1 + n] = (float)v;
    }
    return g;
}

// Symmetric Hamming window of m taps, 0.54 - 0.46 cos(2 pi k / (m - 1)), the
// smoothing window of the commented post-filter in FanProjection.m:265-270.
static std::vector<double> hamming(int m) {
    std::vector<double> h(m, 1.0);
    if (m > 1)
        for (int k = 0; k < m; ++k) h[k] = 0.54 - 0.46 * std::cos(2.0 * kPi * k / (m - 1));
    return h;
}

// Short-scan weight of ParkFunction.m:6-16 for the ray at fan angle gama of the
// view at beta (radians); b0 is the first view angle, fan the full fan angle.
// The two ramps use beta itself, not beta - b0, as ParkFunction.m:9,13 do.
static double parker(double beta, double b0, double gama, double fan) {
    if (beta >= b0 && beta < b0 + fan - 2 * gama) {
        const double s = std::sin(kPi / 4 * beta / (fan / 2 - gama));
        return s * s;
    }
    if (beta >= b0 + fan - 2 * gama && beta <= b0 + kPi - 2 * gama) return 1.0;
    if (beta > b0 + kPi - 2 * gama && beta <= b0 + kPi + fan) {
        const double s = std::sin(kPi / 4 * (kPi + fan - beta) / (fan / 2 + gama));
        return s * s;
    }
    return 0.0;
}

// Short-scan weights per (view, bin), gama = atan(P / D) on the flat detector
// at the isocentre.  Each weight is doubled: a short scan covers each line
// once, and the half-amplitude ramp taps assume the double coverage of a full
// turn (FanProjection.m:280-288 doubles its taps for the same reason).
static std::vector<float> parker_table(const std::vector<float> &beta, const std::vector<float> &P, double D) {
    const int nb = (int)beta.size(), np = (int)P.size();
    const double fan = std::fabs(std::atan((double)P[np - 1] / D) - std::atan((double)P[0] / D));
    std::vector<float> w((size_t)nb * np);
    for (int v = 0; v < nb; ++v)
        for (int p = 0; p < np; ++p)
            w[(size_t)v * np + p] = (float)(2.0 * parker(beta[v], beta[0], std::atan((double)P[p] / D), fan));
    return w;
}

// Filter-stage options of a plan (ct_*_plan_set_filter / _set_short_scan).
struct FilterOpts {
    int kind = CT_FILTER_SHEPP_LOGAN;
    int wlen = 0;
    int short_scan = 0;
};

// Device tables of the filter options: the taps always, the short-scan
// weights and the smoothing window when they are switched on.
static int filter_tables(const FilterOpts &o, float pint, int np, const std::vector<float> &beta,
                         const std::vector<float> &P, double D, DevBuf &G, DevBuf &pwt, DevBuf &win,
                         double &wsum) {
    int s;
    std::vector<float> taps = ramp_taps(o.kind, pint, np);
    if ((s = upload(G, taps.data(), taps.size()))) return s;
    if (o.short_scan) {
        std::vector<float> w = parker_table(beta, P, D);
        if ((s = upload(pwt, w.data(), w.size()))) return s;
    }
    if (o.wlen > 0) {
        std::vector<double> h = hamming(o.wlen);
        wsum = 0.0;
        for (double x : h) wsum += x;
        if ((s = upload(win, h.data(), h.size()))) return s;
    }
    return CT_OK;
}

static void filter_fields(const FilterOpts &o, int rows_per_view, const DevBuf &pwt, const DevBuf &win, double wsum,
                          RowFilter &f) {
    f.pw = o.short_scan ? pwt.as<float>() : nullptr;
    f.pw_div = rows_per_view;
    f.win = o.wlen > 0 ? win.as<double>() : nullptr;
    f.wlen = o.wlen;
    f.wsum = wsum;
}

static int check_filter_opts(int kind, int window_len) {
    CT_REQUIRE(kind == CT_FILTER_SHEPP_LOGAN || kind == CT_FILTER_RAM_LAK, "filter kind must be CT_FILTER_*");
    CT_REQUIRE(window_len >= 0 && window_len <= 1024, "window length must be in [0, 1024]");
    return CT_OK;
}

}  // namespace ct

using namespace ct;

// ---------------------------------------------------------------------------
// cone plan
// ---------------------------------------------------------------------------
struct ct_cone_plan {
    ConeGeom g{};
    DevBuf trig, vsrc, P, xi, xtab, vorder, trigf, vsrcf, Pd, xid;
    DevBuf quads, rcov, G, wtab, norms, volT, volS, cols, pwt, win, scan, bpsum;
    double cols_res[3] = {0, 0, 0};   // voxel pitch the column table was built for
    GrazeBuf graze;
    int bp_chunk = 0;   // views per backprojection chunk; 0: automatic (cone_bp_chunk_views)
    int fdk_filter = CT_FDK_FILTER_LAUNCH_ORDER;
    int fdk_bp = CT_FDK_BP_STICKY;
    FilterOpts filt;
    double wsum = 0.0;
    // host copies of the geometry (drop-in cache key)
    std::vector<float> hb, hp, hx;
    double hsize[3] = {0, 0, 0};
    ~ct_cone_plan() {
        trig.release(); vsrc.release(); P.release(); xi.release(); xtab.release(); vorder.release();
        trigf.release(); vsrcf.release(); Pd.release(); xid.release();
        quads.release(); rcov.release(); G.release(); wtab.release(); norms.release(); graze.release();
        volT.release(); volS.release(); cols.release(); pwt.release(); win.release(); scan.release(); bpsum.release();
    }
};

// The forward projector's column table for the current voxel pitch: built at
// plan creation and again after a caller changes the pitch, synchronously, so
// that no later launch on any stream (or graph capture) can precede it.
static int cone_fp_refresh(ct_cone_plan *plan) {
    const ConeGeom &g = plan->g;
    if (plan->cols.ptr && std::equal(g.res, g.res + 3, plan->cols_res)) return CT_OK;
    int s = plan->cols.ensure(sizeof(FpColumn) * (size_t)g.nb * g.np);
    if (s || (s = cone_fp_columns(g, plan->cols.as<FpColumn>(), nullptr))) return s;
    CT_CUDA(cudaStreamSynchronize(nullptr), "column table");
    std::copy(g.res, g.res + 3, plan->cols_res);
    return CT_OK;
}

// CSR export shared by the cone and fan plans: count pass, grazing-list check,
// scan, and the fill pass when arrays are given.
template <class Launch>
static int sysmat_common(Launch launch, GrazeBuf &graze, DevBuf &scan, long long nrows, long long *d_row_ptr,
                         int *d_col, float *d_val, long long cap, long long *nnz, cudaStream_t st) {
    CT_REQUIRE(d_row_ptr && nnz, "sysmat: null row pointer or nnz");
    CT_REQUIRE(nrows > 0 && nrows < (1LL << 31), "sysmat: row count out of range");
    CT_REQUIRE((d_col == nullptr) == (d_val == nullptr), "sysmat: give both d_col and d_val, or neither");
    GrazeList gl;
    int s;
    // count pass; when the grazing rays overflow the list, grow it to hold
    // them all and count again (the walk visits the same rays every time).
    // The next projection sees the changed layout and clears the buffer.
    int gcap = g_graze_cap;
    for (;;) {
        if ((s = graze_list(graze, gl, 0, st, gcap))) return s;
        if ((s = launch(gl, false))) return s;
        unsigned long long ng = 0;
        CT_CUDA(cudaMemcpyAsync(&ng, gl.count, sizeof(ng), cudaMemcpyDeviceToHost, st), "graze count");
        CT_CUDA(cudaStreamSynchronize(st), "sysmat sync");
        if (ng <= (unsigned long long)gcap) break;
        CT_REQUIRE(ng < (1ULL << 31), "sysmat: more than 2^31 grazing rays");
        gcap = (int)ng;
    }
    if ((s = csr_scan(d_row_ptr, (int)nrows, &scan.ptr, &scan.bytes, st))) return s;
    long long total = 0;
    CT_CUDA(cudaMemcpyAsync(&total, d_row_ptr + nrows, sizeof(long long), cudaMemcpyDeviceToHost, st), "nnz");
    CT_CUDA(cudaStreamSynchronize(st), "sysmat sync");
    *nnz = total;
    if (!d_col) return CT_OK;
    CT_REQUIRE(cap >= total, "sysmat: d_col / d_val hold fewer entries than the matrix has");
    return launch(gl, true);
}

static int check_domain(const float *a, int n, const char *what) {
    if (!a) { set_error(std::string(what) + ": null"); return CT_ERR_ARG; }
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) { set_error(std::string(what) + ": non-finite value"); return CT_ERR_ARG; }
    return CT_OK;
}

extern "C" {

const char *ct_last_error(void) { return g_last_error.c_str(); }
const char *ct_version(void) { return "ctgb 0.1 (sm_103a)"; }

int ct_cone_plan_create(ct_cone_plan **out, int nt, int ns, int nz, const double *Size, const float *beta,
                        int nb, const float *P, int np, const float *xi, int nx, double D) {
    CT_REQUIRE(out, "plan pointer is null");
    *out = nullptr;
    CT_REQUIRE(nt > 0 && ns > 0 && nz > 0, "volume sizes must be positive");
    CT_REQUIRE((long long)nt * ns * nz < (1LL << 31), "volume larger than 2^31 voxels");
    CT_REQUIRE(nb > 0 && nb <= 65535, "number of views must be in [1, 65535]");
    CT_REQUIRE(np > 0 && nx > 0, "detector sizes must be positive");
    CT_REQUIRE((long long)nb * np * nx < (1LL << 40), "sinogram too large");
    CT_REQUIRE(Size && Size[0] > 0 && Size[1] > 0 && Size[2] > 0, "Size must be positive");
    CT_REQUIRE(D > 0.5 * std::sqrt(Size[0] * Size[0] + Size[1] * Size[1]),
               "Distance must exceed the in-plane half diagonal of the volume");
    int s;
    if ((s = check_domain(beta, nb, "BetaScanRange")) || (s = check_domain(P, np, "Pdomain")) ||
        (s = check_domain(xi, nx, "Xigamadomain")))
        return s;
    ct_cone_plan *pl = new ct_cone_plan();
    ConeGeom &g = pl->g;
    g.nt = nt; g.ns = ns; g.nz = nz;
    g.nb = nb; g.np = np; g.nx = nx;
    for (int a = 0; a < 3; ++a) g.size[a] = Size[a];
    g.res[0] = 1.0 * Size[0] / nt;
    g.res[1] = 1.0 * Size[1] / ns;
    g.res[2] = 1.0 * Size[2] / nz;
    for (int a = 0; a < 3; ++a) g.ires[a] = 1.0 / g.res[a];
    cone_geom_derive(g);
    g.D = D;
    // float-range bookkeeping of BackPro / FDKpro (Backprojection3D.cu:304-311)
    g.pint = np > 1 ? std::fabs(P[1] - P[0]) : 1.0f;
    g.xint = nx > 1 ? std::fabs(xi[1] - xi[0]) : 1.0f;
    g.bint = nb > 1 ? std::fabs(beta[1] - beta[0]) : 0.0f;
    g.maxp = std::max(P[0], P[np - 1]);
    g.minp = std::min(P[0], P[np - 1]);
    g.maxx = std::max(xi[0], xi[nx - 1]);
    g.minx = std::min(xi[0], xi[nx - 1]);
    g.p0 = P[0];
    g.x0 = xi[0];
    g.psgn = (np > 1 && P[np - 1] < P[0]) ? -1.0f : 1.0f;
    g.xsgn = (nx > 1 && xi[nx - 1] < xi[0]) ? -1.0f : 1.0f;
    // the reference evaluates sin/cos of the float angle with the
    // single-precision overloads (ProjectionCone_3D.cu:26-28)
    std::vector<double2> tr(nb);
    std::vector<ViewSrc> vs(nb);
    std::vector<float2> trf(nb);
    std::vector<float4> vsf(nb);
    for (int v = 0; v < nb; ++v) {
        const float sf = sinf(beta[v]), cf = cosf(beta[v]);
        const double sb = (double)sf, cb = (double)cf;
        tr[v] = make_double2(sb, cb);
        trf[v] = make_float2(sf, cf);
        vs[v] = ViewSrc{Size[0] / 2 - D * sb, Size[1] / 2 + D * cb, D * sb, D * cb};
        vsf[v] = make_float4((float)vs[v].src_t, (float)vs[v].src_s, (float)vs[v].dsb, (float)vs[v].dcb);
    }
    const std::vector<double> Pdv(P, P + np), xidv(xi, xi + nx);
    // row table of the backprojectors: (x - q(xi[x]), q(xi[x+1]) - x) with the
    // reference's row quotient q(v) = |v - xi[0]| / XigamaInt in double
    std::vector<float2> xt(std::max(nx - 1, 1));
    for (int x = 0; x + 1 < nx; ++x) {
        const double q0 = std::fabs((double)xi[x] - (double)xi[0]) / (double)g.xint;
        const double q1 = std::fabs((double)xi[x + 1] - (double)xi[0]) / (double)g.xint;
        xt[x] = make_float2((float)(x - q0), (float)(q1 - x));
    }
    // forward-projector view order: the views that read the [z][s][t] volume
    // (detector columns closer to t: |cos b| >= |sin b|, as cone_fp_kernel
    // picks) first, then those that read the [z][t][s] copy
    std::vector<int> vo;
    for (int c0 = 0; c0 < nb; c0 += kFpViewChunk)
        for (int pass = 0; pass < 2; ++pass)
            for (int v = c0; v < std::min(nb, c0 + kFpViewChunk); ++v)
                if ((std::fabs(tr[v].y) >= std::fabs(tr[v].x)) == (pass == 0)) vo.push_back(v);
    if ((s = upload(pl->trig, tr.data(), nb)) || (s = upload(pl->vsrc, vs.data(), nb)) || (s = upload(pl->P, P, np)) ||
        (s = upload(pl->xi, xi, nx)) || (s = upload(pl->xtab, xt.data(), xt.size())) ||
        (s = upload(pl->vorder, vo.data(), vo.size())) || (s = upload(pl->trigf, trf.data(), nb)) ||
        (s = upload(pl->vsrcf, vsf.data(), nb)) || (s = upload(pl->Pd, Pdv.data(), np)) ||
        (s = upload(pl->xid, xidv.data(), nx))) {
        delete pl;
        return s;
    }
    g.xtab = pl->xtab.as<float2>();
    g.vorder = pl->vorder.as<int>();
    g.trig = pl->trig.as<double2>();
    g.vsrc = pl->vsrc.as<ViewSrc>();
    g.trigf = pl->trigf.as<float2>();
    g.vsrcf = pl->vsrcf.as<float4>();
    g.Pd = pl->Pd.as<double>();
    g.xid = pl->xid.as<double>();
    g.P = pl->P.as<float>();
    g.xi = pl->xi.as<float>();
    pl->hb.assign(beta, beta + nb);
    pl->hp.assign(P, P + np);
    pl->hx.assign(xi, xi + nx);
    for (int a = 0; a < 3; ++a) pl->hsize[a] = Size[a];
    if ((s = cone_fp_refresh(pl))) {
        delete pl;
        return s;
    }
    *out = pl;
    return CT_OK;
}

int ct_cone_plan_destroy(ct_cone_plan *plan) {
    delete plan;
    return CT_OK;
}

int ct_cone_plan_set_fdk_mode(ct_cone_plan *plan, int filter_mode, int bp_mode) {
    CT_REQUIRE(plan, "plan is null");
    CT_REQUIRE(filter_mode == 0 || filter_mode == 1, "filter_mode must be 0 or 1");
    CT_REQUIRE(bp_mode == 0 || bp_mode == 1, "bp_mode must be 0 or 1");
    plan->fdk_filter = filter_mode;
    plan->fdk_bp = bp_mode;
    return CT_OK;
}

int ct_cone_plan_set_filter(ct_cone_plan *plan, int kind, int window_len) {
    CT_REQUIRE(plan, "plan is null");
    int s = check_filter_opts(kind, window_len);
    if (s) return s;
    plan->filt.kind = kind;
    plan->filt.wlen = window_len;
    plan->G.release();   // tables are rebuilt on the next filter call
    return CT_OK;
}

int ct_cone_plan_set_short_scan(ct_cone_plan *plan, int enable) {
    CT_REQUIRE(plan, "plan is null");
    CT_REQUIRE(enable == 0 || enable == 1, "enable must be 0 or 1");
    plan->filt.short_scan = enable;
    plan->G.release();
    return CT_OK;
}

size_t ct_cone_plan_workspace_bytes(const ct_cone_plan *plan) {
    if (!plan) return 0;
    return plan->quads.bytes + plan->rcov.bytes + plan->G.bytes + plan->wtab.bytes + plan->norms.bytes +
           plan->graze.buf.bytes + plan->volT.bytes + plan->volS.bytes + plan->cols.bytes + plan->bpsum.bytes;
}

// Views per backprojection chunk: the caller's setting, else chunks of about
// kBpChunkBytes of packed quads, evened out over the scan.  Shorter launches
// keep the views the resident blocks are working on close together, so their
// quads stay in L2: at 512^3 / 360 views / 768x512 the backprojection took
// 71.8 ms in one pass, 64.4 / 62.8 / 62.2 / 63.5 ms in chunks of
// 60 / 90 / 120 / 180 views.
constexpr size_t kBpChunkBytes = size_t(768) << 20;
static int cone_bp_chunk_views(const ct_cone_plan *plan) {
    const ConeGeom &g = plan->g;
    if (plan->bp_chunk > 0) return std::min(plan->bp_chunk, g.nb);
    const size_t per_view = cone_quads_bytes(g, 1);
    const int target = (int)std::max<size_t>(1, std::min<size_t>(g.nb, kBpChunkBytes / std::max<size_t>(per_view, 1)));
    const int nch = (g.nb + target - 1) / target;
    return (g.nb + nch - 1) / nch;
}

int ct_cone_plan_get_bp_chunk(const ct_cone_plan *plan, int *views) {
    CT_REQUIRE(plan && views, "ct_cone_plan_get_bp_chunk: null argument");
    *views = cone_bp_chunk_views(plan);
    return CT_OK;
}

int ct_cone_plan_set_bp_chunk(ct_cone_plan *plan, int views) {
    CT_REQUIRE(plan, "plan is null");
    CT_REQUIRE(views >= 0, "views per backprojection chunk must be >= 0");
    plan->bp_chunk = views;
    return CT_OK;
}

static long long cone_rays(const ConeGeom &g) { return (long long)g.nb * g.nx * g.np; }

// The two zero-padded copies of the volume the forward projector reads
// (plan workspace, refreshed every call): [z][s][t] and [z][t][s] (for views
// whose detector rows run along s), each with kFpPadSlices empty slices
// before and after so that the walk needs no index clamp.
static int fp_volumes(ct_cone_plan *plan, const float *d_vol, const float **volS, const float **volT,
                      cudaStream_t st) {
    const size_t slice = (size_t)plan->g.nt * plan->g.ns;
    const size_t n = slice * plan->g.nz, pad = kFpPadSlices * slice;
    CT_REQUIRE(n < (1ULL << 31), "cone forward projection: at most 2^31 - 1 voxels");
    const size_t bytes = (n + 2 * pad) * sizeof(float);
    int s;
    if ((s = plan->volT.ensure(bytes)) || (s = plan->volS.ensure(bytes))) return s;
    float *t = plan->volT.as<float>(), *v = plan->volS.as<float>();
    for (float *b : {t, v}) {
        CT_CUDA(cudaMemsetAsync(b, 0, pad * sizeof(float), st), "pad");
        CT_CUDA(cudaMemsetAsync(b + pad + n, 0, pad * sizeof(float), st), "pad");
    }
    CT_CUDA(cudaMemcpyAsync(v + pad, d_vol, n * sizeof(float), cudaMemcpyDeviceToDevice, st), "volume copy");
    *volS = v + pad;
    *volT = t + pad;
    return cone_transpose_ts(plan->g, d_vol, t + pad, st);
}

int ct_cone_fp(ct_cone_plan *plan, const float *d_vol, float *d_proj, void *stream) {
    CT_REQUIRE(plan && d_vol && d_proj, "ct_cone_fp: null argument");
    GrazeList gl;
    const float *volS, *volT;
    int s;
    if ((s = graze_list(plan->graze, gl, cone_rays(plan->g), as_stream(stream))) ||
        (s = fp_volumes(plan, d_vol, &volS, &volT, as_stream(stream))))
        return s;
    return cone_fp_launch(plan->g, plan->cols.as<FpColumn>(), volS, volT, d_vol, d_proj, nullptr, nullptr, 0.0f,
                          nullptr, 0, gl, as_stream(stream));
}

int ct_cone_fp_residual(ct_cone_plan *plan, const float *d_vol, const float *d_b, const float *d_rowsum,
                        float eps, float *d_out, double *d_norms, void *stream) {
    CT_REQUIRE(plan && d_vol && d_b && d_out && d_norms, "ct_cone_fp_residual: null argument");
    GrazeList gl;
    const float *volS, *volT;
    int s;
    if ((s = graze_list(plan->graze, gl, cone_rays(plan->g), as_stream(stream))) ||
        (s = fp_volumes(plan, d_vol, &volS, &volT, as_stream(stream))))
        return s;
    return cone_fp_launch(plan->g, plan->cols.as<FpColumn>(), volS, volT, d_vol, d_out, d_b, d_rowsum, eps, d_norms,
                          1, gl, as_stream(stream));
}

// Backprojection in chunks of cone_bp_chunk_views views:
// every chunk is packed into quads and backprojected, its sums added to the
// volume (or, for the fused SIRT update, to a partial-sum volume that the last
// chunk folds into the update).
static int cone_bp_common(ct_cone_plan *plan, const float *d_proj, float *d_vol, int weighting,
                          const float *colsum, float eps, float lambda, float lo, float hi, bool update,
                          cudaStream_t st) {
    const ConeGeom &g = plan->g;
    const int chunk = cone_bp_chunk_views(plan);
    const int nchunks = (g.nb + chunk - 1) / chunk;
    int s = plan->quads.ensure(cone_quads_bytes(g, chunk));
    if (s) return s;
    float *part = nullptr;
    if (update && nchunks > 1) {
        if ((s = plan->bpsum.ensure(sizeof(float) * (size_t)g.nt * g.ns * g.nz))) return s;
        part = plan->bpsum.as<float>();
    }
    for (int c = 0; c < nchunks; ++c) {
        const int v0 = c * chunk, nv = std::min(chunk, g.nb - v0);
        const bool last = c == nchunks - 1;
        if ((s = cone_pack_quads(g, d_proj, plan->quads.as<float4>(), v0, nv, st))) return s;
        const float *prev = c == 0 ? nullptr : (update ? part : d_vol);
        float *out = (update && !last) ? part : d_vol;
        if ((s = cone_bp_launch(g, plan->quads.as<float4>(), v0, nv, prev, out, weighting, colsum, eps, lambda, lo,
                                hi, update && last, st)))
            return s;
    }
    return CT_OK;
}

int ct_cone_bp(ct_cone_plan *plan, const float *d_proj, float *d_vol, void *stream) {
    CT_REQUIRE(plan && d_proj && d_vol, "ct_cone_bp: null argument");
    CT_REQUIRE(plan->g.np >= 2 && plan->g.nx >= 2, "ct_cone_bp: detector needs at least 2x2 samples");
    return cone_bp_common(plan, d_proj, d_vol, 0, nullptr, 0.f, 0.f, 0.f, 0.f, false, as_stream(stream));
}

int ct_cone_bp_update(ct_cone_plan *plan, const float *d_proj, const float *d_colsum, float eps, float lambda,
                      float lo, float hi, float *d_vol, void *stream) {
    CT_REQUIRE(plan && d_proj && d_colsum && d_vol, "ct_cone_bp_update: null argument");
    CT_REQUIRE(plan->g.np >= 2 && plan->g.nx >= 2, "ct_cone_bp_update: detector needs at least 2x2 samples");
    return cone_bp_common(plan, d_proj, d_vol, 0, d_colsum, eps, lambda, lo, hi, true, as_stream(stream));
}

static int cone_fdk_filter_into(ct_cone_plan *plan, const float *d_proj, float *d_out, cudaStream_t st) {
    ConeGeom &g = plan->g;
    CT_REQUIRE(g.np >= 2 && g.nx >= 2, "FDK: detector needs at least 2x2 samples");
    int s;
    if (!plan->G.ptr) {
        if ((s = filter_tables(plan->filt, g.pint, g.np, plan->hb, plan->hp, g.D, plan->G, plan->pwt, plan->win,
                               plan->wsum)))
            return s;
        // pre-weight D / sqrt(D^2 + P^2 + xi^2) per (xi, P), in double (FDK.cu:34)
        std::vector<double> w((size_t)g.nx * g.np);
        for (int x = 0; x < g.nx; ++x)
            for (int p = 0; p < g.np; ++p) {
                const double Pv = plan->hp[p], Xv = plan->hx[x];
                w[(size_t)x * g.np + p] = g.D / std::sqrt(1.0 * g.D * g.D + 1.0 * Pv * Pv + 1.0 * Xv * Xv);
            }
        if ((s = upload(plan->wtab, w.data(), w.size()))) return s;
    }
    RowFilter f{};
    f.nrow = g.nb * g.nx;
    f.np = g.np;
    f.pint = g.pint;
    f.G = plan->G.as<float>();
    f.w = plan->wtab.as<double>();
    f.wrows = g.nx;
    f.launch_order = plan->fdk_filter;
    f.tile = 256;        // FDK.h:22 threadX
    f.limit = 2048;      // FDK.h:24 Filterlengthlimit
    f.row_block = 256;   // FDK.h:23 blockX
    f.rowmod = g.nx;
    filter_fields(plan->filt, g.nx, plan->pwt, plan->win, plan->wsum, f);
    return row_filter_launch(f, d_proj, d_out, st);
}

int ct_cone_fdk_filter(ct_cone_plan *plan, const float *d_proj, float *d_filtered, void *stream) {
    CT_REQUIRE(plan && d_proj && d_filtered, "ct_cone_fdk_filter: null argument");
    return cone_fdk_filter_into(plan, d_proj, d_filtered, as_stream(stream));
}

int ct_cone_fdk_bp(ct_cone_plan *plan, const float *d_filtered, float *d_vol, void *stream) {
    CT_REQUIRE(plan && d_filtered && d_vol, "ct_cone_fdk_bp: null argument");
    CT_REQUIRE(plan->g.np >= 2 && plan->g.nx >= 2, "ct_cone_fdk_bp: detector needs at least 2x2 samples");
    return cone_bp_common(plan, d_filtered, d_vol, plan->fdk_bp == CT_FDK_BP_STICKY ? 2 : 1, nullptr, 0.f, 0.f,
                          0.f, 0.f, false, as_stream(stream));
}

int ct_cone_fdk(ct_cone_plan *plan, const float *d_proj, float *d_vol, void *stream) {
    CT_REQUIRE(plan && d_proj && d_vol, "ct_cone_fdk: null argument");
    ConeGeom &g = plan->g;
    cudaStream_t st = as_stream(stream);
    int s;
    if ((s = plan->rcov.ensure(sizeof(float) * (size_t)g.nb * g.nx * g.np))) return s;
    if ((s = cone_fdk_filter_into(plan, d_proj, plan->rcov.as<float>(), st))) return s;
    return ct_cone_fdk_bp(plan, plan->rcov.as<float>(), d_vol, stream);
}

int ct_cone_sysmat(ct_cone_plan *plan, int view0, int nviews, long long *d_row_ptr, int *d_col, float *d_val,
                   long long cap, long long *nnz, void *stream) {
    CT_REQUIRE(plan, "ct_cone_sysmat: null plan");
    const ConeGeom &g = plan->g;
    CT_REQUIRE(view0 >= 0 && nviews > 0 && view0 + nviews <= g.nb, "ct_cone_sysmat: view range out of bounds");
    cudaStream_t st = as_stream(stream);
    auto launch = [&](const GrazeList &gl, bool fill) {
        return cone_sysmat_launch(g, view0, nviews, d_row_ptr, d_col, d_val, fill, gl, st);
    };
    return sysmat_common(launch, plan->graze, plan->scan, (long long)nviews * g.nx * g.np, d_row_ptr, d_col, d_val,
                         cap, nnz, st);
}

int ct_cone_plan_grazing_rays(const ct_cone_plan *plan, long long *n, void *stream) {
    CT_REQUIRE(plan, "ct_cone_plan_grazing_rays: null plan");
    return graze_count(plan->graze, n, as_stream(stream));
}

int ct_set_graze_list_capacity(int cap) {
    CT_REQUIRE(cap >= 1 && cap <= (1 << 26), "ct_set_graze_list_capacity: capacity must be in [1, 2^26]");
    g_graze_cap = cap;
    return CT_OK;
}

int ct_cone_count_segments(ct_cone_plan *plan, long long *segments, void *stream) {
    CT_REQUIRE(plan && segments, "ct_cone_count_segments: null argument");
    cudaStream_t st = as_stream(stream);
    int s = plan->norms.ensure(2 * sizeof(double));
    if (s) return s;
    CT_CUDA(cudaMemsetAsync(plan->norms.ptr, 0, 2 * sizeof(double), st), "memset");
    if ((s = cone_count_launch(plan->g, plan->norms.as<double>(), st))) return s;
    double h = 0;
    CT_CUDA(cudaMemcpyAsync(&h, plan->norms.ptr, sizeof(double), cudaMemcpyDeviceToHost, st), "copy");
    CT_CUDA(cudaStreamSynchronize(st), "sync");
    *segments = (long long)llround(h);
    return CT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// fan plan (2D fan and parallel beam)
// ---------------------------------------------------------------------------
struct ct_fan_plan {
    FanGeom g{};
    DevBuf trig_d, Pd, trig_f, Pf, G, wtab, rcov, pwt, win, scan, rays;
    GrazeBuf graze;
    std::vector<float> hPf, hbf;
    FilterOpts filt;
    double wsum = 0.0;
    ~ct_fan_plan() {
        rays.release();
        trig_d.release(); Pd.release(); trig_f.release(); Pf.release();
        G.release(); wtab.release(); rcov.release(); graze.release(); pwt.release(); win.release(); scan.release();
    }
};

// size2 = extents (fastest axis first), ang/P double; angles and bins are
// rounded to float for the backprojectors as the MATLAB callers do (single()).
static int fan_plan_make(ct_fan_plan **out, int nt, int ns, const double size2[2], const double *ang, int nb,
                         const double *P, int np, double D, int parallel) {
    CT_REQUIRE(out, "plan pointer is null");
    *out = nullptr;
    CT_REQUIRE(nt > 0 && ns > 0, "image sizes must be positive");
    CT_REQUIRE((long long)nt * ns < (1LL << 31), "image too large");
    CT_REQUIRE(nb > 0 && np > 0, "sinogram sizes must be positive");
    CT_REQUIRE(size2[0] > 0 && size2[1] > 0, "Size must be positive");
    CT_REQUIRE(ang && P, "null domain");
    if (!parallel)
        CT_REQUIRE(D > 0.5 * std::sqrt(size2[0] * size2[0] + size2[1] * size2[1]),
                   "Distance must exceed the half diagonal of the image");
    for (int i = 0; i < nb; ++i) CT_REQUIRE(std::isfinite(ang[i]), "non-finite angle");
    for (int i = 0; i < np; ++i) CT_REQUIRE(std::isfinite(P[i]), "non-finite detector coordinate");
    ct_fan_plan *pl = new ct_fan_plan();
    FanGeom &g = pl->g;
    g.nt = nt; g.ns = ns; g.nb = nb; g.np = np;
    g.size[0] = size2[0]; g.size[1] = size2[1];
    g.res[0] = 1.0 * size2[0] / nt;
    g.res[1] = 1.0 * size2[1] / ns;
    g.D = D;
    g.parallel = parallel;
    g.smax = std::max(std::fabs(P[0]), std::fabs(P[np - 1]));
    std::vector<double2> td(nb);
    std::vector<float2> tf(nb);
    std::vector<float> pf(np), bf(nb);
    for (int v = 0; v < nb; ++v) {
        td[v] = make_double2(std::sin(ang[v]), std::cos(ang[v]));
        bf[v] = (float)ang[v];
        tf[v] = make_float2(sinf(bf[v]), cosf(bf[v]));
    }
    for (int p = 0; p < np; ++p) pf[p] = (float)P[p];
    g.pint = np > 1 ? std::fabs(pf[1] - pf[0]) : 1.0f;
    g.bint = nb > 1 ? std::fabs(bf[1] - bf[0]) : 0.0f;
    g.maxp = std::max(pf[0], pf[np - 1]);
    g.minp = std::min(pf[0], pf[np - 1]);
    g.p0 = pf[0];
    g.psgn = (np > 1 && pf[np - 1] < pf[0]) ? -1.0f : 1.0f;
    int s;
    if ((s = upload(pl->trig_d, td.data(), nb)) || (s = upload(pl->Pd, P, np)) ||
        (s = upload(pl->trig_f, tf.data(), nb)) || (s = upload(pl->Pf, pf.data(), np))) {
        delete pl;
        return s;
    }
    g.trig_d = pl->trig_d.as<double2>();
    g.Pd = pl->Pd.as<double>();
    g.trig_f = pl->trig_f.as<float2>();
    g.Pf = pl->Pf.as<float>();
    pl->hPf = pf;
    pl->hbf = bf;
    *out = pl;
    return CT_OK;
}

// The forward walk's set-up table of a plan (48 bytes per ray), built once the
// geometry is final, synchronously (no later launch or graph capture can
// precede it).  The one-call drop-ins skip it and set rays up per call, as
// does a sinogram whose table would pass kFanRayTableMax.
constexpr size_t kFanRayTableMax = size_t(4) << 30;
static int fan_ray_table(ct_fan_plan *pl) {
    const FanGeom &g = pl->g;
    const size_t bytes = sizeof(FanRay) * (size_t)g.nb * g.np;
    if (bytes > kFanRayTableMax) return CT_OK;
    int s = pl->rays.ensure(bytes);
    if (s || (s = fan_ray_table_launch(g, pl->rays.as<FanRay>(), nullptr))) return s;
    CT_CUDA(cudaStreamSynchronize(nullptr), "ray set-up table");
    pl->g.ray_tab = pl->rays.as<FanRay>();
    return CT_OK;
}

extern "C" {

int ct_fan_plan_create(ct_fan_plan **plan, int nt, int ns, const double *Size, const double *beta, int nb,
                       const double *P, int np, double D) {
    CT_REQUIRE(Size, "Size is null");
    int s = fan_plan_make(plan, nt, ns, Size, beta, nb, P, np, D, 0);
    if (!s && (s = fan_ray_table(*plan))) {
        delete *plan;
        *plan = nullptr;
    }
    return s;
}

int ct_fan_plan_destroy(ct_fan_plan *plan) {
    delete plan;
    return CT_OK;
}

int ct_par_plan_create(ct_fan_plan **plan, int height, int width, const double *resolution, const double *thetaRange,
                       int Ltheta, const double *t_Range, int Lt) {
    CT_REQUIRE(resolution && resolution[0] > 0 && resolution[1] > 0, "resolution must be positive");
    // x runs along width (resolution[1]), y along height (resolution[0]); pixel y*width + x,
    // as ProjectionParallel_2D takes them (ProjectionParallel_2D.cpp:10-20)
    const double size2[2] = {resolution[1] * width, resolution[0] * height};
    int s = fan_plan_make(plan, width, height, size2, thetaRange, Ltheta, t_Range, Lt, 0.0, 1);
    if (s) return s;
    (*plan)->g.res[0] = resolution[1];
    (*plan)->g.res[1] = resolution[0];
    if ((s = fan_ray_table(*plan))) {
        delete *plan;
        *plan = nullptr;
    }
    return s;
}

int ct_fan_sysmat(ct_fan_plan *plan, long long *d_row_ptr, int *d_col, float *d_val, long long cap, long long *nnz,
                  void *stream) {
    CT_REQUIRE(plan, "ct_fan_sysmat: null plan");
    const FanGeom &g = plan->g;
    cudaStream_t st = as_stream(stream);
    auto launch = [&](const GrazeList &gl, bool fill) {
        return fan_sysmat_launch(g, d_row_ptr, d_col, d_val, fill, gl, st);
    };
    return sysmat_common(launch, plan->graze, plan->scan, (long long)g.nb * g.np, d_row_ptr, d_col, d_val, cap, nnz,
                         st);
}

int ct_fan_plan_grazing_rays(const ct_fan_plan *plan, long long *n, void *stream) {
    CT_REQUIRE(plan, "ct_fan_plan_grazing_rays: null plan");
    return graze_count(plan->graze, n, as_stream(stream));
}

int ct_fan_plan_set_filter(ct_fan_plan *plan, int kind, int window_len) {
    CT_REQUIRE(plan, "plan is null");
    int s = check_filter_opts(kind, window_len);
    if (s) return s;
    plan->filt.kind = kind;
    plan->filt.wlen = window_len;
    plan->G.release();   // tables are rebuilt on the next filter call
    return CT_OK;
}

int ct_fan_plan_set_short_scan(ct_fan_plan *plan, int enable) {
    CT_REQUIRE(plan, "plan is null");
    CT_REQUIRE(enable == 0 || enable == 1, "enable must be 0 or 1");
    CT_REQUIRE(!plan->g.parallel, "short-scan weights need a fan geometry");
    plan->filt.short_scan = enable;
    plan->G.release();
    return CT_OK;
}

int ct_fan_fp(ct_fan_plan *plan, const float *d_img, float *d_proj, void *stream) {
    CT_REQUIRE(plan && d_img && d_proj, "ct_fan_fp: null argument");
    GrazeList gl;
    int s = graze_list(plan->graze, gl, (long long)plan->g.nb * plan->g.np, as_stream(stream));
    if (s) return s;
    return fan_fp_launch(plan->g, d_img, d_proj, nullptr, nullptr, 0.f, nullptr, 0, gl, as_stream(stream));
}

int ct_fan_fp_residual(ct_fan_plan *plan, const float *d_img, const float *d_b, const float *d_rowsum, float eps,
                       float *d_out, double *d_norms, void *stream) {
    CT_REQUIRE(plan && d_img && d_b && d_out && d_norms, "ct_fan_fp_residual: null argument");
    GrazeList gl;
    int s = graze_list(plan->graze, gl, (long long)plan->g.nb * plan->g.np, as_stream(stream));
    if (s) return s;
    return fan_fp_launch(plan->g, d_img, d_out, d_b, d_rowsum, eps, d_norms, 1, gl, as_stream(stream));
}

int ct_fan_bp(ct_fan_plan *plan, const float *d_proj, float *d_img, void *stream) {
    CT_REQUIRE(plan && d_proj && d_img, "ct_fan_bp: null argument");
    return fan_bp_launch(plan->g, d_proj, d_img, plan->g.parallel ? 2 : 0, nullptr, 0.f, 0.f, 0.f, 0.f, false,
                         as_stream(stream));
}

int ct_fan_bp_update(ct_fan_plan *plan, const float *d_proj, const float *d_colsum, float eps, float lambda,
                     float lo, float hi, float *d_img, void *stream) {
    CT_REQUIRE(plan && d_proj && d_colsum && d_img, "ct_fan_bp_update: null argument");
    return fan_bp_launch(plan->g, d_proj, d_img, 0, d_colsum, eps, lambda, lo, hi, true, as_stream(stream));
}

// FBP of a 2D fan (FBPfan.cu) or parallel (FBPparallel.cu) sinogram.
int ct_fan_fbp(ct_fan_plan *plan, const float *d_proj, float *d_img, int filter_mode, void *stream) {
    CT_REQUIRE(plan && d_proj && d_img, "ct_fan_fbp: null argument");
    FanGeom &g = plan->g;
    CT_REQUIRE(g.np >= 2, "ct_fan_fbp: at least 2 detector bins");
    cudaStream_t st = as_stream(stream);
    int s;
    if (!plan->G.ptr) {
        if ((s = filter_tables(plan->filt, g.pint, g.np, plan->hbf, plan->hPf, g.D, plan->G, plan->pwt, plan->win,
                               plan->wsum)))
            return s;
        if (!g.parallel) {
            std::vector<double> w(g.np);   // Rscan / sqrt(Rscan^2 + P^2) (FBPfan.cu:32)
            for (int p = 0; p < g.np; ++p) {
                const double Pv = plan->hPf[p];
                w[p] = g.D / std::sqrt(1.0 * g.D * g.D + 1.0 * Pv * Pv);
            }
            if ((s = upload(plan->wtab, w.data(), w.size()))) return s;
        }
    }
    if ((s = plan->rcov.ensure(sizeof(float) * (size_t)g.nb * g.np))) return s;
    RowFilter f{};
    f.nrow = g.nb;
    f.np = g.np;
    f.pint = g.pint;
    f.G = plan->G.as<float>();
    f.w = g.parallel ? nullptr : plan->wtab.as<double>();
    f.wrows = 1;
    f.launch_order = filter_mode;
    f.tile = g.parallel ? 256 : 128;          // FBPparallel.h:24 / FBPfan.h:24
    f.limit = g.parallel ? 2048 : 1024;       // FBPparallel.h:26 / FBPfan.h:26
    f.row_block = g.parallel ? 256 : 128;
    f.rowmod = g.nb;
    filter_fields(plan->filt, 1, plan->pwt, plan->win, plan->wsum, f);
    if ((s = row_filter_launch(f, d_proj, plan->rcov.as<float>(), st))) return s;
    return fan_bp_launch(g, plan->rcov.as<float>(), d_img, g.parallel ? 2 : 1, nullptr, 0.f, 0.f, 0.f, 0.f, false,
                         st);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Drop-in host-pointer entry points
// ---------------------------------------------------------------------------
namespace {

std::mutex g_dropin_mutex;

struct DropinState {
    ct_cone_plan *cone = nullptr;
    DevBuf vol, proj;
    // streams and events of the overlapped path (pinned host buffers)
    int dev = -1;
    cudaStream_t cs = nullptr, xs = nullptr;   // kernels, and the copies that overlap them
    std::vector<cudaEvent_t> ev;
};
DropinState &dropin() {
    static DropinState st;
    return st;
}

void dropin_streams_release(DropinState &st) {
    for (cudaEvent_t e : st.ev) cudaEventDestroy(e);
    st.ev.clear();
    if (st.cs) cudaStreamDestroy(st.cs);
    if (st.xs) cudaStreamDestroy(st.xs);
    st.cs = st.xs = nullptr;
    st.dev = -1;
}

// The two streams and nev events of the overlapped path on the current device.
int dropin_streams(DropinState &st, int nev) {
    int dev = 0;
    CT_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (st.cs && st.dev != dev) dropin_streams_release(st);
    if (!st.cs) {
        CT_CUDA(cudaStreamCreateWithFlags(&st.cs, cudaStreamNonBlocking), "drop-in stream");
        CT_CUDA(cudaStreamCreateWithFlags(&st.xs, cudaStreamNonBlocking), "drop-in copy stream");
        st.dev = dev;
    }
    while ((int)st.ev.size() < nev) {
        cudaEvent_t e;
        CT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "drop-in event");
        st.ev.push_back(e);
    }
    return CT_OK;
}

// Page-locked (or registered) host memory: copies from it run asynchronously.
bool host_pinned(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Views per chunk of the overlapped drop-in path: the forward projection of a
// chunk overlaps the copy-out of the previous one, and the copy-in of a chunk
// the backprojection of the previous one.
constexpr int kDropinChunk = kFpViewChunk;
// z slabs of the overlapped backprojection's last chunk, each copied out while
// the next is summed (only the last slab's copy is left after the kernels)
constexpr int kDropinSlabs = 4;

// Reuse the cached cone plan when the geometry is unchanged.
int cached_cone_plan(ct_cone_plan **out, int nt, int ns, int nz, const double *Size, const float *beta, int nb,
                     const float *P, int np, const float *xi, int nx, double D) {
    DropinState &st = dropin();
    ct_cone_plan *pl = st.cone;
    if (pl && pl->g.nt == nt && pl->g.ns == ns && pl->g.nz == nz && pl->g.nb == nb && pl->g.np == np &&
        pl->g.nx == nx && pl->g.D == D && pl->hsize[0] == Size[0] && pl->hsize[1] == Size[1] &&
        pl->hsize[2] == Size[2] && !std::memcmp(pl->hb.data(), beta, sizeof(float) * nb) &&
        !std::memcmp(pl->hp.data(), P, sizeof(float) * np) && !std::memcmp(pl->hx.data(), xi, sizeof(float) * nx)) {
        *out = pl;
        return CT_OK;
    }
    ct_cone_plan *np_ = nullptr;
    int s = ct_cone_plan_create(&np_, nt, ns, nz, Size, beta, nb, P, np, xi, nx, D);
    if (s) return s;
    if (st.cone) ct_cone_plan_destroy(st.cone);
    st.cone = np_;
    *out = np_;
    return CT_OK;
}

}  // namespace

extern "C" {

int ct_dropin_release(void) {
    {
        std::lock_guard<std::mutex> lk(g_dropin_mutex);
        DropinState &st = dropin();
        if (st.cone) ct_cone_plan_destroy(st.cone);
        st.cone = nullptr;
        st.vol.release();
        st.proj.release();
        dropin_streams_release(st);
    }
    iterfdk_release_cache();
    fdkui_release_cache();
    return CT_OK;
}

int ct_ProjectionCone_3D(const float *Pic, float *Projection, const float *BetaScanRange, const float *Pdomain,
                         const float *Xigamadomain, int t_length, int s_length, int z_length, double Center_t,
                         double Center_s, double Center_z, int LBeta, int LP, int LXigama, double Distance,
                         const double *resolution) {
    CT_REQUIRE(Pic && Projection && resolution, "ct_ProjectionCone_3D: null argument");
    std::lock_guard<std::mutex> lk(g_dropin_mutex);
    // the gateway passes Center = Size/2 and resolution = Size/length (ProjectionCone_3D.cpp:10-22)
    const double Size[3] = {resolution[0] * t_length, resolution[1] * s_length, resolution[2] * z_length};
    CT_REQUIRE(std::fabs(Center_t - 0.5 * Size[0]) <= 1e-9 * Size[0] &&
                   std::fabs(Center_s - 0.5 * Size[1]) <= 1e-9 * Size[1] &&
                   std::fabs(Center_z - 0.5 * Size[2]) <= 1e-9 * Size[2],
               "ct_ProjectionCone_3D: the rotation centre must be the volume centre");
    ct_cone_plan *pl;
    int s = cached_cone_plan(&pl, t_length, s_length, z_length, Size, BetaScanRange, LBeta, Pdomain, LP,
                             Xigamadomain, LXigama, Distance);
    if (s) return s;
    // keep the exact resolution the caller passed
    for (int a = 0; a < 3; ++a) {
        pl->g.res[a] = resolution[a];
        pl->g.ires[a] = 1.0 / resolution[a];
    }
    cone_geom_derive(pl->g);
    if ((s = cone_fp_refresh(pl))) return s;
    DropinState &st = dropin();
    const size_t nv = (size_t)t_length * s_length * z_length, npj = (size_t)LBeta * LP * LXigama;
    if ((s = st.vol.ensure(nv * sizeof(float))) || (s = st.proj.ensure(npj * sizeof(float)))) return s;
    if (LBeta <= kDropinChunk || !host_pinned(Pic) || !host_pinned(Projection)) {
        CT_CUDA(cudaMemcpy(st.vol.ptr, Pic, nv * sizeof(float), cudaMemcpyHostToDevice), "H2D volume");
        if ((s = ct_cone_fp(pl, st.vol.as<float>(), st.proj.as<float>(), nullptr))) return s;
        CT_CUDA(cudaMemcpy(Projection, st.proj.ptr, npj * sizeof(float), cudaMemcpyDeviceToHost), "D2H projection");
        return CT_OK;
    }
    // pinned buffers: project view chunks and copy each chunk out while the next is projected
    const int nchunks = (LBeta + kDropinChunk - 1) / kDropinChunk;
    if ((s = dropin_streams(st, nchunks))) return s;
    CT_CUDA(cudaMemcpyAsync(st.vol.ptr, Pic, nv * sizeof(float), cudaMemcpyHostToDevice, st.cs), "H2D volume");
    GrazeList gl;
    const float *volS, *volT;
    if ((s = graze_list(pl->graze, gl, cone_rays(pl->g), st.cs)) ||
        (s = fp_volumes(pl, st.vol.as<float>(), &volS, &volT, st.cs)))
        return s;
    const size_t per_view = (size_t)LP * LXigama;
    for (int c = 0; c < nchunks; ++c) {
        const int v0 = c * kDropinChunk, n = std::min(kDropinChunk, LBeta - v0);
        if ((s = cone_fp_launch(pl->g, pl->cols.as<FpColumn>(), volS, volT, st.vol.as<float>(), st.proj.as<float>(),
                                nullptr, nullptr, 0.0f, nullptr, 0, gl, st.cs, v0, n)))
            return s;
        CT_CUDA(cudaEventRecord(st.ev[c], st.cs), "event");
        CT_CUDA(cudaStreamWaitEvent(st.xs, st.ev[c], 0), "event wait");
        CT_CUDA(cudaMemcpyAsync(Projection + v0 * per_view, st.proj.as<float>() + v0 * per_view,
                                n * per_view * sizeof(float), cudaMemcpyDeviceToHost, st.xs),
                "D2H projection");
    }
    CT_CUDA(cudaStreamSynchronize(st.xs), "sync");
    CT_CUDA(cudaStreamSynchronize(st.cs), "sync");
    return CT_OK;
}

static int cone_bp_dropin(float *Display, const float *R, const float *xi, const float *P, const float *beta,
                          double D, int nb, int np, int nx, const double *Size, int nt, int ns, int nz, bool fdk) {
    CT_REQUIRE(Display && R && Size, "null argument");
    std::lock_guard<std::mutex> lk(g_dropin_mutex);
    ct_cone_plan *pl;
    int s = cached_cone_plan(&pl, nt, ns, nz, Size, beta, nb, P, np, xi, nx, D);
    if (s) return s;
    DropinState &st = dropin();
    const size_t nv = (size_t)nt * ns * nz, npj = (size_t)nb * np * nx;
    if ((s = st.vol.ensure(nv * sizeof(float))) || (s = st.proj.ensure(npj * sizeof(float)))) return s;
    const int bchunk = std::min(cone_bp_chunk_views(pl), kDropinChunk * 2);
    if (!fdk && nb > bchunk && np >= 2 && nx >= 2 && host_pinned(R) && host_pinned(Display)) {
        // pinned buffers: copy view chunks (the backprojector's own chunks) in,
        // each backprojected (and added to the volume) while the next one arrives;
        // the last chunk runs in z slabs, each copied out while the next is summed
        const int nchunks = (nb + bchunk - 1) / bchunk;
        const int ztile = cone_bp_ztile(), ntiles = (nz + ztile - 1) / ztile;
        const int nslab = std::min(kDropinSlabs, ntiles);
        if ((s = dropin_streams(st, nchunks + nslab)) || (s = pl->quads.ensure(cone_quads_bytes(pl->g, bchunk))))
            return s;
        const size_t per_view = (size_t)np * nx;
        for (int c = 0; c < nchunks; ++c) {
            const int v0 = c * bchunk, n = std::min(bchunk, nb - v0);
            CT_CUDA(cudaMemcpyAsync(st.proj.as<float>() + v0 * per_view, R + v0 * per_view,
                                    n * per_view * sizeof(float), cudaMemcpyHostToDevice, st.xs),
                    "H2D projection");
            CT_CUDA(cudaEventRecord(st.ev[c], st.xs), "event");
        }
        for (int c = 0; c < nchunks; ++c) {
            const int v0 = c * bchunk, n = std::min(bchunk, nb - v0);
            const bool last = c == nchunks - 1;
            CT_CUDA(cudaStreamWaitEvent(st.cs, st.ev[c], 0), "event wait");
            if ((s = cone_pack_quads(pl->g, st.proj.as<float>(), pl->quads.as<float4>(), v0, n, st.cs))) return s;
            for (int k = 0; k < (last ? nslab : 1); ++k) {
                const int t0 = last ? k * ntiles / nslab : 0, t1 = last ? (k + 1) * ntiles / nslab : ntiles;
                if ((s = cone_bp_launch(pl->g, pl->quads.as<float4>(), v0, n, c == 0 ? nullptr : st.vol.as<float>(),
                                        st.vol.as<float>(), 0, nullptr, 0.f, 0.f, 0.f, 0.f, false, st.cs, t0,
                                        t1 - t0)))
                    return s;
                if (last) {
                    // slices [t0, t1) * ztile are final: copy them out behind the next slab
                    const size_t slice = (size_t)nt * ns, za = (size_t)t0 * ztile,
                                 zb = std::min<size_t>(nz, (size_t)t1 * ztile);
                    CT_CUDA(cudaEventRecord(st.ev[nchunks + k], st.cs), "event");
                    CT_CUDA(cudaStreamWaitEvent(st.xs, st.ev[nchunks + k], 0), "event wait");
                    CT_CUDA(cudaMemcpyAsync(Display + za * slice, st.vol.as<float>() + za * slice,
                                            (zb - za) * slice * sizeof(float), cudaMemcpyDeviceToHost, st.xs),
                            "D2H volume");
                }
            }
        }
        CT_CUDA(cudaStreamSynchronize(st.xs), "sync");
        CT_CUDA(cudaStreamSynchronize(st.cs), "sync");
        return CT_OK;
    }
    CT_CUDA(cudaMemcpy(st.proj.ptr, R, npj * sizeof(float), cudaMemcpyHostToDevice), "H2D projection");
    s = fdk ? ct_cone_fdk(pl, st.proj.as<float>(), st.vol.as<float>(), nullptr)
            : ct_cone_bp(pl, st.proj.as<float>(), st.vol.as<float>(), nullptr);
    if (s) return s;
    CT_CUDA(cudaMemcpy(Display, st.vol.ptr, nv * sizeof(float), cudaMemcpyDeviceToHost), "D2H volume");
    return CT_OK;
}

int ct_BackPro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
               const float *BetaScanRange, double Distance, int LBeta, int LP, int LXigama, const double *Size,
               int t_length, int s_length, int z_length) {
    return cone_bp_dropin(Display, R, Xigamadomain, Pdomain, BetaScanRange, Distance, LBeta, LP, LXigama, Size,
                          t_length, s_length, z_length, false);
}

int ct_FDKpro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
              const float *BetaScanRange, double Distance, int LBeta, int LP, int LXigama, const double *Size,
              int t_length, int s_length, int z_length) {
    return cone_bp_dropin(Display, R, Xigamadomain, Pdomain, BetaScanRange, Distance, LBeta, LP, LXigama, Size,
                          t_length, s_length, z_length, true);
}

// 2D entry points: small problems, a plan per call.
static int fan2d_run(ct_fan_plan *pl, int which, const void *in, void *out, int filter_mode) {
    FanGeom &g = pl->g;
    const size_t nimg = (size_t)g.nt * g.ns, nsino = (size_t)g.nb * g.np;
    DevBuf a, b;
    int s = 0;
    const bool fp = which == 0;
    if ((s = a.ensure((fp ? nimg : nsino) * sizeof(float))) ||
        (s = b.ensure((fp ? nsino * sizeof(double) : nimg * sizeof(float))))) {
        a.release();
        b.release();
        return s;
    }
    cudaError_t e = cudaMemcpy(a.ptr, in, (fp ? nimg : nsino) * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) s = cuda_status(e, "H2D");
    if (!s) {
        GrazeList gl;
        if (fp && !(s = graze_list(pl->graze, gl, (long long)nsino, 0)))
            s = fan_fp_launch(g, a.as<float>(), b.ptr, nullptr, nullptr, 0.f, nullptr, 3, gl, 0);
        else if (which == 1) s = fan_bp_launch(g, a.as<float>(), b.as<float>(), 0, nullptr, 0, 0, 0, 0, false, 0);
        else s = ct_fan_fbp(pl, a.as<float>(), b.as<float>(), filter_mode, nullptr);
    }
    if (!s) {
        e = cudaMemcpy(out, b.ptr, fp ? nsino * sizeof(double) : nimg * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) s = cuda_status(e, "D2H");
    }
    a.release();
    b.release();
    return s;
}

int ct_ProjectionFan_2D(const float *Pic, double *Projection, const double *BetaScanRange, const double *Pdomain,
                        int t_length, int s_length, double Center_t, double Center_s, int LBeta, int LP,
                        double Distance, const double *resolution) {
    CT_REQUIRE(Pic && Projection && resolution, "ct_ProjectionFan_2D: null argument");
    const double size2[2] = {resolution[0] * t_length, resolution[1] * s_length};
    CT_REQUIRE(std::fabs(Center_t - 0.5 * size2[0]) <= 1e-9 * size2[0] &&
                   std::fabs(Center_s - 0.5 * size2[1]) <= 1e-9 * size2[1],
               "ct_ProjectionFan_2D: the rotation centre must be the image centre");
    ct_fan_plan *pl;
    int s = fan_plan_make(&pl, t_length, s_length, size2, BetaScanRange, LBeta, Pdomain, LP, Distance, 0);
    if (s) return s;
    pl->g.res[0] = resolution[0];
    pl->g.res[1] = resolution[1];
    s = fan2d_run(pl, 0, Pic, Projection, 0);
    ct_fan_plan_destroy(pl);
    return s;
}

int ct_ProjectionParallel_2D(const float *Pic, double *Projection, const double *thetaRange, const double *t_Range,
                             int height, int width, double Center_y, double Center_x, int Ltheta, int Lt,
                             const double *resolution) {
    CT_REQUIRE(Pic && Projection && resolution, "ct_ProjectionParallel_2D: null argument");
    // x runs along width (resolution[1]), y along height (resolution[0]); pixel y*width + x
    const double size2[2] = {resolution[1] * width, resolution[0] * height};
    CT_REQUIRE(std::fabs(Center_x - 0.5 * size2[0]) <= 1e-9 * size2[0] &&
                   std::fabs(Center_y - 0.5 * size2[1]) <= 1e-9 * size2[1],
               "ct_ProjectionParallel_2D: the rotation centre must be the image centre");
    ct_fan_plan *pl;
    int s = fan_plan_make(&pl, width, height, size2, thetaRange, Ltheta, t_Range, Lt, 0.0, 1);
    if (s) return s;
    pl->g.res[0] = resolution[1];
    pl->g.res[1] = resolution[0];
    s = fan2d_run(pl, 0, Pic, Projection, 0);
    ct_fan_plan_destroy(pl);
    return s;
}

static int fan_plan_from_float(ct_fan_plan **pl, const float *P, const float *beta, int nb, int np, const double *Size,
                               int nt, int ns, double D, int parallel) {
    CT_REQUIRE(P && beta && Size, "null argument");
    std::vector<double> bd(beta, beta + nb), pd(P, P + np);
    return fan_plan_make(pl, nt, ns, Size, bd.data(), nb, pd.data(), np, D, parallel);
}

int ct_BackprojectionFan2D(float *Display, const float *R, const float *Pdomain, const float *BetaScanRange,
                           int LBeta, int LP, const double *Size, int t_length, int s_length, double Rscan) {
    CT_REQUIRE(Display && R, "ct_BackprojectionFan2D: null argument");
    ct_fan_plan *pl;
    int s = fan_plan_from_float(&pl, Pdomain, BetaScanRange, LBeta, LP, Size, t_length, s_length, Rscan, 0);
    if (s) return s;
    s = fan2d_run(pl, 1, R, Display, 0);
    ct_fan_plan_destroy(pl);
    return s;
}

int ct_FBPfan(float *Display, const float *R, const float *Pdomain, const float *BetaScanRange, int LBeta, int LP,
              const double *Size, int t_length, int s_length, double Rscan) {
    CT_REQUIRE(Display && R, "ct_FBPfan: null argument");
    ct_fan_plan *pl;
    int s = fan_plan_from_float(&pl, Pdomain, BetaScanRange, LBeta, LP, Size, t_length, s_length, Rscan, 0);
    if (s) return s;
    s = fan2d_run(pl, 2, R, Display, CT_FDK_FILTER_LAUNCH_ORDER);
    ct_fan_plan_destroy(pl);
    return s;
}

int ct_FBPpara(float *Display, const float *R, const float *Tdomain, const float *ThetaScanRange, int LTheta, int LT,
               const double *Size, int t_length, int s_length) {
    CT_REQUIRE(Display && R, "ct_FBPpara: null argument");
    ct_fan_plan *pl;
    int s = fan_plan_from_float(&pl, Tdomain, ThetaScanRange, LTheta, LT, Size, t_length, s_length, 0.0, 1);
    if (s) return s;
    s = fan2d_run(pl, 2, R, Display, 0);
    ct_fan_plan_destroy(pl);
    return s;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batches of uneven 2D fan slices (fan_batch.cu)
// ---------------------------------------------------------------------------
struct ct_fan_batch {
    std::vector<ct_fan_plan *> plans;
    std::vector<BatchSlice> h;
    DevBuf desc;
    GrazeBuf graze;
    int fp_block = 128, bp_block = 128;
    int fp_blocks = 0, bp_blocks = 0;
    long long img_total = 0, sino_total = 0;
    ~ct_fan_batch() {
        for (ct_fan_plan *p : plans) delete p;
        desc.release();
        graze.release();
    }
};

// Offsets of every slice in the packed buffers and its first block in each grid.
static int batch_layout(ct_fan_batch *b) {
    long long io = 0, so = 0, fb = 0, bb = 0;
    for (size_t k = 0; k < b->plans.size(); ++k) {
        BatchSlice &s = b->h[k];
        s.g = b->plans[k]->g;
        fan_geom_derive(s.g);
        s.img_off = io;
        s.sino_off = so;
        s.ray_blk0 = (int)fb;
        s.pix_blk0 = (int)bb;
        const long long nr = (long long)s.g.nb * s.g.np, npx = (long long)s.g.nt * s.g.ns;
        io += npx;
        so += nr;
        fb += (nr + b->fp_block - 1) / b->fp_block;
        bb += (npx + b->bp_block - 1) / b->bp_block;
    }
    CT_REQUIRE(fb < (1LL << 31) && bb < (1LL << 31), "batch too large for one launch");
    b->img_total = io;
    b->sino_total = so;
    b->fp_blocks = (int)fb;
    b->bp_blocks = (int)bb;
    return upload(b->desc, b->h.data(), b->h.size());
}

extern "C" {

int ct_fan_batch_create(ct_fan_batch **out, int nslices, const int *t_length, const int *s_length, const double *Size,
                        const double *const *BetaScanRange, const int *LBeta, const double *const *Pdomain,
                        const int *LP, const double *Distance) {
    CT_REQUIRE(out && nslices > 0 && t_length && s_length && Size && BetaScanRange && LBeta && Pdomain && LP &&
                   Distance,
               "ct_fan_batch_create: null argument");
    CT_REQUIRE(nslices < (1 << 23), "ct_fan_batch_create: too many slices");
    *out = nullptr;
    ct_fan_batch *b = new ct_fan_batch();
    b->plans.assign(nslices, nullptr);
    b->h.resize(nslices);
    for (int k = 0; k < nslices; ++k) {
        int s = LP[k] >= 2 ? ct_fan_plan_create(&b->plans[k], t_length[k], s_length[k], Size + 2 * k,
                                                 BetaScanRange[k], LBeta[k], Pdomain[k], LP[k], Distance[k])
                           : (set_error("ct_fan_batch_create: every slice needs at least 2 detector bins"), CT_ERR_ARG);
        if (!s && (long long)LBeta[k] * LP[k] >= (1LL << 40)) {
            set_error("ct_fan_batch_create: slice sinogram too large");
            s = CT_ERR_ARG;
        }
        if (s) {
            delete b;
            return s;
        }
    }
    int s = batch_layout(b);
    if (s) {
        delete b;
        return s;
    }
    *out = b;
    return CT_OK;
}

int ct_fan_batch_destroy(ct_fan_batch *batch) {
    delete batch;
    return CT_OK;
}

int ct_fan_batch_layout(const ct_fan_batch *b, long long *img_offsets, long long *sino_offsets) {
    CT_REQUIRE(b && img_offsets && sino_offsets, "ct_fan_batch_layout: null argument");
    const size_t n = b->h.size();
    for (size_t k = 0; k < n; ++k) {
        img_offsets[k] = b->h[k].img_off;
        sino_offsets[k] = b->h[k].sino_off;
    }
    img_offsets[n] = b->img_total;
    sino_offsets[n] = b->sino_total;
    return CT_OK;
}

int ct_fan_batch_set_blocks(ct_fan_batch *b, int fp_block, int bp_block) {
    CT_REQUIRE(b, "ct_fan_batch_set_blocks: null batch");
    CT_REQUIRE(fp_block >= 32 && fp_block <= 512 && fp_block % 32 == 0 && bp_block >= 32 && bp_block <= 512 &&
                   bp_block % 32 == 0,
               "ct_fan_batch_set_blocks: block sizes must be multiples of 32 in [32, 512]");
    b->fp_block = fp_block;
    b->bp_block = bp_block;
    return batch_layout(b);
}

int ct_fan_batch_set_filter(ct_fan_batch *b, int kind, int window_len, int short_scan) {
    CT_REQUIRE(b, "ct_fan_batch_set_filter: null batch");
    for (ct_fan_plan *p : b->plans) {
        int s;
        if ((s = ct_fan_plan_set_filter(p, kind, window_len)) || (s = ct_fan_plan_set_short_scan(p, short_scan)))
            return s;
    }
    return CT_OK;
}

int ct_fan_batch_grazing_rays(const ct_fan_batch *b, long long *n, void *stream) {
    CT_REQUIRE(b, "ct_fan_batch_grazing_rays: null batch");
    return graze_count(b->graze, n, as_stream(stream));
}

int ct_fan_batch_fp(ct_fan_batch *b, const float *d_img, float *d_proj, void *stream) {
    CT_REQUIRE(b && d_img && d_proj, "ct_fan_batch_fp: null argument");
    GrazeList gl;
    int s = graze_list(b->graze, gl, b->sino_total, as_stream(stream));
    if (s) return s;
    return fan_batch_fp_launch(b->desc.as<BatchSlice>(), (int)b->h.size(), b->fp_blocks, b->fp_block, d_img, d_proj,
                               nullptr, nullptr, 0.f, nullptr, 0, gl, as_stream(stream));
}

int ct_fan_batch_fp_residual(ct_fan_batch *b, const float *d_img, const float *d_b, const float *d_rowsum, float eps,
                             float *d_out, double *d_norms, void *stream) {
    CT_REQUIRE(b && d_img && d_b && d_out && d_norms, "ct_fan_batch_fp_residual: null argument");
    GrazeList gl;
    int s = graze_list(b->graze, gl, b->sino_total, as_stream(stream));
    if (s) return s;
    return fan_batch_fp_launch(b->desc.as<BatchSlice>(), (int)b->h.size(), b->fp_blocks, b->fp_block, d_img, d_out,
                               d_b, d_rowsum, eps, d_norms, 1, gl, as_stream(stream));
}

int ct_fan_batch_bp(ct_fan_batch *b, const float *d_proj, float *d_img, void *stream) {
    CT_REQUIRE(b && d_proj && d_img, "ct_fan_batch_bp: null argument");
    return fan_batch_bp_launch(b->desc.as<BatchSlice>(), (int)b->h.size(), b->bp_blocks, b->bp_block, d_proj, d_img, 0,
                               nullptr, 0.f, 0.f, 0.f, 0.f, false, as_stream(stream));
}

int ct_fan_batch_bp_update(ct_fan_batch *b, const float *d_proj, const float *d_colsum, float eps, float lambda,
                           float lo, float hi, float *d_img, void *stream) {
    CT_REQUIRE(b && d_proj && d_colsum && d_img, "ct_fan_batch_bp_update: null argument");
    return fan_batch_bp_launch(b->desc.as<BatchSlice>(), (int)b->h.size(), b->bp_blocks, b->bp_block, d_proj, d_img, 0,
                               d_colsum, eps, lambda, lo, hi, true, as_stream(stream));
}

int ct_fan_batch_fbp(ct_fan_batch *b, const float *d_proj, float *d_img, int filter_mode, void *stream) {
    CT_REQUIRE(b && d_proj && d_img, "ct_fan_batch_fbp: null argument");
    for (size_t k = 0; k < b->h.size(); ++k) {
        int s = ct_fan_fbp(b->plans[k], d_proj + b->h[k].sino_off, d_img + b->h[k].img_off, filter_mode, stream);
        if (s) return s;
    }
    return CT_OK;
}

}  // extern "C"
