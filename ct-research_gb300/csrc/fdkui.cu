// fdkui.cu -- curved-detector (equiangular) short-scan FDK of ImplementUI.cu.
//
// The scanner pipeline of the reference (ImplementUI.cu:6-158): R is double,
// [view][xi][gamma] on an equiangular detector (gamma in radians, xi rows in
// mm at the source-to-detector distance Ds2d).
//  1. Taps per xi row (GFunction :6-22): the S-L kernel of the equiangular
//     detector, 2/(pi dG')^2 at the centre and
//     -2 n^2 / pi^2 / (4n^2 - 1) / sin^2(n dG') at offset n, dG' = dG * prop(xi)
//     with prop = Ds2d / sqrt(Ds2d^2 + xi^2).
//  2. Weight and filter (PreWeightFiltration :25-86): every sample times
//     (D / prop) cos(gamma prop) W, W the Parker weight of
//     (beta prop, b0 prop, gamma prop, fan prop); then the row convolved with
//     its taps, times dG'.
//  3. Backprojection (BackProjection :88-150): per voxel and view, the
//     bilinear sample at gamma = atan(t_rot / (D - s_rot)) and
//     xi = Ds2d tan(asin(z / |voxel - source|)), times dBeta / (dG dXi) / L2 / prop.
//
// GB300 design:
//  * Filter: one block per row.  The weights run in double exactly as the
//    reference orders them (the Parker branch tests decide between 0, a ramp
//    and 1, and at a symmetric detector's edge the reference's own rounding
//    yields NaN rows, reproduced).  The O(LG^2) convolution runs in FP32 on
//    float pairs (~2^-46 relative per product, TwoSum accumulation), not in
//    GB300's 1/64-rate FP64; the row goes out as float.
//  * Backprojection: one thread per (t, s) column and 16 z, views inside.
//    The row coordinates sit in shared memory.  Per
//    column-view the offset of gamma from its detector sample is computed in
//    double (one division, by the tangent-difference identity) since its
//    bilinear weights are differences at the scale of dG ~ 1e-3 rad; the
//    xi position is linear in z (tan(asin(z/sqrt(L2))) = z / sqrt(L2 - z^2),
//    and L2 - z^2 is the in-plane distance), so the per-voxel work is FP32,
//    accumulated in float pairs and written once as double.
#include <cmath>
#include <mutex>
#include <vector>

#include "devbuf.cuh"
#include "kernels.cuh"

namespace ct {

namespace {

constexpr double kPiUI = 3.141592653589793;

struct UIGeom {
    int lg, lb, lx;               // gammas, views, xi rows
    int nt, ns, nz;               // display: Size[0] x Size[1] x z_length
    double gint, xint, bint;
    double ming, maxg, minx, maxx;
    double g0, x0;
    double b0, fan, D, ds2d;
    double ct, cs, cz, rz;
};

// ---------------------------------------------------------------------------
// filter
// ---------------------------------------------------------------------------
constexpr int kUIFilterBlock = 256;

__device__ __forceinline__ float2 split(double d) {
    const float h = (float)d;
    return make_float2(h, (float)(d - (double)h));
}

// One block per (view, xi) row.  Shared memory: the weighted row and the
// row's taps, both as float pairs.
__global__ void __launch_bounds__(kUIFilterBlock)
fdkui_filter_kernel(const UIGeom g, const double *__restrict__ R, const double *__restrict__ beta,
                    const double *__restrict__ gama, const double *__restrict__ xi, const float2 *__restrict__ taps,
                    float *__restrict__ rcov) {
    extern __shared__ float2 smu[];
    float2 *w = smu;              // lg
    float2 *G = smu + g.lg;       // 2 lg - 1
    const int row = blockIdx.x;   // view * lx + x
    const int b = row / g.lx, x = row % g.lx;
    const double xv = xi[x];
    const double pr = __ddiv_rn(g.ds2d, sqrt(__dadd_rn(__dmul_rn(g.ds2d, g.ds2d), __dmul_rn(xv, xv))));
    const double bp = __dmul_rn(beta[b], pr), b0p = __dmul_rn(g.b0, pr), mgp = __dmul_rn(g.fan, pr);
    const double dp = __ddiv_rn(g.D, pr), gip = __dmul_rn(g.gint, pr);
    const double *in = R + (long long)row * g.lg;
    const int fs = 2 * g.lg - 1;
    const float2 *tr = taps + (long long)x * fs;
    for (int i = threadIdx.x; i < fs; i += blockDim.x) G[i] = tr[i];
    for (int q = threadIdx.x; q < g.lg; q += blockDim.x) {
        const double gp = __dmul_rn(gama[q], pr);
        const double gp2 = __dmul_rn(2.0, gp);
        double W;
        // Parker weight, the reference's tests in its order (:54-61)
        if (bp >= b0p && bp < __dsub_rn(__dadd_rn(b0p, mgp), gp2)) {
            const double sn = sin(__ddiv_rn(__dmul_rn(kPiUI / 4, bp), __dsub_rn(__ddiv_rn(mgp, 2.0), gp)));
            W = __dmul_rn(sn, sn);
        } else if (bp >= __dsub_rn(__dadd_rn(b0p, mgp), gp2) && bp <= __dsub_rn(__dadd_rn(b0p, kPiUI), gp2)) {
            W = 1.0;
        } else if (bp > __dsub_rn(__dadd_rn(b0p, kPiUI), gp2) && bp <= __dadd_rn(__dadd_rn(b0p, kPiUI), mgp)) {
            const double sn = sin(__ddiv_rn(__dmul_rn(kPiUI / 4, __dsub_rn(__dadd_rn(kPiUI, mgp), bp)),
                                            __dadd_rn(__ddiv_rn(mgp, 2.0), gp)));
            W = __dmul_rn(sn, sn);
        } else {
            W = 0.0;
        }
        w[q] = split(__dmul_rn(__dmul_rn(__dmul_rn(in[q], dp), cos(gp)), W));
    }
    __syncthreads();
    float *o = rcov + (long long)row * g.lg;
    for (int p = threadIdx.x; p < g.lg; p += blockDim.x) {
        const float2 *gq = G + (g.lg - 1) + p;
        float sh = 0.0f, sl = 0.0f;
        for (int q = 0; q < g.lg; ++q) {
            const float2 a = w[q], c = gq[-q];
            const float ph = __fmul_rn(a.x, c.x);
            float pl = fmaf(a.x, c.x, -ph);
            pl = fmaf(a.x, c.y, pl);
            pl = fmaf(a.y, c.x, pl);
            const float t = __fadd_rn(sh, ph);
            const float bb = __fsub_rn(t, sh);
            const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(ph, bb));
            sh = t;
            sl = __fadd_rn(sl, __fadd_rn(e, pl));
        }
        o[p] = (float)__dmul_rn(gip, (double)sh + (double)sl);
    }
}

// ---------------------------------------------------------------------------
// backprojection
// ---------------------------------------------------------------------------
constexpr int kUIZ = 16;

// a / b in double to ~4e-15 relative: the FP32 reciprocal and one Newton step
// (the offsets it feeds need far less than a correctly rounded division)
__device__ __forceinline__ double ratio(double a, double b) {
    double r = (double)__frcp_rn((float)b);
    r = fma(r, fma(-b, r, 1.0), r);
    return a * r;
}

struct UIView {
    double cb, sb, st, ss;        // cos, sin of beta; source position
};

__global__ void __launch_bounds__(128)
fdkui_bp_kernel(const UIGeom g, const UIView *__restrict__ views, const double *__restrict__ gama,
                const double *__restrict__ tang, const float *__restrict__ dgam, const float *__restrict__ xif,
                const float *__restrict__ rcov, double *__restrict__ disp) {
    // detector-row coordinate pairs (xi[x], xi[x+1]) for the row weights
    extern __shared__ float2 xrow[];
    for (int x = threadIdx.x + 32 * threadIdx.y; x < g.lx - 1; x += 128) xrow[x] = make_float2(xif[x], xif[x + 1]);
    __syncthreads();
    const int t = blockIdx.x * 32 + threadIdx.x;
    const int s = blockIdx.y * 4 + threadIdx.y;
    const int z0 = blockIdx.z * kUIZ;
    if (t >= g.nt || s >= g.ns) return;
    const int nzc = min(kUIZ, g.nz - z0);
    const double it = (t - 0.5) - g.ct, is = (s - 0.5) - g.cs;
    float izs[kUIZ];
    float acc_h[kUIZ], acc_l[kUIZ];
#pragma unroll
    for (int k = 0; k < kUIZ; ++k) {
        izs[k] = (float)((z0 + k - 0.5) * g.rz - g.cz);
        acc_h[k] = 0.0f;
        acc_l[k] = 0.0f;
    }
    const float x0 = (float)g.x0, ixint = (float)(1.0 / g.xint);
    const float minx = (float)g.minx, maxx = (float)g.maxx;
    const float sx = (g.lx > 1 && xif[g.lx - 1] < xif[0]) ? -1.0f : 1.0f;
    const float cw0 = (float)(g.bint / (g.gint * g.xint));
    const float gsc = (float)(1.0 / g.gint);
    const long long vstride = (long long)g.lx * g.lg;
    for (int v = 0; v < g.lb; ++v) {
        const UIView vw = views[v];
        const double dt = it * vw.cb + is * vw.sb;
        const double ds = -it * vw.sb + is * vw.cb;
        const double den = g.D - ds;
        // gamma = atan(dt / den).  Its bilinear weights are differences at the
        // scale of dG, so the offset from a sample is computed in double from the
        // tangent-difference identity: gamma - G_k = atan(u),
        // u = (dt - T_k den) / (den + dt T_k), T_k = tan(G_k), |u| <~ dG, and
        // atan(u) = u - u^3/3 to 1e-16.  An FP32 atan picks the cell.
        const float gf = atanf((float)dt / (float)den);
        int g1 = (int)floorf(fabsf(gf - (float)g.g0) * gsc);
        g1 = min(max(g1, 0), g.lg - 2);
        double u = ratio(dt - tang[g1] * den, den + dt * tang[g1]);
        float dg = dgam[g1];
        float del = (float)u;
        del = del - del * del * del * (1.0f / 3.0f);
        // one step to the neighbouring cell if the estimate missed
        const float sg = dg >= 0.0f ? 1.0f : -1.0f;
        const int step = (sg * del < 0.0f && g1 > 0) ? -1 : ((sg * del > sg * dg && g1 < g.lg - 2) ? 1 : 0);
        if (step != 0) {
            g1 += step;
            u = ratio(dt - tang[g1] * den, den + dt * tang[g1]);
            dg = dgam[g1];
            del = (float)u;
            del = del - del * del * del * (1.0f / 3.0f);
        }
        const double gm = gama[g1] + (double)del;
        if (!(gm >= g.ming && gm < g.maxg)) continue;
        const float wg1 = fabsf(del), wg2 = fabsf(dg - del);
        const float ex = (float)(it - vw.st), es = (float)(is - vw.ss);
        const float l2xy = fmaf(ex, ex, es * es);
        const float rxy = sqrtf(l2xy);
        const float kx = (float)g.ds2d / rxy;              // xi per unit z
        const float cw = cw0 * rxy;                         // dBeta/(dG dXi) sqrt(L2xy)
        const float *rv = rcov + (long long)v * vstride + g1;
#pragma unroll
        for (int k = 0; k < kUIZ; ++k) {
            const float iz = izs[k];
            const float X = kx * iz;
            if (k >= nzc || !(X >= minx && X < maxx)) continue;
            int x1 = (int)floorf(fabsf(X - x0) * ixint);
            x1 = min(x1, g.lx - 2);
            const float2 xd = xrow[x1];
            const float wx1 = sx * (X - xd.x), wx2 = sx * (xd.y - X);
            const float *r1 = rv + x1 * g.lg, *r2 = r1 + g.lg;
            const float val = wx2 * fmaf(wg2, __ldg(r1), wg1 * __ldg(r1 + 1)) +
                              wx1 * fmaf(wg2, __ldg(r2), wg1 * __ldg(r2 + 1));
            const float l2 = fmaf(iz, iz, l2xy);
            const float r = rsqrtf(l2);
            const float term = val * (cw * r * r * r);      // / L2 / prop = sqrt(L2xy) / L2^1.5
            const float tt = acc_h[k] + term;
            const float bb = tt - acc_h[k];
            acc_l[k] += (acc_h[k] - (tt - bb)) + (term - bb);
            acc_h[k] = tt;
        }
    }
    double *o = disp + ((long long)z0 * g.ns + s) * g.nt + t;
    const long long plane = (long long)g.ns * g.nt;
#pragma unroll
    for (int k = 0; k < kUIZ; ++k)
        if (k < nzc) o[k * plane] = (double)acc_h[k] + (double)acc_l[k];
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
struct UIState {
    DevBuf beta, gama, tang, dgam, xi, xif, taps, views, rcov, R, disp;
    void release() {
        for (DevBuf *b : {&beta, &gama, &tang, &dgam, &xi, &xif, &taps, &views, &rcov, &R, &disp}) b->release();
    }
};
std::mutex g_ui_mutex;
UIState &ui_state() {
    static UIState st;
    return st;
}

// Equiangular S-L taps per xi row in double as GFunction computes them, as float pairs.
std::vector<float2> ui_taps(const UIGeom &g, const double *xi) {
    const int fs = 2 * g.lg - 1;
    std::vector<float2> out((size_t)g.lx * fs);
    for (int x = 0; x < g.lx; ++x) {
        const double gp = g.gint * (g.ds2d / std::sqrt(1.0 * g.ds2d * g.ds2d + 1.0 * xi[x] * xi[x]));
        float2 *row = out.data() + (size_t)x * fs;
        auto put = [&](int i, double v) {
            row[i].x = (float)v;
            row[i].y = (float)(v - (double)row[i].x);
        };
        put(g.lg - 1, 2.0 / (1.0 * (kPiUI * gp) * (kPiUI * gp)));
        for (int n = 1; n < g.lg; ++n) {
            const double sn = std::sin(n * gp);
            const double v = -2.0 * (1.0 * n * n) / (1.0 * kPiUI * kPiUI) / (4 * (1.0 * n * n) - 1) / (1.0 * sn * sn);
            put(g.lg - 1 - n, v);
            put(g.lg - 1 + n, v);
        }
    }
    return out;
}

int ui_make(UIGeom &g, const double *xi, const double *gama, const double *beta, double b0, double fan, double D,
            double ds2d, int lg, int lb, int lx, const int *size, int nz) {
    CT_REQUIRE(xi && gama && beta && size, "FDKUI: null argument");
    CT_REQUIRE(lg >= 2 && lb >= 2 && lx >= 2, "FDKUI: at least 2 gammas, views and xi rows");
    CT_REQUIRE(lg <= 4096, "FDKUI: at most 4096 gammas per row");
    CT_REQUIRE((long long)lb * lx < (1LL << 31), "FDKUI: too many rows");
    CT_REQUIRE(size[0] > 0 && size[1] > 0 && size[2] > 0 && nz > 0, "FDKUI: display sizes must be positive");
    CT_REQUIRE(size[1] <= 65535 * 4, "FDKUI: Size[1] too large");
    CT_REQUIRE(D > 0 && ds2d > 0, "FDKUI: distances must be positive");
    for (int i = 0; i < lg; ++i) CT_REQUIRE(std::isfinite(gama[i]), "FDKUI: non-finite Gamadomain");
    for (int i = 0; i < lx; ++i) CT_REQUIRE(std::isfinite(xi[i]), "FDKUI: non-finite Xigamadomain");
    for (int i = 0; i < lb; ++i) CT_REQUIRE(std::isfinite(beta[i]), "FDKUI: non-finite BetaScanRange");
    g = UIGeom{};
    g.lg = lg; g.lb = lb; g.lx = lx;
    g.nt = size[0]; g.ns = size[1]; g.nz = nz;
    g.gint = std::fabs(gama[1] - gama[0]);
    g.xint = std::fabs(xi[1] - xi[0]);
    g.bint = std::fabs(beta[1] - beta[0]);
    g.maxg = std::max(gama[0], gama[lg - 1]);
    g.ming = std::min(gama[0], gama[lg - 1]);
    g.maxx = std::max(xi[0], xi[lx - 1]);
    g.minx = std::min(xi[0], xi[lx - 1]);
    g.g0 = gama[0];
    g.x0 = xi[0];
    g.b0 = b0; g.fan = fan; g.D = D; g.ds2d = ds2d;
    // integer halves of the integer extents, as the reference divides them (:103-105)
    g.ct = size[0] / 2;
    g.cs = size[1] / 2;
    g.cz = size[2] / 2;
    g.rz = 1.0 * size[2] / nz;
    CT_REQUIRE(g.gint > 0 && g.xint > 0, "FDKUI: domains must have a non-zero step");
    return CT_OK;
}

int ui_upload(UIState &S, const UIGeom &g, const double *xi, const double *gama, const double *beta) {
    std::vector<float> xf(g.lx);
    for (int i = 0; i < g.lx; ++i) xf[i] = (float)xi[i];
    std::vector<UIView> vw(g.lb);
    for (int v = 0; v < g.lb; ++v) {
        const double b = beta[v];
        vw[v] = UIView{std::cos(b), std::sin(b), g.D * std::cos(b + kPiUI / 2), g.D * std::sin(b + kPiUI / 2)};
    }
    std::vector<float2> taps = ui_taps(g, xi);
    // per gamma sample: tan(G_k) and the cell width G_{k+1} - G_k
    std::vector<double> tg(g.lg);
    std::vector<float> dg(g.lg, 0.0f);
    for (int k = 0; k < g.lg; ++k) {
        tg[k] = std::tan(gama[k]);
        if (k + 1 < g.lg) dg[k] = (float)(gama[k + 1] - gama[k]);
    }
    int s;
    if ((s = upload(S.tang, tg.data(), tg.size())) || (s = upload(S.dgam, dg.data(), dg.size()))) return s;
    if ((s = upload(S.beta, beta, (size_t)g.lb)) || (s = upload(S.gama, gama, (size_t)g.lg)) ||
        (s = upload(S.xi, xi, (size_t)g.lx)) || (s = upload(S.xif, xf.data(), xf.size())) ||
        (s = upload(S.taps, taps.data(), taps.size())) || (s = upload(S.views, vw.data(), vw.size())))
        return s;
    return CT_OK;
}

int ui_filter(UIState &S, const UIGeom &g, const double *d_R, float *d_rcov, cudaStream_t st) {
    const size_t smem = sizeof(float2) * (size_t)(3 * g.lg - 1);
    if (smem > 48 * 1024)
        CT_CUDA(cudaFuncSetAttribute(fdkui_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "fdkui filter smem attribute");
    fdkui_filter_kernel<<<g.lb * g.lx, kUIFilterBlock, smem, st>>>(g, d_R, S.beta.as<double>(), S.gama.as<double>(),
                                                                   S.xi.as<double>(), S.taps.as<float2>(), d_rcov);
    CT_LAUNCH_CHECK("fdkui_filter_kernel");
    return CT_OK;
}

int ui_bp(UIState &S, const UIGeom &g, const float *d_rcov, double *d_disp, cudaStream_t st) {
    dim3 grid((g.nt + 31) / 32, (g.ns + 3) / 4, (g.nz + kUIZ - 1) / kUIZ);
    CT_REQUIRE(grid.z <= 65535, "FDKUI: z_length too large");
    const size_t smem = sizeof(float2) * (size_t)g.lx;
    CT_REQUIRE(smem <= 48 * 1024, "FDKUI: at most 6144 detector rows");
    fdkui_bp_kernel<<<grid, dim3(32, 4), smem, st>>>(g, S.views.as<UIView>(), S.gama.as<double>(),
                                                     S.tang.as<double>(), S.dgam.as<float>(), S.xif.as<float>(),
                                                     d_rcov, d_disp);
    CT_LAUNCH_CHECK("fdkui_bp_kernel");
    return CT_OK;
}

}  // namespace

// Free the device buffers the drop-in keeps between calls (ct_dropin_release).
void fdkui_release_cache() {
    std::lock_guard<std::mutex> lk(g_ui_mutex);
    ui_state().release();
}

}  // namespace ct

using namespace ct;

extern "C" {

int ct_fdkui_filter(const double *d_R, float *d_Rcov, const double *Xigamadomain, const double *Gamadomain,
                    const double *BetaScanRange, double betaStartAngle, double MaxGama, double Distance,
                    double Distance_s2d, int LGama, int LBeta, int LXigama, void *stream) {
    CT_REQUIRE(d_R && d_Rcov, "ct_fdkui_filter: null argument");
    const int one[3] = {1, 1, 1};
    UIGeom g;
    int s = ui_make(g, Xigamadomain, Gamadomain, BetaScanRange, betaStartAngle, MaxGama, Distance, Distance_s2d,
                    LGama, LBeta, LXigama, one, 1);
    if (s) return s;
    std::lock_guard<std::mutex> lk(g_ui_mutex);
    UIState &S = ui_state();
    if ((s = ui_upload(S, g, Xigamadomain, Gamadomain, BetaScanRange))) return s;
    return ui_filter(S, g, d_R, d_Rcov, as_stream(stream));
}

int ct_fdkui_bp(const float *d_Rcov, double *d_Display, const double *Xigamadomain, const double *Gamadomain,
                const double *BetaScanRange, double Distance, double Distance_s2d, int LGama, int LBeta,
                int LXigama, const int *Size, int z_length, void *stream) {
    CT_REQUIRE(d_Rcov && d_Display, "ct_fdkui_bp: null argument");
    UIGeom g;
    int s = ui_make(g, Xigamadomain, Gamadomain, BetaScanRange, 0.0, 0.0, Distance, Distance_s2d, LGama, LBeta,
                    LXigama, Size, z_length);
    if (s) return s;
    std::lock_guard<std::mutex> lk(g_ui_mutex);
    UIState &S = ui_state();
    if ((s = ui_upload(S, g, Xigamadomain, Gamadomain, BetaScanRange))) return s;
    return ui_bp(S, g, d_Rcov, d_Display, as_stream(stream));
}

int ct_FDKUI(double *Display, const double *R, const double *Xigamadomain, const double *Gamadomain,
             const double *BetaScanRange, double betaStartAngle, double MaxGama, double Distance,
             double Distance_s2d, int LGama, int LBeta, int LXigama, const int *Size, int z_length) {
    CT_REQUIRE(Display && R, "ct_FDKUI: null argument");
    UIGeom g;
    int s = ui_make(g, Xigamadomain, Gamadomain, BetaScanRange, betaStartAngle, MaxGama, Distance, Distance_s2d,
                    LGama, LBeta, LXigama, Size, z_length);
    if (s) return s;
    std::lock_guard<std::mutex> lk(g_ui_mutex);
    UIState &S = ui_state();
    const size_t nr = (size_t)LGama * LBeta * LXigama, nd = (size_t)Size[0] * Size[1] * z_length;
    if ((s = ui_upload(S, g, Xigamadomain, Gamadomain, BetaScanRange)) || (s = S.R.ensure(nr * sizeof(double))) ||
        (s = S.rcov.ensure(nr * sizeof(float))) || (s = S.disp.ensure(nd * sizeof(double))))
        return s;
    CT_CUDA(cudaMemcpy(S.R.ptr, R, nr * sizeof(double), cudaMemcpyHostToDevice), "H2D projections");
    if ((s = ui_filter(S, g, S.R.as<double>(), S.rcov.as<float>(), nullptr)) ||
        (s = ui_bp(S, g, S.rcov.as<float>(), S.disp.as<double>(), nullptr)))
        return s;
    CT_CUDA(cudaMemcpy(Display, S.disp.ptr, nd * sizeof(double), cudaMemcpyDeviceToHost), "D2H display");
    return CT_OK;
}

}  // extern "C"
