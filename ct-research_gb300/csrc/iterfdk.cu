// iterfdk.cu -- the IterativeFDK error slice (IterativeFDKerrCompute.cu:12-76).
//
// For image slice t and every (view beta, z, s) the reference sums, over the
// depth samples U along each ray of the view and every detector bin P,
//
//   0.5 LR^2 (pic[Zd][Yd][Xd] - pic[z][Yd][Xd]) sqrt(1 + (P/D)^2) G[fi] D / sqrt(D^2 + P^2) dU dP dBeta
//
// where (Xd, Yd) is the voxel of the ray point at depth U, Zd that point's
// slice as seen from (t, s, z), fi the filter tap of the voxel's detector
// offset and LR = D / (D - s_rot).  It launches one grid per (view, U) and
// adds into a float output, so each output is a float accumulator updated in
// double, U major and P minor.
//
// GB300 design.  One launch covers all views (in chunks) and every thread owns
// one output, looping U and P in the reference's order with the sum in a
// register and one store.  GB300's FP64 rate is 1/64 of its FP32 rate, so the
// per-iteration work is FP32:
//  * (Xd, Yd) depend on (view, U, P) only: a table per view chunk, computed
//    exactly in double by a small kernel.
//  * Zd (per U) and fi (per P) are computed in FP32 with an error bound; only
//    when the FP32 value falls within that bound of an integer is the
//    reference's double expression evaluated, so the indices are exact.
//  * The double term and the float-rounded double accumulation are carried
//    as float pairs: the term to ~2^-46 relative, and the sum rounded to
//    float from an error-free TwoSum (Knuth).  The result equals the
//    reference's unless a double term lands within ~2^-46 of a float rounding
//    boundary of the running sum.
#include <cmath>
#include <mutex>
#include <vector>

#include "devbuf.cuh"
#include "kernels.cuh"

namespace ct {

namespace {

struct IfdkGeom {
    int nt, ns, nz, nb, np, nu, lg, t;
    double ct, cs, cz;
    double res[3];
    double D, pint;
    float bint, du;
};

constexpr int kIfdkBlock = 128;

// (Xd, Yd) of the ray point at depth U[u] for bin P[p] of view v0 + blockIdx.z,
// as the column index yd * nt + xd, or -1 outside the slice (:46-59).
__global__ void iterfdk_table_kernel(const IfdkGeom g, const float2 *__restrict__ trig, const float *__restrict__ U,
                                     const double *__restrict__ P, int v0, int *__restrict__ tab) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int u = blockIdx.y;
    const int vl = blockIdx.z;
    if (p >= g.np) return;
    const float2 sc = trig[v0 + vl];   // (sin, cos) of the float angle
    const float uu = U[u];
    const float tr = (float)__ddiv_rn(__dmul_rn(P[p], __dsub_rn(g.D, (double)uu)), g.D);
    const float xr = __fsub_rn(__fmul_rn(tr, sc.y), __fmul_rn(uu, sc.x));
    const float yr = __fadd_rn(__fmul_rn(tr, sc.x), __fmul_rn(uu, sc.y));
    const double xf = floor(__ddiv_rn(__dadd_rn((double)xr, g.ct), g.res[0]));
    const double yf = floor(__ddiv_rn(__dadd_rn((double)yr, g.cs), g.res[1]));
    int idx = -1;
    if (xf >= 0.0 && xf < (double)g.nt && yf >= 0.0 && yf < (double)g.ns) idx = (int)yf * g.nt + (int)xf;
    tab[((long long)vl * g.nu + u) * g.np + p] = idx;
}

__device__ __forceinline__ bool near_int(float w, float fl, float marg) {
    return (w - fl < marg) || (fl + 1.0f - w < marg);
}

// One thread per (view, z, s) output of slice t.
__global__ void __launch_bounds__(kIfdkBlock, 12)
iterfdk_kernel(const IfdkGeom g, const float *__restrict__ pic, const int *__restrict__ tab, int v0,
               const float2 *__restrict__ trig, const float *__restrict__ U, const double *__restrict__ P,
               const float *__restrict__ Pf, const float2 *__restrict__ K, const float2 *__restrict__ Gff,
               float pmax, float *__restrict__ err) {
    extern __shared__ float2 sm2[];
    float2 *Ks = sm2;                                    // np
    float2 *Gs = sm2 + g.np;                             // lg
    float *Ps = reinterpret_cast<float *>(sm2 + g.np + g.lg);   // np
    for (int i = threadIdx.x; i < g.np; i += blockDim.x) {
        Ks[i] = K[i];
        Ps[i] = Pf[i];
    }
    for (int i = threadIdx.x; i < g.lg; i += blockDim.x) Gs[i] = Gff[i];
    __syncthreads();

    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    const int vl = blockIdx.z;
    const int v = v0 + vl;
    if (s >= g.ns) return;

    // voxel centre and its rotated coordinates in float, as the reference (:36-45)
    const float2 sc = trig[v];
    const float sb = sc.x, cb = sc.y;
    const float it = (float)__dsub_rn(__dmul_rn((double)g.t + 0.5, g.res[0]), g.ct);
    const float is = (float)__dsub_rn(__dmul_rn((double)s + 0.5, g.res[1]), g.cs);
    const float iz = (float)__dsub_rn(__dmul_rn((double)z + 0.5, g.res[2]), g.cz);
    const float dt = __fadd_rn(__fmul_rn(it, cb), __fmul_rn(is, sb));
    const float ds = __fadd_rn(__fmul_rn(-it, sb), __fmul_rn(is, cb));
    const float dz = iz;
    const double den = __dsub_rn(g.D, (double)ds);
    const float lr = (float)__ddiv_rn(g.D, den);
    const float a = __fmul_rn(dt, lr);
    const double c0 = __dmul_rn(0.5, __dmul_rn((double)lr, (double)lr));
    const float ch = (float)c0, cl = (float)(c0 - (double)ch);

    const float invden = (float)(1.0 / den);
    const float invres2 = (float)(1.0 / g.res[2]);
    const float czf = (float)g.cz;
    const float invp = (float)(1.0 / g.pint);
    // bound on |FP32 value - exact value| of the filter position (a - P) / dP
    const float qmarg = 2e-6f * (fabsf(a) + pmax) * invp + 1e-6f;

    const long long plane = (long long)g.nt * g.ns;
    const float *row2 = pic + (long long)z * plane;
    const int *tabv = tab + (long long)vl * g.nu * g.np;
    float acc = 0.0f;

    for (int u = 0; u < g.nu; ++u) {
        const float uu = U[u];
        // Zd of the ray point at depth U (:45, :55); float product as the reference
        const float m = __fmul_rn(__fsub_rn(ds, uu), dz);
        const float zq = m * invden;
        const float w = (dz + zq + czf) * invres2;
        float zfl = floorf(w);
        const float zmarg = 4e-6f * (fabsf(dz) + fabsf(zq) + czf) * invres2 + 1e-6f;
        if (near_int(w, zfl, zmarg)) {
            const float zx = (float)__dadd_rn((double)dz, __ddiv_rn((double)m, den));
            zfl = (float)floor(__ddiv_rn(__dadd_rn((double)zx, g.cz), g.res[2]));
        }
        if (!(zfl >= 0.0f && zfl < (float)g.nz)) continue;
        const int zi = (int)zfl;
        if (zi == z) continue;                       // both samples are the same voxel: every term is 0
        const float *row1 = pic + (long long)zi * plane;
        const int *tabu = tabv + (long long)u * g.np;
        for (int p = 0; p < g.np; ++p) {
            const int col = __ldg(tabu + p);
            if (col < 0) continue;
            // filter tap floor((a - P) / dP) + LP (:49)
            const float qf = (a - Ps[p]) * invp;
            float fl = floorf(qf);
            if (near_int(qf, fl, qmarg)) fl = (float)floor(__ddiv_rn(__dsub_rn((double)a, P[p]), g.pint));
            const int fi = (int)fl + g.np;
            if (fi < 0 || fi >= g.lg) continue;
            const float diff = __fsub_rn(__ldg(row1 + col), __ldg(row2 + col));
            if (diff == 0.0f) continue;              // a +-0 term leaves the float sum unchanged
            // term = c0 * diff * K[p] * G[fi] as a float pair
            const float2 kp = Ks[p], gg = Gs[fi];
            const float p1 = __fmul_rn(kp.x, gg.x);
            float e1 = fmaf(kp.x, gg.x, -p1);
            e1 = fmaf(kp.x, gg.y, e1);
            e1 = fmaf(kp.y, gg.x, e1);
            const float q1 = __fmul_rn(p1, ch);
            float f1 = fmaf(p1, ch, -q1);
            f1 = fmaf(p1, cl, f1);
            f1 = fmaf(e1, ch, f1);
            const float r = __fmul_rn(q1, diff);
            float g1 = fmaf(q1, diff, -r);
            g1 = fmaf(f1, diff, g1);
            // acc = float(acc + r + g1): TwoSum of (acc, r), then the low parts
            const float sum = __fadd_rn(acc, r);
            const float bb = __fsub_rn(sum, acc);
            const float ee = __fadd_rn(__fsub_rn(acc, __fsub_rn(sum, bb)), __fsub_rn(r, bb));
            acc = __fadd_rn(sum, __fadd_rn(ee, g1));
        }
    }
    err[((long long)v * g.nz + z) * g.ns + s] = acc;
}

struct IfdkState {
    DevBuf trig, U, P, Pf, K, G, tab, pic, err;
    void release() {
        for (DevBuf *b : {&trig, &U, &P, &Pf, &K, &G, &tab, &pic, &err}) b->release();
    }
};
std::mutex g_ifdk_mutex;
IfdkState &ifdk_state() {
    static IfdkState st;
    return st;
}

void to_pair(double d, float2 &f) {
    f.x = (float)d;
    f.y = (float)(d - (double)f.x);
}

int iterfdk_run(const IfdkGeom &g, const float *d_pic, float *d_err, const float *beta, const float *U,
                const double *P, const double *G, cudaStream_t st) {
    CT_REQUIRE(g.nt > 0 && g.ns > 0 && g.nz > 0, "IterativeFDKerrCompute: image sizes must be positive");
    CT_REQUIRE((long long)g.nt * g.ns * g.nz < (1LL << 31), "IterativeFDKerrCompute: image too large");
    CT_REQUIRE(g.nb > 0 && g.nb <= 65535 && g.nu > 0 && g.np > 0 && g.lg > 0,
               "IterativeFDKerrCompute: LBeta in [1, 65535], LU, LP, LG positive");
    CT_REQUIRE(g.nz <= 65535, "IterativeFDKerrCompute: z_length at most 65535");
    CT_REQUIRE(g.t >= 0 && g.t < g.nt, "IterativeFDKerrCompute: slice index t out of range");
    CT_REQUIRE(g.D > 0 && g.pint > 0 && g.res[0] > 0 && g.res[1] > 0 && g.res[2] > 0,
               "IterativeFDKerrCompute: Distance, PInt and the resolution must be positive");
    CT_REQUIRE(beta && U && P && G, "IterativeFDKerrCompute: null domain");
    const size_t smem = sizeof(float2) * ((size_t)g.np + g.lg) + sizeof(float) * g.np;
    CT_REQUIRE(smem <= 200 * 1024, "IterativeFDKerrCompute: LP and LG too large for shared memory");
    for (int i = 0; i < g.np; ++i) CT_REQUIRE(std::isfinite(P[i]), "IterativeFDKerrCompute: non-finite Pdomain");
    for (int i = 0; i < g.nu; ++i) CT_REQUIRE(std::isfinite(U[i]), "IterativeFDKerrCompute: non-finite Udomain");
    for (int i = 0; i < g.nb; ++i)
        CT_REQUIRE(std::isfinite(beta[i]), "IterativeFDKerrCompute: non-finite BetaScanRange");

    IfdkState &S = ifdk_state();
    // host tables: sin/cos of the float angles (single-precision overloads, as
    // the reference's cos(Beta) of a float), the P-dependent factor
    // K = sqrt(1 + (P/D)^2) D / sqrt(D^2 + P^2) dU dP dBeta, and G as float pairs
    std::vector<float2> tr(g.nb), kk(g.np), gg(g.lg);
    std::vector<float> pf(g.np);
    float pmax = 0.0f;
    for (int v = 0; v < g.nb; ++v) tr[v] = make_float2(sinf(beta[v]), cosf(beta[v]));
    for (int p = 0; p < g.np; ++p) {
        const double pv = P[p];
        const double k = std::sqrt(1 + 1.0 * (pv / g.D) * (pv / g.D)) * g.D / std::sqrt(1.0 * g.D * g.D + pv * pv) *
                         (double)g.du * g.pint * (double)g.bint;
        to_pair(k, kk[p]);
        pf[p] = (float)pv;
        pmax = std::max(pmax, std::fabs(pf[p]));
    }
    for (int i = 0; i < g.lg; ++i) to_pair(G[i], gg[i]);
    int s;
    if ((s = upload(S.trig, tr.data(), tr.size())) || (s = upload(S.U, U, (size_t)g.nu)) ||
        (s = upload(S.P, P, (size_t)g.np)) || (s = upload(S.Pf, pf.data(), pf.size())) ||
        (s = upload(S.K, kk.data(), kk.size())) || (s = upload(S.G, gg.data(), gg.size())))
        return s;

    // (Xd, Yd) tables for chunks of views, at most 256 MiB at a time
    const size_t per_view = sizeof(int) * (size_t)g.nu * g.np;
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>(g.nb, (size_t(256) << 20) / per_view));
    if ((s = S.tab.ensure(per_view * chunk))) return s;
    if (smem > 48 * 1024)
        CT_CUDA(cudaFuncSetAttribute(iterfdk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "iterfdk smem attribute");
    CT_REQUIRE(g.nu <= 65535, "IterativeFDKerrCompute: LU at most 65535");
    for (int v0 = 0; v0 < g.nb; v0 += chunk) {
        const int nv = std::min(chunk, g.nb - v0);
        dim3 tg((g.np + 127) / 128, g.nu, nv);
        iterfdk_table_kernel<<<tg, 128, 0, st>>>(g, S.trig.as<float2>(), S.U.as<float>(), S.P.as<double>(), v0,
                                                 S.tab.as<int>());
        CT_LAUNCH_CHECK("iterfdk_table_kernel");
        dim3 grid((g.ns + kIfdkBlock - 1) / kIfdkBlock, g.nz, nv);
        iterfdk_kernel<<<grid, kIfdkBlock, smem, st>>>(g, d_pic, S.tab.as<int>(), v0, S.trig.as<float2>(),
                                                       S.U.as<float>(), S.P.as<double>(), S.Pf.as<float>(),
                                                       S.K.as<float2>(), S.G.as<float2>(), pmax, d_err);
        CT_LAUNCH_CHECK("iterfdk_kernel");
    }
    return CT_OK;
}

}  // namespace

// Free the device buffers the drop-in keeps between calls (ct_dropin_release).
void iterfdk_release_cache() {
    std::lock_guard<std::mutex> lk(g_ifdk_mutex);
    ifdk_state().release();
}

}  // namespace ct

using namespace ct;

extern "C" {

int ct_iterfdk_err(const float *d_Pic, float *d_Err, const float *BetaScanRange, int LBeta, const float *Udomain,
                   int LU, const double *Pdomain, int LP, const double *G, int LG, const double *Size, int t_length,
                   int s_length, int z_length, double Distance, int t, void *stream) {
    CT_REQUIRE(d_Pic && d_Err && Size, "ct_iterfdk_err: null argument");
    CT_REQUIRE(LBeta >= 2 && LU >= 2 && LP >= 2, "ct_iterfdk_err: at least 2 views, U samples and bins");
    CT_REQUIRE(t_length > 0 && s_length > 0 && z_length > 0, "ct_iterfdk_err: image sizes must be positive");
    CT_REQUIRE(BetaScanRange && Udomain && Pdomain && G, "ct_iterfdk_err: null domain");
    // argument derivation of the MEX gateway (IterativeFDKerrCompute.cpp:10-31)
    IfdkGeom g{};
    g.nt = t_length; g.ns = s_length; g.nz = z_length;
    g.nb = LBeta; g.np = LP; g.nu = LU; g.lg = LG; g.t = t;
    g.ct = Size[0] / 2; g.cs = Size[1] / 2; g.cz = Size[2] / 2;
    g.res[0] = Size[0] / t_length; g.res[1] = Size[1] / s_length; g.res[2] = Size[2] / z_length;
    g.D = Distance;
    g.bint = std::fabs(BetaScanRange[1] - BetaScanRange[0]);
    g.du = std::fabs(Udomain[1] - Udomain[0]);
    g.pint = std::fabs(Pdomain[1] - Pdomain[0]);
    std::lock_guard<std::mutex> lk(g_ifdk_mutex);
    return iterfdk_run(g, d_Pic, d_Err, BetaScanRange, Udomain, Pdomain, G, as_stream(stream));
}

int ct_IterativeFDKerrCompute(const float *Pic, float *ErrorSlicecuda, const float *BetaScanRange,
                              const float *Udomain, const double *Pdomain, const double *G, const double *Size,
                              int t_length, int s_length, int z_length, double Center_t, double Center_s,
                              double Center_z, int LBeta, int LP, int LU, int LG, double Distance,
                              const double *resolution2, int t, float BetaScanInt, float dU, double PInt) {
    CT_REQUIRE(Pic && ErrorSlicecuda && resolution2 && Size, "ct_IterativeFDKerrCompute: null argument");
    IfdkGeom g{};
    g.nt = t_length; g.ns = s_length; g.nz = z_length;
    g.nb = LBeta; g.np = LP; g.nu = LU; g.lg = LG; g.t = t;
    g.ct = Center_t; g.cs = Center_s; g.cz = Center_z;
    for (int a = 0; a < 3; ++a) g.res[a] = resolution2[a];
    g.D = Distance;
    g.bint = BetaScanInt;
    g.du = dU;
    g.pint = PInt;
    std::lock_guard<std::mutex> lk(g_ifdk_mutex);
    IfdkState &S = ifdk_state();
    CT_REQUIRE(t_length > 0 && s_length > 0 && z_length > 0 && LBeta > 0,
               "ct_IterativeFDKerrCompute: sizes must be positive");
    const size_t nv = (size_t)t_length * s_length * z_length, ne = (size_t)LBeta * s_length * z_length;
    int s;
    if ((s = S.pic.ensure(nv * sizeof(float))) || (s = S.err.ensure(ne * sizeof(float)))) return s;
    CT_CUDA(cudaMemcpy(S.pic.ptr, Pic, nv * sizeof(float), cudaMemcpyHostToDevice), "H2D image");
    if ((s = iterfdk_run(g, S.pic.as<float>(), S.err.as<float>(), BetaScanRange, Udomain, Pdomain, G, nullptr)))
        return s;
    CT_CUDA(cudaMemcpy(ErrorSlicecuda, S.err.ptr, ne * sizeof(float), cudaMemcpyDeviceToHost), "D2H error slice");
    return CT_OK;
}

}  // extern "C"
