// cone_bp.cu -- voxel-driven cone-beam backprojection for sm_103a.
//
// Two weightings of the same bilinear detector interpolation:
//  * CHORD (Backprojection3D.cu:8-291): each voxel-view adds
//      bilinear(R) * 2 * |entry - centre|, the chord of the source->voxel-centre
//      line through the voxel.  For a line through the centre the chord is
//      2 * min_a(h_a / |d_a|) * |d| (h = half voxel, d = centre - source),
//      which equals the reference's low-face construction.
//  * FDK (FDK.cu:50-126): bilinear(filtered R) * LR^2 * dbeta, where
//      LR = D / (D - dect_s); in STICKY mode a voxel whose projection leaves
//      the detector re-adds the last in-range value of its column, as the
//      reference does because it never resets Display_pBeta (:73, :100-123).
//
// Layout: each view's projection is first repacked into 2x2 quads,
//   Q[v][x][p] = (R[x][p], R[x][p+1], R[x+1][p], R[x+1][p+1]),
// so the four bilinear taps of a voxel-view are one aligned 16-byte load.
// This trades HBM capacity (4x the sinogram, 2.3 GB at 360x512x768) for a
// quarter of the load instructions on a load-issue-bound kernel.
//
// Interpolation follows the reference's discontinuous index rule exactly:
// column floor(|P - P0| / PInt) and row floor(|xi - xi0| / XigamaInt), with
// PInt and XigamaInt the spacing of the first two (float) samples and the
// weights |P - P[i]| / PInt, |xi - xi[j]| / XigamaInt from the actual sample
// values (Backprojection3D.cu:73-87).  Float samples drift from that implied
// grid (by ~1e-3 mm across a 512-row detector), so an index one off changes a
// weight by up to ~4e-3: the column coordinate is computed per column-view in
// float-float (ffloat.cuh), and the row quotient, affine in z, is stepped in
// 64-bit fixed point with a per-row table of the samples' own quotients.
//
// Threads own one (t, s) column and ZC consecutive z; the view loop runs
// inside the thread with the ZC sums in registers, and each voxel is written
// once at the end (no atomics, deterministic).  The fused SIRT variant writes
// clamp(x + lambda * bp / (colsum + eps), lo, hi) instead of bp.
#include <type_traits>

#include "cone_geom.cuh"
#include "ffloat.cuh"

namespace ct {

namespace {

#ifndef CT_BP_ZC
#define CT_BP_ZC 32
#endif
// Blocks per SM the register allocation aims at.  Chord weighting: 4 (128
// registers, a few bytes spilled on the out-of-line tie paths) measured 71.8 ms
// at 512^3 / 360 views against 73.0 ms at 3 (168 registers) and 85.7 ms at 2.
// FDK weighting at 256^3 / 360 views: 8.08 ms at 3, 8.20 at 4, 12.5 at 5.
#ifndef CT_BP_MINB
#define CT_BP_MINB 4
#endif
#ifndef CT_BP_MINB_FDK
#define CT_BP_MINB_FDK 3
#endif
constexpr int BP_BX = 32;          // t per block
// s rows per block (warps of 32 t).  Chord weighting at 512^3 / 360 views,
// 128 registers: 4 rows 54.6 ms, 2 rows 55.1, 1 row 56.6, 8 rows 57.4.
#ifndef CT_BP_BY
#define CT_BP_BY 4
#endif
constexpr int BP_BY = CT_BP_BY;    // s per block
constexpr int BP_ZC = CT_BP_ZC;    // z per thread (register accumulators)
static_assert(BP_ZC >= 1 && BP_ZC <= 64, "cone_bp: 1 to 64 z per thread");
// bit k: z0 + k of the thread takes the view
using zmask_t = std::conditional_t<(BP_ZC > 32), unsigned long long, unsigned>;
constexpr zmask_t kZAll = BP_ZC >= 8 * (int)sizeof(zmask_t) ? ~zmask_t(0) : ((zmask_t(1) << BP_ZC) - 1);

// Quads of nb views; R points at the first of them.
__global__ void __launch_bounds__(256)
pack_quads_kernel(const float *__restrict__ R, float4 *__restrict__ Q, int nb, int nx, int np) {
    const long long n = (long long)nb * nx * np;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(i % np);
        const long long rv = i / np;
        const int x = (int)(rv % nx);
        const bool pr = p + 1 < np, xr = x + 1 < nx;
        float4 q;
        q.x = R[i];
        q.y = pr ? R[i + 1] : 0.0f;
        q.z = xr ? R[i + np] : 0.0f;
        q.w = (pr && xr) ? R[i + np + 1] : 0.0f;
        Q[i] = q;
    }
}

enum { W_CHORD = 0, W_FDK_ZERO = 1, W_FDK_STICKY = 2 };

// FP64 re-evaluation of the reference's detector-range tests for one column
// and view (Backprojection3D.cu:31-43 and :66-71, FDK.cu:80-100):
// P in [minP, maxP) and xi(z) in [minXigama, maxXigama).  Used only when the
// FP32 decision lies within rounding distance of a detector edge; it matters
// most for the sticky FDK value, which is taken at the last in-range z.
__device__ __noinline__ void range_fp64(const ConeGeom &g, int ti, int si, double sb, double cb, bool &pin,
                                        int &zlo, int &zhi) {
    const double it = (ti + 0.5) * g.res[0] - 0.5 * g.size[0];
    const double is = (si + 0.5) * g.res[1] - 0.5 * g.size[1];
    const double dect_t = it * cb + is * sb;
    const double dect_s = -it * sb + is * cb;
    const double lr = g.D / (g.D - dect_s);
    const double P = dect_t * lr;
    pin = (P >= (double)g.minp) && (P < (double)g.maxp);
    const double rz = g.res[2], cz = 0.5 * g.size[2];
    const double mnx = g.minx, mxx = g.maxx;
    int lo = min(max(zlo, 0), g.nz);
    while (lo > 0 && ((lo - 1 + 0.5) * rz - cz) * lr >= mnx) --lo;
    while (lo < g.nz && !(((lo + 0.5) * rz - cz) * lr >= mnx)) ++lo;
    int hi = min(max(zhi, -1), g.nz - 1);
    while (hi + 1 < g.nz && ((hi + 1 + 0.5) * rz - cz) * lr < mxx) ++hi;
    while (hi >= 0 && !(((hi + 0.5) * rz - cz) * lr < mxx)) --hi;
    zlo = lo;
    zhi = hi;
}

// The reference's chord construction for one voxel-view in FP64
// (Backprojection3D.cu:243-281): false when no low face of the voxel holds the
// entry point of the source->centre line, in which case the reference returns
// and the rest of the column gets nothing from this view.  Each operation is
// rounded separately (no FMA contraction), as the host build of that code is.
__device__ __noinline__ bool chord_entry_found(const ConeGeom &g, int ti, int si, int zi, double sb, double cb) {
    const double EPS = 1e-15;
    const double ct = g.size[0] / 2, cs = g.size[1] / 2, cz = g.size[2] / 2;
    const double rt = g.res[0], rs = g.res[1], rz = g.res[2];
    const double it = __dsub_rn(__dmul_rn(ti + 0.5, rt), ct);
    const double is = __dsub_rn(__dmul_rn(si + 0.5, rs), cs);
    const double iz = __dsub_rn(__dmul_rn(zi + 0.5, rz), cz);
    const double st = __dsub_rn(ct, __dmul_rn(g.D, sb)), ss = __dadd_rn(cs, __dmul_rn(g.D, cb)), sz = cz;
    const double et = __dadd_rn(it, ct), es = __dadd_rn(is, cs), ez = __dadd_rn(iz, cz);
    const double tlo = __dmul_rn((double)ti, rt), thi = __dmul_rn((double)(ti + 1), rt);
    const double slo = __dmul_rn((double)si, rs), shi = __dmul_rn((double)(si + 1), rs);
    const double zlo = __dmul_rn((double)zi, rz), zhi = __dmul_rn((double)(zi + 1), rz);
    const double dt = __dsub_rn(et, st), ds = __dsub_rn(es, ss), dz = __dsub_rn(ez, sz);
    const double dte = __dadd_rn(dt, EPS), dse = __dadd_rn(ds, EPS), dze = __dadd_rn(dz, EPS);
    auto hit = [](double a0, double off, double d1, double de) {   // a0 + off * d1 / de
        return __dadd_rn(a0, __ddiv_rn(__dmul_rn(off, d1), de));
    };
    const double tlo_s = hit(ss, __dsub_rn(tlo, st), ds, dte), tlo_z = hit(sz, __dsub_rn(tlo, st), dz, dte);
    if (tlo_s >= slo && tlo_s <= shi && tlo_z >= zlo && tlo_z <= zhi) return true;
    const double slo_t = hit(st, __dsub_rn(slo, ss), dt, dse), slo_z = hit(sz, __dsub_rn(slo, ss), dz, dse);
    if (slo_t >= tlo && slo_t <= thi && slo_z >= zlo && slo_z <= zhi) return true;
    const double zlo_t = hit(st, __dsub_rn(zlo, sz), dt, dze), zlo_s = hit(ss, __dsub_rn(zlo, sz), ds, dze);
    return zlo_t >= tlo && zlo_t <= thi && zlo_s >= slo && zlo_s <= shi;
}

// The in-plane parts of the reference's first two face tests, which do not
// depend on z (Backprojection3D.cu:262-270): the line from the source to the
// voxel centre crosses the low t face within the voxel's s bounds, or the low
// s face within its t bounds.  Same operations as chord_entry_found.
__device__ __noinline__ bool chord_side_found(const ConeGeom &g, int ti, int si, double sb, double cb) {
    const double EPS = 1e-15;
    const double ct = g.size[0] / 2, cs = g.size[1] / 2;
    const double rt = g.res[0], rs = g.res[1];
    const double it = __dsub_rn(__dmul_rn(ti + 0.5, rt), ct);
    const double is = __dsub_rn(__dmul_rn(si + 0.5, rs), cs);
    const double st = __dsub_rn(ct, __dmul_rn(g.D, sb)), ss = __dadd_rn(cs, __dmul_rn(g.D, cb));
    const double et = __dadd_rn(it, ct), es = __dadd_rn(is, cs);
    const double tlo = __dmul_rn((double)ti, rt), thi = __dmul_rn((double)(ti + 1), rt);
    const double slo = __dmul_rn((double)si, rs), shi = __dmul_rn((double)(si + 1), rs);
    const double dt = __dsub_rn(et, st), ds = __dsub_rn(es, ss);
    const double dte = __dadd_rn(dt, EPS), dse = __dadd_rn(ds, EPS);
    const double tlo_s = __dadd_rn(ss, __ddiv_rn(__dmul_rn(__dsub_rn(tlo, st), ds), dte));
    if (tlo_s >= slo && tlo_s <= shi) return true;
    const double slo_t = __dadd_rn(st, __ddiv_rn(__dmul_rn(__dsub_rn(slo, ss), dt), dse));
    return slo_t >= tlo && slo_t <= thi;
}

// Last z of a column that a view reaches when the source->centre line passes
// near a voxel edge (two faces' chord parameters tie within FP32 margins): the
// reference's FP64 face tests may then all fail at some z, and it returns,
// dropping that z and all above it for this view.  Called rarely (symmetric
// geometries); kept out of line so the hot loop keeps its registers.
__device__ __noinline__ int chord_end_z(const ConeGeom &g, int ti, int si, double sb, double cb, int zlo, int zhi,
                                        bool tie_ts, float ztie, float mmax, bool tz1, float zc1, bool tz2, float zc2) {
    const float rz = (float)g.res[2];
    const float hz = 0.5f * rz;
    const float x_base = (float)(0.5 * g.res[2] - 0.5 * g.size[2]);
    int zab = 0x7fffffff;
    // A face crossing lies |iz| * h_a / |d_a| off the voxel centre in z.  Where
    // that stays below hz (10% margin) at every z of the column, the z parts of
    // the t and s face tests pass everywhere and their z-independent in-plane
    // parts decide every z at once; near the diagonal views this replaces a
    // per-z FP64 replay of the whole column.
    const float izc = fmaxf(fabsf(fmaf((float)max(zlo, 0), rz, x_base)), fabsf(fmaf((float)min(zhi, g.nz - 1), rz, x_base)));
    if (tie_ts && izc * mmax < 0.9f * hz && chord_side_found(g, ti, si, sb, cb)) tie_ts = false;
    if (tie_ts) {
        // t/s faces limit the chord where |iz| <= ztie: check those z in order
        for (int z = max(zlo, 0); z <= min(zhi, g.nz - 1); ++z) {
            const float iz = fmaf((float)z, rz, x_base);
            if (fabsf(iz) > ztie * (1.0f + 1e-5f)) continue;
            if (!chord_entry_found(g, ti, si, z, sb, cb)) { zab = z; break; }
        }
    }
    const int r1 = (int)rintf(zc1), r2 = (int)rintf(zc2);
    if (tz1 && r1 >= zlo && r1 <= zhi && r1 < zab && !chord_entry_found(g, ti, si, r1, sb, cb)) zab = r1;
    if (tz2 && r2 >= zlo && r2 <= zhi && r2 < zab && !chord_entry_found(g, ti, si, r2, sb, cb)) zab = r2;
    return min(zhi, zab - 1);
}

// Views [v0, v0 + nv) of the scan, whose quads Q holds (Q[0] = view v0).
// Each voxel's sum b = (sum over these views) + prev (when prev is given) is
// written to out, or with UPDATE folded into out = vol as
// clamp(vol + lambda * b / (colsum + eps), lo, hi).
template <int WMODE, bool UPDATE>
__global__ void __launch_bounds__(BP_BX * BP_BY, WMODE == W_CHORD ? CT_BP_MINB : CT_BP_MINB_FDK)
cone_bp_kernel(const ConeGeom g, const float4 *__restrict__ Q, int v0, int nv, const float *prev, float *out,
               const float *__restrict__ colsum, float eps, float lambda, float lo, float hi, int zt0) {
    // the row table (x - q(xi[x]), q(xi[x+1]) - x) of ConeGeom::xtab
    extern __shared__ float2 xtab[];
    const int tid = threadIdx.x + BP_BX * threadIdx.y;
    for (int x = tid; x < g.nx - 1; x += BP_BX * BP_BY) xtab[x] = g.xtab[x];
    __syncthreads();

    const int ti = blockIdx.x * BP_BX + threadIdx.x;
    const int si = blockIdx.y * BP_BY + threadIdx.y;
    const int z0 = (zt0 + (int)blockIdx.z) * BP_ZC;
    if (ti >= g.nt || si >= g.ns) return;

    // voxel-centre coordinates relative to the rotation centre, exact to ~2^-48
    const ff it2 = ff_from((ti + 0.5) * g.res[0] - 0.5 * g.size[0]);
    const ff is2 = ff_from((si + 0.5) * g.res[1] - 0.5 * g.size[1]);
    const ff iz02 = ff_from((z0 + 0.5) * g.res[2] - 0.5 * g.size[2]);
    const ff D2 = {g.bp_D.x, g.bp_D.y};
    const ff ipint2 = {g.bp_ipint.x, g.bp_ipint.y};
    const ff xq2 = {g.bp_xq.x, g.bp_xq.y};   // row quotient per mm of xi
    const ff p02 = {g.p0, 0.0f};
    // the view-independent factors of the row quotient: (iz lr - xi0) xq = lr (iz xq) - xi0 xq
    const ff rzxq2 = {g.bp_rzxq.x, g.bp_rzxq.y}, iz0xq2 = ff_mul(iz02, xq2), x0xq2 = {g.bp_x0xq.x, g.bp_x0xq.y};

    const float rz = g.bp_rz;
    const float it = it2.hi, is = is2.hi;
    const float D = g.bp_Df;
    const float ipint = g.bp_ipintf;
    const float ht = g.bp_ht, hs = g.bp_hs, hz = g.bp_hz;
    const float czf = g.bp_czf;
    const float x_base = g.bp_xbase;   // iz at z = 0
    const float iz0 = iz02.hi;         // iz of this thread's first z
    // largest |iz| of the thread's z range: decides whether z faces can limit the chord
    const float izmax = fmaxf(fabsf(iz0), fabsf(fmaf((float)(BP_ZC - 1), rz, iz0)));
    const float iz_vol = fabsf(x_base);   // largest |iz| of the volume
    const float irz = g.bp_irz, iD = g.bp_iD;
    const long long vstride = (long long)g.nx * g.np;

    float acc[BP_ZC];
#pragma unroll
    for (int k = 0; k < BP_ZC; ++k) acc[k] = 0.0f;

    for (int v = v0; v < v0 + nv; ++v) {
        const float2 tr = g.trigf[v];   // float (sin, cos): no FP64 conversion in the loop
        const float sb = tr.x, cb = tr.y;
        // detector coordinates of the column in float-float: the reference's
        // FP64 dect_t, dect_s, LengthRatio = D / (D - dect_s) and P = dect_t * LR
        // (Backprojection3D.cu:28-37)
        const ff dt2 = ff_add(ff_mul_f(it2, cb), ff_mul_f(is2, sb));
        const ff ds2 = ff_sub(ff_mul_f(is2, cb), ff_mul_f(it2, sb));
        const ff den2 = ff_sub(D2, ds2);
        const ff lr2 = ff_div_r(D2, den2, __fdividef(1.0f, den2.hi));
        const ff P2 = ff_mul(dt2, lr2);
        const float dect_s = ds2.hi, lr = lr2.hi, P = P2.hi;
        bool pin = P >= g.minp && P < g.maxp;
        // xi(z) = iz(z) * lr; detector rows in range for z in [zlo, zhi]
        // xi(z) >= minx  <=>  z >= (minx / lr - x_base) / rz, with 1/lr = (D - dect_s) / D
        const float ilr = (D - dect_s) * iD;
        const float zlo_f = fmaf(g.minx, ilr, -x_base) * irz, zhi_f = fmaf(g.maxx, ilr, -x_base) * irz;
        int zlo = (int)ceilf(zlo_f);             // first z with xi >= minx
        int zhi = (int)ceilf(zhi_f) - 1;         // last z with xi < maxx
        // FP32 rounding is ~3e-5 in z units: re-decide in FP64 near an edge
        const bool near_edge = fabsf(zlo_f - rintf(zlo_f)) < 2.5e-4f || fabsf(zhi_f - rintf(zhi_f)) < 2.5e-4f ||
                               fabsf(P - g.minp) < 2e-4f || fabsf(P - g.maxp) < 2e-4f;
        if (near_edge) range_fp64(g, ti, si, g.trig[v].x, g.trig[v].y, pin, zlo, zhi);
        if (!pin) continue;   // whole column off the detector for this view
        if (WMODE == W_FDK_STICKY && zhi < zlo) continue;
        // detector column floor(|P - P0| / PInt) and weights |P - P[p1]| / PInt,
        // |P[p1+1] - P| / PInt from the domain values (Backprojection3D.cu:73-83)
        const int p1 = min(max(ff_floor(ff_mul(ff_abs(ff_sub(P2, p02)), ipint2)), 0), g.np - 2);
        const float pa = __ldg(g.P + p1), pb = __ldg(g.P + p1 + 1);
        const float wq1 = fabsf(__fadd_rn(__fsub_rn(P2.hi, pa), P2.lo)) * ipint;   // weight of column p1+1
        const float wq0 = fabsf(__fsub_rn(__fsub_rn(pb, P2.hi), P2.lo)) * ipint;   // weight of column p1
        const float4 *Qv = Q + (long long)(v - v0) * vstride + p1;
        // row quotient q(z) = |xi(z) - xi[0]| / XigamaInt, affine in z, as 64-bit
        // fixed point (32 fraction bits): floor and weights follow the
        // reference's FP64 values except within ~1e-8 of a row boundary
        const long long dqf = ff_fixed32(ff_mul(rzxq2, lr2));
        long long r = ff_fixed32(ff_sub(ff_mul(iz0xq2, lr2), x0xq2));

        float wv = 1.0f, mts = 0.0f, qq = 0.0f;
        int zend = zhi;           // last z that receives this view's value
        bool zlimit = false;      // some z face limits a chord in this thread's range
        if (WMODE == W_CHORD) {
            const float dt = it + D * sb, ds = is - D * cb;
            // approximate reciprocals (a few ulp): the chord factor needs ~1e-7, and the
            // tie tests below have margins of 1e-5
            const float mt = __fdividef(ht, fabsf(dt)), ms = __fdividef(hs, fabsf(ds));
            mts = fminf(mt, ms);
            qq = fmaf(dt, dt, ds * ds);
            zlimit = izmax * mts > hz;
            // The source->centre line passes near a voxel edge when two faces'
            // parameters tie; only then can the reference's FP64 face tests all
            // fail and end the column.  Ties are found in FP32 with a wide margin
            // and decided in FP64 (chord_end_z).  A z face can tie only where
            // |iz| reaches hz / mts, i.e. when the volume is tall enough.
            const bool tie_ts = fabsf(mt - ms) <= 1e-5f * mts;
            bool tz1 = false, tz2 = false;
            float zc1 = 0.0f, zc2 = 0.0f;
            if (iz_vol * mts > 0.999f * hz) {
                const float ztie = __fdividef(hz, mts);   // |iz| where the z faces tie with mts
                zc1 = (czf + ztie) * irz - 0.5f;
                zc2 = (czf - ztie) * irz - 0.5f;
                tz1 = fabsf(zc1 - rintf(zc1)) < 1e-3f;
                tz2 = fabsf(zc2 - rintf(zc2)) < 1e-3f;
            }
            if (tie_ts || tz1 || tz2)
                zend = chord_end_z(g, ti, si, g.trig[v].x, g.trig[v].y, zlo, zhi, tie_ts, hz / mts, fmaxf(mt, ms), tz1, zc1, tz2,
                                   zc2);
        } else {
            wv = lr * lr * g.bint;
        }
        // the chord factor 2 * mts (or the FDK weight) folds into the detector-column
        // weights; where a z face can limit the chord the factor becomes
        // min(1, hz / (|iz| mts))
        const float c0 = (WMODE == W_CHORD) ? 2.0f * mts : wv;
        const float wa = wq0 * c0, wb = wq1 * c0;
        // sticky FDK: z above zhi re-add the value at zhi (the row quotient stops there)
        const int kz = zhi - z0;
        if (WMODE == W_FDK_STICKY && kz < 0) r += (long long)kz * dqf;
        // z of this thread that take this view, as a bit mask over k
        const int klo = max(zlo - z0, 0), khi = min(((WMODE == W_FDK_STICKY) ? 0x7fff : zend) - z0, BP_ZC - 1);
        const zmask_t inmask = (klo > khi) ? zmask_t(0)
                               : ((khi >= BP_ZC - 1 ? kZAll : ((zmask_t(2) << khi) - 1)) & ~((zmask_t(1) << klo) - 1));
        // Fast path: every z of the thread takes the view, no z face limits the
        // chord, and the chord length |d| = sqrt(qq + iz^2) is the quadratic in k
        // about the thread's middle z (relative error below 1e-7, bounded by the
        // third-order term |iz| h^3 / (2 |d|^4), h the half span of the 32 z).
        const float kc = 0.5f * (BP_ZC - 1);
        const float izc = fmaf(kc, rz, iz0);
        const float lc2 = fmaf(izc, izc, qq);
        const float ilc = rsqrtf(lc2), lc = lc2 * ilc;
        const float l1 = izc * rz * ilc, l2 = 0.5f * qq * rz * rz * ilc * ilc * ilc;
        const float hspan = kc * rz;
        // more than 32 z: a cubic term, whose error (fourth order) is below
        // h^4 / (2 |d|^4)
        const float l3 = (BP_ZC > 32) ? -0.5f * qq * izc * rz * rz * rz * ilc * ilc * ilc * ilc * ilc : 0.0f;
        const float hl = hspan * ilc;
        const bool quad_ok = WMODE != W_CHORD ||
                             ((BP_ZC > 32) ? 0.5f * hl * hl * hl * hl < 2e-7f
                                           : fabsf(izc) * hspan * hspan * hspan * ilc * ilc * ilc * ilc < 2e-7f);
        const bool fast = inmask == kZAll && !zlimit && quad_ok &&
                          !(WMODE == W_FDK_STICKY && kz < BP_ZC - 1);
        auto body = [&](auto fastpath) {
            constexpr bool FAST = decltype(fastpath)::value;
            long long rk = r;
#pragma unroll
            for (int k = 0; k < BP_ZC; ++k) {
                if (k > 0) rk += (!FAST && WMODE == W_FDK_STICKY && k > kz) ? 0LL : dqf;
                // an index outside [0, nx-2] (z off the detector, or a negative
                // quotient wrapped by the unsigned compare) is clamped for the read only
                const unsigned x1 = min((unsigned)(int)(rk >> 32), (unsigned)(g.nx - 2));
                const float fr = __uint2float_rn((unsigned)rk);          // fraction * 2^32
                const float2 xt = xtab[x1];
                const float w1 = fmaf(fr, 2.3283064365386963e-10f, xt.x);    // |w1|: weight of row x1+1
                const float w0 = fmaf(fr, -2.3283064365386963e-10f, xt.y);   // |w0|: weight of row x1
                const float4 q = __ldg(Qv + (int)x1 * g.np);
                const float top = fmaf(wa, q.x, wb * q.y);
                const float bot = fmaf(wa, q.z, wb * q.w);
                const float val = fmaf(fabsf(w0), top, fabsf(w1) * bot);
                float w;
                if (WMODE == W_CHORD) {
                    // chord 2 * min(h_a / |d_a|) * |d|, d = (dt, ds, iz); the factor
                    // min(1, hz / (|iz| mts)) is 1 where no z face limits the chord
                    if (FAST) {
                        const float dk = (float)k - kc;
                        if constexpr (BP_ZC > 32) w = fmaf(dk, fmaf(dk, fmaf(dk, l3, l2), l1), lc);
                        else w = fmaf(dk, fmaf(dk, l2, l1), lc);
                    } else {
                        const float iz = fmaf((float)k, rz, iz0);
                        const float d2 = fmaf(iz, iz, qq);
                        w = fminf(1.0f, hz / (fabsf(iz) * mts)) * (d2 * rsqrtf(d2));
                    }
                } else {
                    w = 1.0f;
                }
                if (FAST) {
                    acc[k] = fmaf(val, w, acc[k]);
                } else {
                    const bool in = (inmask >> k) & 1;
                    acc[k] = in ? fmaf(val, w, acc[k]) : acc[k];
                }
            }
        };
        if (fast) body(std::true_type{});
        else body(std::false_type{});
    }
#pragma unroll
    for (int k = 0; k < BP_ZC; ++k) {
        const int z = z0 + k;
        if (z < g.nz) {
            const long long o = ((long long)z * g.ns + si) * g.nt + ti;
            const float b = prev ? acc[k] + prev[o] : acc[k];
            if (UPDATE) {
                const float x = out[o] + lambda * b / (colsum[o] + eps);
                out[o] = fminf(fmaxf(x, lo), hi);
            } else {
                out[o] = b;
            }
        }
    }
}

}  // namespace

size_t cone_quads_bytes(const ConeGeom &g, int nviews) { return sizeof(float4) * (size_t)nviews * g.nx * g.np; }

int cone_pack_quads(const ConeGeom &g, const float *R, float4 *Q, int v0, int nv, cudaStream_t st) {
    const long long n = (long long)nv * g.nx * g.np;
    int blocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 16);
    pack_quads_kernel<<<blocks, 256, 0, st>>>(R + (long long)v0 * g.nx * g.np, Q, nv, g.nx, g.np);
    CT_LAUNCH_CHECK("pack_quads_kernel");
    return CT_OK;
}

int cone_bp_ztile() { return BP_ZC; }

// weighting: 0 chord, 1 FDK (off-detector adds 0), 2 FDK sticky
int cone_bp_launch(const ConeGeom &g, const float4 *Q, int v0, int nv, const float *prev, float *out, int weighting,
                   const float *colsum, float eps, float lambda, float lo, float hi, bool update, cudaStream_t st,
                   int zt0, int nzt) {
    CT_REQUIRE(g.np >= 2 && g.nx >= 2, "cone_bp: detector needs at least 2x2 samples");
    CT_REQUIRE(v0 >= 0 && nv > 0 && v0 + nv <= g.nb, "cone_bp: view range out of bounds");
    const int ntiles = (g.nz + BP_ZC - 1) / BP_ZC;
    if (nzt <= 0) nzt = ntiles - zt0;
    CT_REQUIRE(zt0 >= 0 && nzt > 0 && zt0 + nzt <= ntiles, "cone_bp: z tile range out of bounds");
    ConeGeom gk = g;   // with the set-up's constants
    cone_bp_consts(gk);
    dim3 block(BP_BX, BP_BY);
    dim3 grid((g.nt + BP_BX - 1) / BP_BX, (g.ns + BP_BY - 1) / BP_BY, nzt);
    const size_t smem = sizeof(float2) * (size_t)g.nx;
    CT_REQUIRE(smem <= 48 * 1024, "cone_bp: at most 6144 detector rows");
#define CT_BP_CASE(W, U)                                                                     \
    cone_bp_kernel<W, U><<<grid, block, smem, st>>>(gk, Q, v0, nv, prev, out, colsum, eps, lambda, lo, hi, zt0)
    if (update) {
        if (weighting == W_CHORD) CT_BP_CASE(W_CHORD, true);
        else if (weighting == W_FDK_ZERO) CT_BP_CASE(W_FDK_ZERO, true);
        else CT_BP_CASE(W_FDK_STICKY, true);
    } else {
        if (weighting == W_CHORD) CT_BP_CASE(W_CHORD, false);
        else if (weighting == W_FDK_ZERO) CT_BP_CASE(W_FDK_ZERO, false);
        else CT_BP_CASE(W_FDK_STICKY, false);
    }
#undef CT_BP_CASE
    CT_LAUNCH_CHECK("cone_bp_kernel");
    return CT_OK;
}

}  // namespace ct
