// ref_walk.cu -- FP64 grid walks of the reference projectors, for rays that
// graze a grid plane.
//
// A ray that runs within ~1e-9 of a t, s or z plane over its whole length (it
// is parallel to the plane to FP64 precision) is charged by the reference
// according to the rounding of a slope that is clamped at 1e16
// (ProjectionCone_3D.cu:44-84, ProjectionFan_2D.cu:37-49); no FP32 walk can
// reproduce that.  The fast kernels put such rays on a list (siddon.cuh sets
// RayWalk::grazing) and this file re-walks them with the reference's own
// algorithm in FP64: nearest plane by squared distance, voxel by the floor of
// the segment midpoint, the reference's loop bounds and exits.
//
// This translation unit is compiled with -fmad=false so that every operation
// rounds on its own, as the host build of that arithmetic does.  None of the
// benchmark geometries has such rays; symmetric test geometries (a detector
// bin at P = 0 with views at multiples of pi) do.
#include "kernels.cuh"

namespace ct {

namespace {

constexpr double EPS15 = 1e-15, ERR5 = 1e-5, EPS30 = 1e-30;

__device__ __forceinline__ double sq(double x) { return 1.0 * x * x; }
__device__ __forceinline__ double clamp16(double x) {
    x = x > 1e16 ? 1e16 : x;
    return x < -1e16 ? -1e16 : x;
}
__device__ __forceinline__ double d3(double a0, double a1, double a2, double b0, double b1, double b2) {
    return sq(a0 - b0) + sq(a1 - b1) + sq(a2 - b2);
}
__device__ __forceinline__ double d2(double a0, double a1, double b0, double b1) {
    return sq(a0 - b0) + sq(a1 - b1);
}

// ProjectionCone (ProjectionCone_3D.cu:25-375) for one ray; sb, cb are the
// single-precision sin/cos of the float angle, widened.  visit(voxel, length)
// is called for every segment in walk order.
template <class Visit>
__device__ void cone_walk_ref(const ConeGeom &g, double sb, double cb, float P, float xi, Visit &&visit) {
    const double r1 = g.res[0], r2 = g.res[1], r3 = g.res[2], D = g.D;
    const double ct = g.size[0] / 2, cs = g.size[1] / 2, cz = g.size[2] / 2;
    const int nt = g.nt, ns = g.ns, nz = g.nz;
    const double src_t = ct - D * sb, src_s = cs + D * cb, src_z = cz;
    const double gama = atan(xi / D);
    const double dshift = D / cos(gama);
    const double theta = atan(P / dshift);
    const double smax = 2 * D;
    const double end_t = ct + smax * sin(theta) * cb - (D - smax * cos(theta) * cos(gama)) * sb;
    const double end_s = cs + smax * sin(theta) * sb + (D - smax * cos(theta) * cos(gama)) * cb;
    const double end_z = cz + smax * cos(theta) * sin(gama);
    const double dt = end_t - src_t, ds = end_s - src_s, dz = end_z - src_z;
    double t2s, t2z, s2t, s2z, z2t, z2s;
    if (dt == 0) { t2s = ds / (dt + EPS15); t2z = dz / (dt + EPS15); } else { t2s = ds / dt; t2z = dz / dt; }
    if (ds == 0) { s2t = dt / (ds + EPS15); s2z = dz / (ds + EPS15); } else { s2t = dt / ds; s2z = dz / ds; }
    if (dz == 0) { z2t = dt / (dz + EPS15); z2s = ds / (dz + EPS15); } else { z2t = dt / dz; z2s = ds / dz; }
    t2s = clamp16(t2s); t2z = clamp16(t2z); s2t = clamp16(s2t);
    s2z = clamp16(s2z); z2t = clamp16(z2t); z2s = clamp16(z2s);
    const int sig_t = end_t >= src_t ? 1 : -1, sig_s = end_s >= src_s ? 1 : -1, sig_z = end_z >= src_z ? 1 : -1;
    const double tlo = 0, thi = nt * r1, slo = 0, shi = ns * r2, zlo = 0, zhi = nz * r3;
    const double ft[6] = {tlo, thi, src_t + (slo - src_s) * s2t, src_t + (shi - src_s) * s2t,
                          src_t + (zlo - src_z) * z2t, src_t + (zhi - src_z) * z2t};
    const double fs[6] = {src_s + (tlo - src_t) * t2s, src_s + (thi - src_t) * t2s, slo, shi,
                          src_s + (zlo - src_z) * z2s, src_s + (zhi - src_z) * z2s};
    const double fz[6] = {src_z + (tlo - src_t) * t2z, src_z + (thi - src_t) * t2z, src_z + (slo - src_s) * s2z,
                          src_z + (shi - src_s) * s2z, zlo, zhi};
    bool ok[6];
    ok[0] = fs[0] >= 0 && fs[0] <= shi && fz[0] >= 0 && fz[0] <= zhi;
    ok[1] = fs[1] >= 0 && fs[1] <= shi && fz[1] >= 0 && fz[1] <= zhi;
    ok[2] = ft[2] >= 0 && ft[2] <= thi && fz[2] >= 0 && fz[2] <= zhi;
    ok[3] = ft[3] >= 0 && ft[3] <= thi && fz[3] >= 0 && fz[3] <= zhi;
    ok[4] = ft[4] >= 0 && ft[4] <= thi && fs[4] >= 0 && fs[4] <= shi;
    ok[5] = ft[5] >= 0 && ft[5] <= thi && fs[5] >= 0 && fs[5] <= shi;
    int first = -1, second = -1;
    for (int f = 0; f < 6; ++f) if (ok[f]) { first = f; break; }
    if (first < 0 || first == 5) return;
    for (int f = first + 1; f < 6; ++f) if (ok[f]) { second = f; break; }
    const double T1 = ft[first], S1 = fs[first], Z1 = fz[first];
    double T2 = 0, S2 = 0, Z2 = 0;
    if (second >= 0) { T2 = ft[second]; S2 = fs[second]; Z2 = fz[second]; }
    double Ts, Ss, Zs;
    if (d3(T1, S1, Z1, src_t, src_s, src_z) >= d3(T2, S2, Z2, src_t, src_s, src_z)) { Ts = T2; Ss = S2; Zs = Z2; }
    else { Ts = T1; Ss = S1; Zs = Z1; }
    double tc = Ts / r1, sc = Ss / r2, zc = Zs / r3;
    const int up_t = (1 + sig_t) / 2, up_s = (1 + sig_s) / 2, up_z = (1 + sig_z) / 2;
    for (int i = 0; i < nt + ns + nz - 2; ++i) {
        short gt, gs, gz;
        if (tc - (double)((short)tc) < EPS15) gt = (short)(tc + sig_t); else gt = (short)(floor(tc) + up_t);
        const double gt_s = (src_s + (gt * r1 - src_t) * t2s) / r2, gt_z = (src_z + (gt * r1 - src_t) * t2z) / r3;
        if (sc - (double)((short)sc) < EPS15) gs = (short)(sc + sig_s); else gs = (short)(floor(sc) + up_s);
        const double gs_t = (src_t + (gs * r2 - src_s) * s2t) / r1, gs_z = (src_z + (gs * r2 - src_s) * s2z) / r3;
        if (zc - (double)((short)zc) < EPS15) gz = (short)(zc + sig_z); else gz = (short)(floor(zc) + up_z);
        const double gz_t = (src_t + (gz * r3 - src_z) * z2t) / r1, gz_s = (src_s + (gz * r3 - src_z) * z2s) / r2;
        const double dT = d3(gt, gt_s, gt_z, tc, sc, zc), dS = d3(gs_t, gs, gs_z, tc, sc, zc);
        const double dZ = d3(gz_t, gz_s, gz, tc, sc, zc);
        double nt_, ns_, nz_;
        if (dT <= dS) {
            if (dZ <= dT) { nt_ = gz_t; ns_ = gz_s; nz_ = gz; } else { nt_ = gt; ns_ = gt_s; nz_ = gt_z; }
        } else {
            if (dZ <= dS) { nt_ = gz_t; ns_ = gz_s; nz_ = gz; } else { nt_ = gs_t; ns_ = gs; nz_ = gs_z; }
        }
        const double w = sqrt(d3(nt_ * r1, ns_ * r2, nz_ * r3, tc * r1, sc * r2, zc * r3));
        const int it = (int)floor((nt_ + tc) / 2), is = (int)floor((ns_ + sc) / 2), iz = (int)floor((nz_ + zc) / 2);
        tc = nt_; sc = ns_; zc = nz_;
        if (it >= 0 && it < nt && is >= 0 && is < ns && iz >= 0 && iz < nz)
            visit(((long long)iz * ns + is) * nt + it, w);
        else
            break;
    }
}

__device__ float cone_ray_ref(const ConeGeom &g, const float *__restrict__ vol, double sb, double cb, float P,
                              float xi) {
    double ray = 0;
    cone_walk_ref(g, sb, cb, P, xi, [&](long long i, double w) { ray += w * vol[i]; });
    return (float)ray;
}

// ProjectionFan (ProjectionFan_2D.cu:19-216): double angle and bin.
template <class Visit>
__device__ void fan_walk_ref(const FanGeom &g, double sb, double cb, double P, Visit &&visit) {
    const double r1 = g.res[0], r2 = g.res[1], D = g.D;
    const int nt = g.nt, ns = g.ns;
    const double ct = g.size[0] / 2, cs = g.size[1] / 2;
    // sin(-beta) = -sin(beta), cos(-beta) = cos(beta)
    const double src_t = ct + D * (-sb), src_s = cs + D * cb;
    const double theta = atan(P / D), smax = 2 * D;
    const double end_t = ct + smax * sin(theta) * cb + (D - smax * cos(theta)) * (-sb);
    const double end_s = cs - smax * sin(theta) * (-sb) + (D - smax * cos(theta)) * cb;
    const double dt = end_t - src_t, ds = end_s - src_s;
    double t2s = (dt == 0) ? ds / (dt + EPS15) : ds / dt;
    double s2t = (ds == 0) ? dt / (ds + EPS15) : dt / ds;
    t2s = clamp16(t2s); s2t = clamp16(s2t);
    const int sig_t = end_t >= src_t ? 1 : -1, sig_s = end_s >= src_s ? 1 : -1;
    const double tlo = 0, thi = nt * r1, slo = 0, shi = ns * r2;
    const double ft[4] = {tlo, thi, src_t + (slo - src_s) * s2t, src_t + (shi - src_s) * s2t};
    const double fs[4] = {src_s + (tlo - src_t) * t2s, src_s + (thi - src_t) * t2s, slo, shi};
    const bool ok[4] = {fs[0] >= 0 && fs[0] <= shi, fs[1] >= 0 && fs[1] <= shi, ft[2] >= 0 && ft[2] <= thi,
                        ft[3] >= 0 && ft[3] <= thi};
    int first = -1, second = -1;
    for (int f = 0; f < 4; ++f) if (ok[f]) { first = f; break; }
    if (first < 0 || first == 3) return;
    for (int f = first + 1; f < 4; ++f) if (ok[f]) { second = f; break; }
    const double T1 = ft[first], S1 = fs[first];
    double T2 = 0, S2 = 0;
    if (second >= 0) { T2 = ft[second]; S2 = fs[second]; }
    double Ts, Ss;
    if (d2(T1, S1, src_t, src_s) >= d2(T2, S2, src_t, src_s)) { Ts = T2; Ss = S2; } else { Ts = T1; Ss = S1; }
    double tc = Ts / r1, sc = Ss / r2;
    const int up_t = (1 + sig_t) / 2, up_s = (1 + sig_s) / 2;
    for (int i = 0; i < nt + ns - 1; ++i) {
        short gt, gs;
        if (fabs(tc - round(tc)) < EPS15) gt = (short)(round(tc) + sig_t); else gt = (short)(floor(tc) + up_t);
        const double gt_s = (src_s + (gt * r1 - src_t) * t2s) / r2;
        if (fabs(sc - round(sc)) < EPS15) gs = (short)(round(sc) + sig_s); else gs = (short)(floor(sc) + up_s);
        const double gs_t = (src_t + (gs * r2 - src_s) * s2t) / r1;
        double w, nt_, ns_;
        if (d2(gt, gt_s, tc, sc) <= d2(gs_t, gs, tc, sc)) {
            w = sqrt(d2(gt * r1, gt_s * r2, tc * r1, sc * r2)); nt_ = gt; ns_ = gt_s;
        } else {
            w = sqrt(d2(gs_t * r1, gs * r2, tc * r1, sc * r2)); nt_ = gs_t; ns_ = gs;
        }
        const int it = (int)floor((nt_ + tc) / 2), is = (int)floor((ns_ + sc) / 2);
        tc = nt_; sc = ns_;
        if (it >= 0 && it < nt && is >= 0 && is < ns) visit((long long)is * nt + it, w);
        else break;
    }
}

__device__ double fan_ray_ref(const FanGeom &g, const float *__restrict__ pic, double sb, double cb, double P) {
    double ray = 0;
    fan_walk_ref(g, sb, cb, P, [&](long long i, double w) { ray += w * pic[i]; });
    return ray;
}

// ProjectionParallel (ProjectionParallel_2D.cu:23-243); x = t axis (width),
// y = s axis (height) of the FanGeom.
template <class Visit>
__device__ void par_walk_ref(const FanGeom &g, double sb, double cb, double t, Visit &&visit) {
    const double rx = g.res[0], ry = g.res[1], smax = g.smax;
    const int wd = g.nt, h = g.ns;
    const double cx = g.size[0] / 2, cy = g.size[1] / 2;
    const double xs = cx + t * cb + (-smax) * (-sb), ys = cy - t * (-sb) + (-smax) * cb;
    const double xe = cx + t * cb + smax * (-sb), ye = cy - t * (-sb) + smax * cb;
    double x2y = (xe - xs == 0) ? (ye - ys) / (xe - xs + EPS30) : (ye - ys) / (xe - xs);
    double y2x = (ye - ys == 0) ? (xe - xs) / (ye - ys + EPS30) : (xe - xs) / (ye - ys);
    x2y = clamp16(x2y); y2x = clamp16(y2x);
    const int sig_y = (ye >= ys) ? 1 : (ye < ys ? -1 : 0), sig_x = (xe >= xs) ? 1 : (xe < xs ? -1 : 0);
    const double xhi = wd * rx, yhi = h * ry;
    const double fx[4] = {xs + (0 - ys) * y2x, xs + (yhi - ys) * y2x, 0, xhi};
    const double fy[4] = {0, yhi, ys + (0 - xs) * x2y, ys + (xhi - xs) * x2y};
    const bool ok[4] = {fx[0] >= 0 && fx[0] <= xhi, fx[1] >= 0 && fx[1] <= xhi, fy[2] >= 0 && fy[2] <= yhi,
                        fy[3] >= 0 && fy[3] <= yhi};
    int first = -1;
    for (int f = 0; f < 4; ++f) if (ok[f]) { first = f; break; }
    if (first < 0 || first == 3) return;
    const int order[3][3] = {{2, 3, 1}, {2, 3, -1}, {3, -1, -1}};
    int second = -1;
    for (int k = 0; k < 3; ++k) {
        const int f = order[first][k];
        if (f >= 0 && ok[f]) { second = f; break; }
    }
    const double X1 = fx[first], Y1 = fy[first];
    double X2 = 0, Y2 = 0;
    if (second >= 0) { X2 = fx[second]; Y2 = fy[second]; }
    double Xs, Ys;
    if (d2(X1, Y1, xs, ys) >= d2(X2, Y2, xs, ys)) { Xs = X2; Ys = Y2; } else { Xs = X1; Ys = Y1; }
    double xc = Xs / rx, yc = Ys / ry;
    const int up_x = (1 + sig_x) / 2, up_y = (1 + sig_y) / 2;
    for (int i = 0; i < h + wd - 1; ++i) {
        short gx, gy;
        if (fabs(xc - round(xc)) < ERR5) gx = (short)(round(xc) + sig_x); else gx = (short)(floor(xc) + up_x);
        const double gx_y = (ys + (gx * rx - xs) * x2y) / ry;
        if (fabs(yc - round(yc)) < ERR5) gy = (short)(round(yc) + sig_y); else gy = (short)(floor(yc) + up_y);
        const double gy_x = (xs + (gy * ry - ys) * y2x) / rx;
        double w, nx_, ny_;
        if (d2(gx, gx_y, xc, yc) >= d2(gy_x, gy, xc, yc)) {
            w = sqrt(d2(gy_x * rx, gy * ry, xc * rx, yc * ry)); nx_ = gy_x; ny_ = gy;
        } else {
            w = sqrt(d2(gx * rx, gx_y * ry, xc * rx, yc * ry)); nx_ = gx; ny_ = gx_y;
        }
        const int ix = (int)floor((nx_ + xc) / 2), iy = (int)floor((ny_ + yc) / 2);
        xc = nx_; yc = ny_;
        if (ix >= 0 && ix < wd && iy >= 0 && iy < h) visit((long long)iy * wd + ix, w);
        else break;
    }
}

__device__ double par_ray_ref(const FanGeom &g, const float *__restrict__ pic, double sb, double cb, double t) {
    double ray = 0;
    par_walk_ref(g, sb, cb, t, [&](long long i, double w) { ray += w * pic[i]; });
    return ray;
}

// Visit every grazing ray the fast kernel recorded: the listed entries, and,
// when the list overflowed, every bit of the overflow bitmap.  Each bitmap
// word is cleared as it is read, so the bitmap is all zeros again for the
// next launch.  Grid-stride over both; call with the whole grid.
template <class OnEntry, class OnBit>
__device__ __forceinline__ void graze_drain(const GrazeList &gl, OnEntry on_entry, OnBit on_bit) {
    const unsigned long long cnt = *gl.count;
    const long long n = (long long)min(cnt, (unsigned long long)gl.cap);
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // list entries dealt one per block first (entry i to block i mod grid), so a
    // short list spreads over the SMs: the re-walk is FP64-bound (64 batched
    // slices, 102 listed rays: 6.73 -> 6.59 ms for the projection with it)
    const long long lt = (long long)threadIdx.x * gridDim.x + blockIdx.x;
    for (long long i = lt; i < n; i += stride) on_entry(gl.rays[i]);
    if (cnt > (unsigned long long)gl.cap && gl.bits) {
        const long long nw = (gl.nbits + 31) >> 5;
        for (long long w = tid; w < nw; w += stride) {
            unsigned m = gl.bits[w];
            if (!m) continue;
            gl.bits[w] = 0u;
            while (m) {
                const int bit = __ffs(m) - 1;
                m &= m - 1;
                on_bit((unsigned long long)w * 32 + bit);
            }
        }
    }
}

// Re-walk the recorded rays.  mode 0: out = A x;  mode 1: out = (b - A x) * scale
// with norms[0] corrected by the change of the squared residual.
__global__ void __launch_bounds__(64)
cone_fixup_kernel(const ConeGeom g, const float *__restrict__ vol, float *__restrict__ out,
                  const float *__restrict__ b, const float *__restrict__ rowsum, float eps, double *norms, int mode,
                  const GrazeList gl) {
    auto fix = [&](unsigned long long r) {
        const int p = (int)(r % g.np), x = (int)((r / g.np) % g.nx), v = (int)(r / ((unsigned long long)g.np * g.nx));
        const double2 tr = g.trig[v];
        const float val = cone_ray_ref(g, vol, tr.x, tr.y, g.P[p], g.xi[x]);
        if (mode == 0) {
            out[r] = val;
        } else {
            const float sc = rowsum ? 1.0f / (rowsum[r] + eps) : 1.0f;
            const float rr = b[r] - val;
            out[r] = rr * sc;
            atomicAdd(norms, (double)rr * rr);   // the fast kernel left this ray out of the norm
        }
    };
    graze_drain(gl, fix, fix);
}

template <typename OutT>
__global__ void __launch_bounds__(64)
fan_fixup_kernel(const FanGeom g, const float *__restrict__ img, OutT *__restrict__ out,
                 const float *__restrict__ b, const float *__restrict__ rowsum, float eps, double *norms, int mode,
                 const GrazeList gl) {
    auto fix = [&](unsigned long long r) {
        const int p = (int)(r % g.np), v = (int)(r / g.np);
        const double2 tr = g.trig_d[v];
        const double val = g.parallel ? par_ray_ref(g, img, tr.x, tr.y, g.Pd[p]) : fan_ray_ref(g, img, tr.x, tr.y, g.Pd[p]);
        if (mode == 0) {
            out[r] = (OutT)val;
        } else {
            const float sc = rowsum ? 1.0f / (rowsum[r] + eps) : 1.0f;
            const float rr = b[r] - (float)val;
            out[r] = (OutT)(rr * sc);
            atomicAdd(norms, (double)rr * rr);   // the fast kernel left this ray out of the norm
        }
    };
    graze_drain(gl, fix, fix);
}

// Batched slices: list entries are (slice << 40) | ray; bitmap bits are the
// ray's offset in the packed sinogram.
__global__ void __launch_bounds__(64)
fan_batch_fixup_kernel(const BatchSlice *__restrict__ sl, int nsl, const float *__restrict__ img,
                       float *__restrict__ out, const float *__restrict__ b, const float *__restrict__ rowsum,
                       float eps, double *norms, int mode, const GrazeList gl) {
    auto fix = [&](int k, unsigned long long r) {
        const FanGeom g = sl[k].g;
        const int p = (int)(r % g.np), v = (int)(r / g.np);
        const double2 tr = g.trig_d[v];
        const float *im = img + sl[k].img_off;
        const double val = g.parallel ? par_ray_ref(g, im, tr.x, tr.y, g.Pd[p]) : fan_ray_ref(g, im, tr.x, tr.y, g.Pd[p]);
        const long long o = sl[k].sino_off + (long long)r;
        if (mode == 0) {
            out[o] = (float)val;
        } else {
            const float sc = rowsum ? 1.0f / (rowsum[o] + eps) : 1.0f;
            const float rr = b[o] - (float)val;
            out[o] = rr * sc;
            atomicAdd(norms + 2 * k, (double)rr * rr);   // left out by the fast kernel
        }
    };
    auto on_entry = [&](unsigned long long e) { fix((int)(e >> 40), e & ((1ULL << 40) - 1)); };
    auto on_bit = [&](unsigned long long o) {
        int lo = 0, hi = nsl - 1;   // last slice whose sinogram starts at or before o
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((unsigned long long)sl[mid].sino_off <= o) lo = mid; else hi = mid - 1;
        }
        fix(lo, o - (unsigned long long)sl[lo].sino_off);
    };
    graze_drain(gl, on_entry, on_bit);
}

// One CSR row from a reference walk: pieces of zero length are dropped and
// consecutive pieces in the same voxel merged, as the fast export does.
struct CsrRow {
    bool fill;
    int *col;
    float *val;
    long long base;
    int n;
    long long prev;
    __device__ void operator()(long long i, double w) {
        if (!(w > 0.0)) return;
        if (i == prev) {
            if (fill) val[base + n - 1] += (float)w;
            return;
        }
        if (fill) {
            col[base + n] = (int)i;
            val[base + n] = (float)w;
        }
        ++n;
        prev = i;
    }
};

// Rows of the listed (grazing) rays: counts into row_ptr[row + 1] or entries
// at row_ptr[row]; rows are ray - r0.
__global__ void __launch_bounds__(64)
cone_sysmat_ref_kernel(const ConeGeom g, long long r0, long long *__restrict__ row_ptr, int *__restrict__ col,
                       float *__restrict__ val, bool fill, const GrazeList gl) {
    auto row_of = [&](unsigned long long r) {
        const int p = (int)(r % g.np), x = (int)((r / g.np) % g.nx), v = (int)(r / ((unsigned long long)g.np * g.nx));
        const long long row = (long long)r - r0;
        const double2 tr = g.trig[v];
        CsrRow e{fill, col, val, fill ? row_ptr[row] : 0, 0, -1};
        cone_walk_ref(g, tr.x, tr.y, g.P[p], g.xi[x], e);
        if (!fill) row_ptr[row + 1] = e.n;
    };
    graze_drain(gl, row_of, row_of);
}

__global__ void __launch_bounds__(64)
fan_sysmat_ref_kernel(const FanGeom g, long long *__restrict__ row_ptr, int *__restrict__ col, float *__restrict__ val,
                      bool fill, const GrazeList gl) {
    auto row_of = [&](unsigned long long r) {
        const int p = (int)(r % g.np), v = (int)(r / g.np);
        const double2 tr = g.trig_d[v];
        CsrRow e{fill, col, val, fill ? row_ptr[r] : 0, 0, -1};
        if (g.parallel) par_walk_ref(g, tr.x, tr.y, g.Pd[p], e);
        else fan_walk_ref(g, tr.x, tr.y, g.Pd[p], e);
        if (!fill) row_ptr[r + 1] = e.n;
    };
    graze_drain(gl, row_of, row_of);
}

}  // namespace

// The re-walk grids: four 64-thread blocks per SM, grid-stride over the list
// and the overflow bitmap.  A launch with nothing
// recorded reads the count and returns.
static unsigned fixup_blocks() { return (unsigned)(4 * sm_count()); }

int fan_batch_fixup_launch(const BatchSlice *d_sl, int nsl, const float *img, float *out, const float *b,
                           const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl,
                           cudaStream_t st) {
    fan_batch_fixup_kernel<<<fixup_blocks(), 64, 0, st>>>(d_sl, nsl, img, out, b, rowsum, eps, norms, mode, gl);
    CT_LAUNCH_CHECK("fan_batch_fixup_kernel");
    return CT_OK;
}

int cone_fixup_launch(const ConeGeom &g, const float *vol, float *out, const float *b, const float *rowsum,
                      float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st) {
    cone_fixup_kernel<<<fixup_blocks(), 64, 0, st>>>(g, vol, out, b, rowsum, eps, norms, mode, gl);
    CT_LAUNCH_CHECK("cone_fixup_kernel");
    return CT_OK;
}

int fan_fixup_launch(const FanGeom &g, const float *img, void *out, bool out_double, const float *b,
                     const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st) {
    if (out_double)
        fan_fixup_kernel<double><<<fixup_blocks(), 64, 0, st>>>(g, img, (double *)out, b, rowsum, eps, norms, mode, gl);
    else
        fan_fixup_kernel<float><<<fixup_blocks(), 64, 0, st>>>(g, img, (float *)out, b, rowsum, eps, norms, mode, gl);
    CT_LAUNCH_CHECK("fan_fixup_kernel");
    return CT_OK;
}

int cone_sysmat_ref_launch(const ConeGeom &g, long long r0, long long *row_ptr, int *col, float *val, bool fill,
                           const GrazeList &gl, cudaStream_t st) {
    cone_sysmat_ref_kernel<<<fixup_blocks(), 64, 0, st>>>(g, r0, row_ptr, col, val, fill, gl);
    CT_LAUNCH_CHECK("cone_sysmat_ref_kernel");
    return CT_OK;
}

int fan_sysmat_ref_launch(const FanGeom &g, long long *row_ptr, int *col, float *val, bool fill, const GrazeList &gl,
                          cudaStream_t st) {
    fan_sysmat_ref_kernel<<<fixup_blocks(), 64, 0, st>>>(g, row_ptr, col, val, fill, gl);
    CT_LAUNCH_CHECK("fan_sysmat_ref_kernel");
    return CT_OK;
}

}  // namespace ct
