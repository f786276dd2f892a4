/*
 * ct_oracle.c -- FP64 CPU restatement of the CT-Research projector /
 * backprojector operators.  TEST INFRASTRUCTURE ONLY: this file is the
 * checker for the CUDA path (tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py); nothing in the product library
 * links or calls it.
 *
 * Each function follows one kernel of the reference, step for step, in the
 * reference's own precision (double arithmetic on float data, float
 * accumulators where the reference accumulates into float buffers), so that
 * its output agrees with the reference kernel to the last bits on the same
 * inputs.  The file:line of the reference code each part follows is cited.
 * All reference paths are relative to the CT-Research project root.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/build.py).
 * -ffp-contract=off keeps a*b+c as two roundings on every host (x86 and Arm).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OC_API __attribute__((visibility("default")))

static const double OC_EPS15 = 1e-15;   /* ProjectionCone_3D.cu:5, ProjectionFan_2D.cu:5 */
static const double OC_ERR5 = 1e-5;     /* ProjectionParallel_2D.cu:6 */
static const double OC_EPS30 = 1e-30;   /* ProjectionParallel_2D.cu:5 */
static const double OC_PI = 3.141592653589793;  /* FDK.cu:4 */

static inline double sq(double x) { return 1.0 * x * x; }
static inline double slope_clamp(double x) {   /* Maxlim / Minlim, ProjectionCone_3D.h:29-30 */
    x = x > 1e16 ? 1e16 : x;
    return x < -1e16 ? -1e16 : x;
}
static inline double dist3sq(double a0, double a1, double a2, double b0, double b1, double b2) {
    return sq(a0 - b0) + sq(a1 - b1) + sq(a2 - b2);
}
static inline double dist2sq(double a0, double a1, double b0, double b1) {
    return sq(a0 - b0) + sq(a1 - b1);
}
static void set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* 3D cone-beam Siddon forward projection: one ray (beta, P, xi).           */
/* Follows ProjectionCone (ProjectionCone_3D.cu:8-379).                    */
/* ------------------------------------------------------------------------ */
static float cone_ray(const float *vol, int nt, int ns, int nz, const double res[3],
                      double ct, double cs, double cz, float beta, float P, float xi, double D)
{
    const double r1 = res[0], r2 = res[1], r3 = res[2];
    /* source and far end of the ray, :26-42 */
    /* Beta is a float kernel argument, so sin(Beta)/cos(Beta) resolve to the
       single-precision overloads in the reference (C++ overloading). */
    const double sb = sinf(beta), cb = cosf(beta);
    double src_t = ct - D * sb;
    double src_s = cs + D * cb;
    double src_z = cz;
    double gama = atan(xi / D);
    double dshift = D / cos(gama);
    double theta = atan(P / dshift);
    double smax = 2 * D;
    double end_t = ct + smax * sin(theta) * cb - (D - smax * cos(theta) * cos(gama)) * sb;
    double end_s = cs + smax * sin(theta) * sb + (D - smax * cos(theta) * cos(gama)) * cb;
    double end_z = cz + smax * cos(theta) * sin(gama);

    /* six slopes, :44-84 */
    double dt = end_t - src_t, ds = end_s - src_s, dz = end_z - src_z;
    double t2s, t2z, s2t, s2z, z2t, z2s;
    if (dt == 0) { t2s = ds / (dt + OC_EPS15); t2z = dz / (dt + OC_EPS15); }
    else { t2s = ds / dt; t2z = dz / dt; }
    if (ds == 0) { s2t = dt / (ds + OC_EPS15); s2z = dz / (ds + OC_EPS15); }
    else { s2t = dt / ds; s2z = dz / ds; }
    if (dz == 0) { z2t = dt / (dz + OC_EPS15); z2s = ds / (dz + OC_EPS15); }
    else { z2t = dt / dz; z2s = ds / dz; }
    t2s = slope_clamp(t2s); t2z = slope_clamp(t2z); s2t = slope_clamp(s2t);
    s2z = slope_clamp(s2z); z2t = slope_clamp(z2t); z2s = slope_clamp(z2s);

    int sig_t = end_t >= src_t ? 1 : -1;   /* :87-108 */
    int sig_s = end_s >= src_s ? 1 : -1;
    int sig_z = end_z >= src_z ? 1 : -1;

    /* box faces and their hit points, :111-129 */
    double tlo = 0, thi = nt * r1, slo = 0, shi = ns * r2, zlo = 0, zhi = nz * r3;
    double tlo_s = src_s + (tlo - src_t) * t2s, tlo_z = src_z + (tlo - src_t) * t2z;
    double thi_s = src_s + (thi - src_t) * t2s, thi_z = src_z + (thi - src_t) * t2z;
    double slo_t = src_t + (slo - src_s) * s2t, slo_z = src_z + (slo - src_s) * s2z;
    double shi_t = src_t + (shi - src_s) * s2t, shi_z = src_z + (shi - src_s) * s2z;
    double zlo_t = src_t + (zlo - src_z) * z2t, zlo_s = src_s + (zlo - src_z) * z2s;
    double zhi_t = src_t + (zhi - src_z) * z2t, zhi_s = src_s + (zhi - src_z) * z2s;

    /* first two faces found, in the reference's search order, :132-218 */
    int f_tlo = tlo_s >= 0 && tlo_s <= shi && tlo_z >= 0 && tlo_z <= zhi;
    int f_thi = thi_s >= 0 && thi_s <= shi && thi_z >= 0 && thi_z <= zhi;
    int f_slo = slo_t >= 0 && slo_t <= thi && slo_z >= 0 && slo_z <= zhi;
    int f_shi = shi_t >= 0 && shi_t <= thi && shi_z >= 0 && shi_z <= zhi;
    int f_zlo = zlo_t >= 0 && zlo_t <= thi && zlo_s >= 0 && zlo_s <= shi;
    int f_zhi = zhi_t >= 0 && zhi_t <= thi && zhi_s >= 0 && zhi_s <= shi;
    double ft[6] = {tlo, thi, slo_t, shi_t, zlo_t, zhi_t};
    double fs[6] = {tlo_s, thi_s, slo, shi, zlo_s, zhi_s};
    double fz[6] = {tlo_z, thi_z, slo_z, shi_z, zlo, zhi};
    int ok[6] = {f_tlo, f_thi, f_slo, f_shi, f_zlo, f_zhi};
    int first = -1, second = -1;
    for (int f = 0; f < 6; ++f) if (ok[f]) { first = f; break; }
    if (first < 0 || first == 5) return 0.0f;         /* zhi alone is never a first face, :214-218 */
    for (int f = first + 1; f < 6; ++f) if (ok[f]) { second = f; break; }
    double T1 = ft[first], S1 = fs[first], Z1 = fz[first];
    double T2 = 0, S2 = 0, Z2 = 0;                    /* unset second point stays 0, :132 */
    if (second >= 0) { T2 = ft[second]; S2 = fs[second]; Z2 = fz[second]; }

    /* start point = the one nearer the source, :221-233 */
    double Ts, Ss, Zs;
    if (dist3sq(T1, S1, Z1, src_t, src_s, src_z) >= dist3sq(T2, S2, Z2, src_t, src_s, src_z)) {
        Ts = T2; Ss = S2; Zs = Z2;
    } else {
        Ts = T1; Ss = S1; Zs = Z1;
    }

    /* grid walk, :257-375 */
    double ray = 0;
    double tc = Ts / r1, sc = Ss / r2, zc = Zs / r3;
    int nit = nt + ns + nz - 2;
    int up_t = (1 + sig_t) / 2, up_s = (1 + sig_s) / 2, up_z = (1 + sig_z) / 2;
    for (int i = 0; i < nit; ++i) {
        short gt, gs, gz;
        if (tc - (double)((short)tc) < OC_EPS15) gt = (short)(tc + sig_t);
        else gt = (short)(floor(tc) + up_t);
        double gt_s = (src_s + (gt * r1 - src_t) * t2s) / r2;
        double gt_z = (src_z + (gt * r1 - src_t) * t2z) / r3;
        if (sc - (double)((short)sc) < OC_EPS15) gs = (short)(sc + sig_s);
        else gs = (short)(floor(sc) + up_s);
        double gs_t = (src_t + (gs * r2 - src_s) * s2t) / r1;
        double gs_z = (src_z + (gs * r2 - src_s) * s2z) / r3;
        if (zc - (double)((short)zc) < OC_EPS15) gz = (short)(zc + sig_z);
        else gz = (short)(floor(zc) + up_z);
        double gz_t = (src_t + (gz * r3 - src_z) * z2t) / r1;
        double gz_s = (src_s + (gz * r3 - src_z) * z2s) / r2;

        double nt_, ns_, nz_;   /* chosen crossing point in grid units */
        double dT = dist3sq(gt, gt_s, gt_z, tc, sc, zc);
        double dS = dist3sq(gs_t, gs, gs_z, tc, sc, zc);
        double dZ = dist3sq(gz_t, gz_s, gz, tc, sc, zc);
        if (dT <= dS) {
            if (dZ <= dT) { nt_ = gz_t; ns_ = gz_s; nz_ = gz; }
            else { nt_ = gt; ns_ = gt_s; nz_ = gt_z; }
        } else {
            if (dZ <= dS) { nt_ = gz_t; ns_ = gz_s; nz_ = gz; }
            else { nt_ = gs_t; ns_ = gs; nz_ = gs_z; }
        }
        double w = sqrt(dist3sq(nt_ * r1, ns_ * r2, nz_ * r3, tc * r1, sc * r2, zc * r3));
        short it = (short)floor((nt_ + tc) / 2);
        short is = (short)floor((ns_ + sc) / 2);
        short iz = (short)floor((nz_ + zc) / 2);
        tc = nt_; sc = ns_; zc = nz_;
        if (it >= 0 && it < nt && is >= 0 && is < ns && iz >= 0 && iz < nz) {
            long id = (long)iz * nt * ns + (long)is * nt + it;
            ray += w * vol[id];
        } else {
            break;
        }
    }
    return (float)ray;
}

OC_API void oc_cone_fp(const float *vol, float *proj, const float *beta, const float *P,
                       const float *xi, int nt, int ns, int nz, double ct, double cs, double cz,
                       int nb, int np, int nx, double D, const double *res, int nthreads)
{
    set_threads(nthreads);
    long nray = (long)nb * nx * np;
#pragma omp parallel for schedule(dynamic, 256)
    for (long r = 0; r < nray; ++r) {
        int ip = (int)(r % np);
        int ix = (int)((r / np) % nx);
        int ib = (int)(r / ((long)np * nx));
        proj[r] = cone_ray(vol, nt, ns, nz, res, ct, cs, cz, beta[ib], P[ip], xi[ix], D);
    }
}

/* ------------------------------------------------------------------------ */
/* Shared detector-range bookkeeping of the voxel-driven backprojectors.    */
/* PInt/XigamaInt/minP/maxP are computed in float as in BackPro            */
/* (Backprojection3D.cu:304-311) and FDKpro (FDK.cu:140-147).              */
/* ------------------------------------------------------------------------ */
typedef struct {
    float pint, xint, bint, minp, maxp, minx, maxx;
} det_range;

static det_range make_range(const float *P, int np, const float *xi, int nx, const float *beta, int nb)
{
    det_range r;
    r.pint = fabsf(P[1] - P[0]);
    r.xint = (xi && nx > 1) ? fabsf(xi[1] - xi[0]) : 0.0f;
    r.bint = (beta && nb > 1) ? fabsf(beta[1] - beta[0]) : 0.0f;
    r.maxp = P[0] > P[np - 1] ? P[0] : P[np - 1];
    r.minp = P[0] < P[np - 1] ? P[0] : P[np - 1];
    if (xi) {
        r.maxx = xi[0] > xi[nx - 1] ? xi[0] : xi[nx - 1];
        r.minx = xi[0] < xi[nx - 1] ? xi[0] : xi[nx - 1];
    } else {
        r.maxx = r.minx = 0;
    }
    return r;
}

/* ------------------------------------------------------------------------ */
/* 3D cone voxel-driven backprojection with chord weight.                   */
/* Follows BackProjection3D (Backprojection3D.cu:8-291); the view loop is   */
/* the per-view launch loop of BackPro (:445-520), so the float             */
/* accumulation order over views is the reference's.                        */
/* ------------------------------------------------------------------------ */
OC_API void oc_cone_bp(float *disp, const float *R, const float *xi, const float *P,
                       const float *beta, double D, int nb, int np, int nx, const double *size,
                       int nt, int ns, int nz, int nthreads)
{
    set_threads(nthreads);
    det_range g = make_range(P, np, xi, nx, beta, nb);
    const double rt = 1.0 * size[0] / nt, rs = 1.0 * size[1] / ns, rz = 1.0 * size[2] / nz;
    const double ct = size[0] / 2, cs = size[1] / 2, cz = size[2] / 2;
    memset(disp, 0, sizeof(float) * (size_t)nt * ns * nz);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
    for (int si = 0; si < ns; ++si)
    for (int ti = 0; ti < nt; ++ti) {
        for (int b = 0; b < nb; ++b) {
            const float bet = beta[b];
            double it = (ti + 0.5) * rt - ct;
            double is = (si + 0.5) * rs - cs;
            const double sb = sinf(bet), cb = cosf(bet);   /* float overloads, as in the reference */
            double dect_t = it * cb + is * sb;
            double dect_s = -it * sb + is * cb;
            double lr = D / (D - dect_s);
            double p = dect_t * lr;
            double src_t = ct - D * sb, src_s = cs + D * cb;
            double end_t = it + ct, end_s = is + cs;
            double tlo = ti * rt, thi = (ti + 1) * rt, slo = si * rs, shi = (si + 1) * rs;
            for (int zi = 0; zi < nz; ++zi) {
                double iz = (zi + 0.5) * rz - cz;
                double x = iz * lr;
                if (!((p >= g.minp) && (p < g.maxp) && (x >= g.minx) && (x < g.maxx))) continue;
                unsigned short x1 = (unsigned short)floor(fabs(x - xi[0]) / g.xint);
                unsigned short x2 = x1 + 1;
                unsigned short p1 = (unsigned short)floor(fabs(p - P[0]) / g.pint);
                unsigned short p2 = p1 + 1;
                double xg1 = fabs(x - xi[x1]), xg2 = fabs(xi[x2] - x);
                double pg1 = fabs(p - P[p1]), pg2 = fabs(P[p2] - p);
                long vb = (long)b * np * nx;
                double val = (xg2 * pg2 * R[vb + (long)x1 * np + p1] + xg1 * pg2 * R[vb + (long)x2 * np + p1]
                            + xg2 * pg1 * R[vb + (long)x1 * np + p2] + xg1 * pg1 * R[vb + (long)x2 * np + p2])
                            / (g.pint * g.xint);
                /* chord through the voxel: entry on a low face, :243-283 */
                double src_z = cz, end_z = iz + cz;
                double zlo = zi * rz, zhi = (zi + 1) * rz;
                double tlo_s = src_s + (tlo - src_t) * (end_s - src_s) / (end_t - src_t + OC_EPS15);
                double tlo_z = src_z + (tlo - src_t) * (end_z - src_z) / (end_t - src_t + OC_EPS15);
                double slo_t = src_t + (slo - src_s) * (end_t - src_t) / (end_s - src_s + OC_EPS15);
                double slo_z = src_z + (slo - src_s) * (end_z - src_z) / (end_s - src_s + OC_EPS15);
                double zlo_t = src_t + (zlo - src_z) * (end_t - src_t) / (end_z - src_z + OC_EPS15);
                double zlo_s = src_s + (zlo - src_z) * (end_s - src_s) / (end_z - src_z + OC_EPS15);
                double T1, S1, Z1;
                if (tlo_s >= slo && tlo_s <= shi && tlo_z >= zlo && tlo_z <= zhi) { T1 = tlo; S1 = tlo_s; Z1 = tlo_z; }
                else if (slo_t >= tlo && slo_t <= thi && slo_z >= zlo && slo_z <= zhi) { T1 = slo_t; S1 = slo; Z1 = slo_z; }
                else if (zlo_t >= tlo && zlo_t <= thi && zlo_s >= slo && zlo_s <= shi) { T1 = zlo_t; S1 = zlo_s; Z1 = zlo; }
                else break;   /* the reference returns: the rest of this column is skipped for this view, :277-281 */
                double len = 2 * sqrt(dist3sq(T1, S1, Z1, end_t, end_s, end_z));
                long id = (long)zi * nt * ns + (long)si * nt + ti;
                disp[id] = (float)((double)disp[id] + val * len);
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Shepp-Logan-form ramp filter taps, GFunction (FDK.cu:6-19; identical in   */
/* FBPfan.cu:6-19 and FBPparallel.cu:6-19).  g has 2*np-1 taps, centre np-1. */
/* ------------------------------------------------------------------------ */
OC_API void oc_sl_filter(float *g, float pint, int np)
{
    for (int n = 0; n < np; ++n) {
        if (n == 0) g[np - 1] = (float)(1.0 / sq(OC_PI * pint));
        else {
            float v = (float)(-1.0 / sq(pint * OC_PI) / (4 * sq(n) - 1));
            g[np - 1 - n] = v;
            g[np - 1 + n] = v;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* FDK: cosine pre-weight + S-L ramp + weighted bilinear BP.                 */
/* PreWeightFilter (FDK.cu:21-48), BackProjection (FDK.cu:50-126).          */
/* stage outputs are exposed for the parity tests: rcov may be NULL.        */
/* ------------------------------------------------------------------------ */
/* The pre-weighted input R * D / sqrt(D^2 + P^2 + xi^2), double product
   rounded to float as the in-place update of PreWeightFilter (FDK.cu:34-36). */
OC_API void oc_fdk_weight_apply(float *out, const float *R, const float *P, const float *xi, int nb,
                                int np, int nx, double D)
{
    for (long b = 0; b < nb; ++b)
        for (int x = 0; x < nx; ++x)
            for (int p = 0; p < np; ++p) {
                long i = (b * nx + x) * np + p;
                out[i] = (float)(R[i] * (D / sqrt(sq(D) + sq(P[p]) + sq(xi[x]))));
            }
}

/* Same for FBPfan: R * Rscan / sqrt(Rscan^2 + P^2) (FBPfan.cu:31-34). */
OC_API void oc_fbpfan_weight_apply(float *out, const float *R, const float *P, int nb, int np, double rscan)
{
    for (long b = 0; b < nb; ++b)
        for (int p = 0; p < np; ++p)
            out[b * np + p] = (float)(R[b * np + p] * (rscan / sqrt(sq(rscan) + sq(P[p]))));
}

/* Filter-stage options beyond the reference's GPU path.  NULL / 0 fields
   give the reference's behaviour. */
typedef struct {
    const float *pw;      /* short-scan weights [view][np], or NULL */
    int pw_div;           /* rows per view */
    const double *win;    /* smoothing window, or NULL */
    int wlen;
    double wsum;
} filt_opts;

/* Pre-weight + ramp convolution of detector rows, shared by FDK and FBPfan.
   mode 0 ("clean"): every output sees the fully pre-weighted row.
   mode 1 ("launch order"): the reference weights the row in place inside the
   kernel that convolves it, one P-tile per launch and `limit` taps per chunk
   (FDK.cu:21-48 with the launch loops :333-477; FBPfan.cu:21-43 with
   :286-420).  Model: a P-tile sees earlier tiles fully weighted, its own tile
   weighted once per chunk processed so far, later tiles unweighted; rows of
   the residual row tile (row % rowmod beyond the last full block of
   row_block rows) run the residual P-tile first.
   Options: short-scan weights multiply the raw row (float product) before any
   of this; the smoothing window runs over the finished filtered row. */
static void filter_rows(float *rcov, const float *R, long nrow, int np, float pint, const float *g,
                        const double *wd, int wrows, int tile, int limit, int row_block, int rowmod,
                        int mode, const filt_opts *o)
{
#pragma omp parallel
    {
        float *cur = (float *)malloc(sizeof(float) * np);
        float *tmp = (float *)malloc(sizeof(float) * np);
        int *pos = (int *)malloc(sizeof(int) * (np / tile + 2));
#pragma omp for schedule(dynamic, 4)
        for (long row = 0; row < nrow; ++row) {
            const float *in = R + row * np;
            const double *w = wd + (row % wrows) * np;
            const float *pw = o->pw ? o->pw + (row / o->pw_div) * np : NULL;
            float *out = rcov + row * np;
            for (int p = 0; p < np; ++p) out[p] = 0.0f;
            for (int p = 0; p < np; ++p) tmp[p] = pw ? in[p] * pw[p] : in[p];
            int gtime = (int)ceil(1.0 * np / limit);
            if (mode == 0) {
                for (int p = 0; p < np; ++p) cur[p] = (float)(tmp[p] * w[p]);
                for (int c = 0; c < gtime; ++c) {
                    int g0 = c * limit, g1 = (c == gtime - 1) ? np : (c + 1) * limit;
                    for (int p = 0; p < np; ++p) {
                        double acc = 0;
                        for (int q = g0; q < g1; ++q) acc += cur[q] * g[(np - 1) + p - q];
                        out[p] = (float)((double)out[p] + pint * acc);
                    }
                }
            } else {
                int nfull = np / tile, resid = np % tile, ntiles = nfull + (resid ? 1 : 0);
                int ridx = (int)(row % rowmod);
                int in_resid_rows = (rowmod % row_block) != 0 && ridx >= (rowmod / row_block) * row_block;
                for (int k = 0; k < ntiles; ++k)
                    pos[k] = (in_resid_rows && resid) ? ((k == nfull) ? 0 : k + 1) : k;
                for (int p = 0; p < np; ++p) cur[p] = tmp[p];
                for (int step = 0; step < ntiles; ++step) {
                    int k = 0;
                    for (int j = 0; j < ntiles; ++j) if (pos[j] == step) k = j;
                    int p0 = k * tile, p1 = (k == nfull) ? np : p0 + tile;
                    for (int c = 0; c < gtime; ++c) {
                        for (int p = p0; p < p1; ++p) cur[p] = (float)(cur[p] * w[p]);
                        int g0 = c * limit, g1 = (c == gtime - 1) ? np : (c + 1) * limit;
                        for (int p = p0; p < p1; ++p) {
                            double acc = 0;
                            for (int q = g0; q < g1; ++q) acc += cur[q] * g[(np - 1) + p - q];
                            out[p] = (float)((double)out[p] + pint * acc);
                        }
                    }
                }
            }
            if (o->win) {
                /* out[p] = sum_i win[i] x[p + i - wlen/2] / wsum, x zero outside */
                for (int p = 0; p < np; ++p) tmp[p] = out[p];
                int c = o->wlen / 2;
                for (int p = 0; p < np; ++p) {
                    double acc = 0;
                    for (int i = 0; i < o->wlen; ++i) {
                        int k = p + i - c;
                        if (k >= 0 && k < np) acc += (double)tmp[k] * o->win[i];
                    }
                    out[p] = (float)(acc / o->wsum);
                }
            }
        }
        free(cur);
        free(tmp);
        free(pos);
    }
}

/* Ramp taps by kind: 0 Shepp-Logan (GFunction, as oc_sl_filter); 1 Ram-Lak,
   the kernel of FBP_parallel.m:241-251 (h0 = 1/(2 dP)^2, even n 0, odd n
   -1/(n pi dP)^2) times 1/2, the amplitude convention of the S-L taps. */
OC_API void oc_ramp_taps(float *g, int kind, float pint, int np)
{
    if (kind != 1) { oc_sl_filter(g, pint, np); return; }
    for (int n = 0; n < np; ++n) {
        double v;
        if (n == 0) v = 0.5 / ((2.0 * pint) * (2.0 * pint));
        else if (n % 2 == 0) v = 0.0;
        else { double a = (double)n * OC_PI * pint; v = -0.5 / (a * a); }
        g[np - 1 - n] = (float)v;
        g[np - 1 + n] = (float)v;
    }
}

/* MATLAB hamming(m): 0.54 - 0.46 cos(2 pi k / (m - 1)), k = 0..m-1 (1 for m = 1). */
OC_API void oc_hamming(double *h, int m)
{
    for (int k = 0; k < m; ++k) h[k] = (m > 1) ? 0.54 - 0.46 * cos(2.0 * OC_PI * k / (m - 1)) : 1.0;
}

/* ParkFunction.m:6-16 (beta, b0, gama in radians; fan = full fan angle). */
static double park(double beta, double b0, double gama, double fan)
{
    if (beta >= b0 && beta < b0 + fan - 2 * gama) {
        double s = sin(OC_PI / 4 * beta / (fan / 2 - gama));
        return s * s;
    } else if (beta >= b0 + fan - 2 * gama && beta <= b0 + OC_PI - 2 * gama) {
        return 1.0;
    } else if (beta > b0 + OC_PI - 2 * gama && beta <= b0 + OC_PI + fan) {
        double s = sin(OC_PI / 4 * (OC_PI + fan - beta) / (fan / 2 + gama));
        return s * s;
    }
    return 0.0;
}

/* 2 x ParkFunction weight per (view, bin): gama = atan(P / D), b0 = beta[0],
   fan = |atan(P_last / D) - atan(P_0 / D)|; the factor 2 restores the full
   amplitude of a once-covered line under the half-amplitude ramp taps. */
OC_API void oc_parker_weights(float *pw, const float *beta, int nb, const float *P, int np, double D)
{
    double fan = fabs(atan((double)P[np - 1] / D) - atan((double)P[0] / D));
    for (int v = 0; v < nb; ++v)
        for (int p = 0; p < np; ++p)
            pw[(long)v * np + p] = (float)(2.0 * park(beta[v], beta[0], atan((double)P[p] / D), fan));
}

static void make_opts(filt_opts *o, float **pwbuf, double **winbuf, const float *beta, int nb,
                      const float *P, int np, double D, int rows_per_view, int wlen, int short_scan)
{
    memset(o, 0, sizeof(*o));
    *pwbuf = NULL;
    *winbuf = NULL;
    if (short_scan) {
        *pwbuf = (float *)malloc(sizeof(float) * (size_t)nb * np);
        oc_parker_weights(*pwbuf, beta, nb, P, np, D);
        o->pw = *pwbuf;
        o->pw_div = rows_per_view;
    }
    if (wlen > 0) {
        *winbuf = (double *)malloc(sizeof(double) * wlen);
        oc_hamming(*winbuf, wlen);
        double sum = 0;
        for (int i = 0; i < wlen; ++i) sum += (*winbuf)[i];
        o->win = *winbuf;
        o->wlen = wlen;
        o->wsum = sum;
    }
}

/* FDK filter stage with options: taps kind, smoothing window, short scan. */
OC_API void oc_fdk_filter_ex(float *rcov, const float *R, const float *xi, const float *P,
                             const float *beta, int nb, int np, int nx, double D, int mode, int kind,
                             int wlen, int short_scan, int nthreads)
{
    set_threads(nthreads);
    det_range rg = make_range(P, np, xi, nx, NULL, 0);
    float *g = (float *)malloc(sizeof(float) * (2 * np - 1));
    oc_ramp_taps(g, kind, rg.pint, np);
    /* the weight depends on (xi, P) only; the reference recomputes it per launch
       in double and multiplies in double, so keep it in double here */
    double *wd = (double *)malloc(sizeof(double) * (size_t)nx * np);
    for (int x = 0; x < nx; ++x)
        for (int p = 0; p < np; ++p)
            wd[(long)x * np + p] = D / sqrt(sq(D) + sq(P[p]) + sq(xi[x]));
    filt_opts o;
    float *pwb;
    double *winb;
    make_opts(&o, &pwb, &winb, beta, nb, P, np, D, nx, wlen, short_scan);
    filter_rows(rcov, R, (long)nb * nx, np, rg.pint, g, wd, nx, 256, 2048, 256, nx, mode, &o);  /* FDK.h:22-24 */
    free(pwb);
    free(winb);
    free(wd);
    free(g);
}

OC_API void oc_fdk_filter(float *rcov, const float *R, const float *xi, const float *P, int nb,
                          int np, int nx, double D, int mode, int nthreads)
{
    oc_fdk_filter_ex(rcov, R, xi, P, NULL, nb, np, nx, D, mode, 0, 0, 0, nthreads);
}

/* FDK backprojection of filtered projections (FDK.cu:50-126 with the view
   loop :508-582).  sticky=1 keeps the reference's behaviour that a voxel
   whose projection leaves the detector re-adds the last in-range value of its
   column (Display_pBeta is not reset, :73 and :100-123); sticky=0 adds 0. */
OC_API void oc_fdk_bp(float *disp, const float *rcov, const float *xi, const float *P,
                      const float *beta, double D, int nb, int np, int nx, const double *size,
                      int nt, int ns, int nz, int sticky, int nthreads)
{
    set_threads(nthreads);
    det_range g = make_range(P, np, xi, nx, beta, nb);
    const double rt = 1.0 * size[0] / nt, rs = 1.0 * size[1] / ns, rz = 1.0 * size[2] / nz;
    const double ct = size[0] / 2, cs = size[1] / 2, cz = size[2] / 2;
    memset(disp, 0, sizeof(float) * (size_t)nt * ns * nz);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
    for (int si = 0; si < ns; ++si)
    for (int ti = 0; ti < nt; ++ti) {
        for (int b = 0; b < nb; ++b) {
            const float bet = beta[b];
            double it = (ti + 0.5) * rt - ct;
            double is = (si + 0.5) * rs - cs;
            const double sb = sinf(bet), cb = cosf(bet);   /* float overloads, as in the reference */
            double dect_t = it * cb + is * sb;
            double dect_s = -it * sb + is * cb;
            double lr = D / (D - dect_s);
            double p = dect_t * lr;
            double val = 0;
            for (int zi = 0; zi < nz; ++zi) {
                double iz = (zi + 0.5) * rz - cz;
                double x = iz * lr;
                if ((p >= g.minp) && (p < g.maxp) && (x >= g.minx) && (x < g.maxx)) {
                    unsigned int x1 = (unsigned int)floor(fabs(x - xi[0]) / g.xint), x2 = x1 + 1;
                    unsigned int p1 = (unsigned int)floor(fabs(p - P[0]) / g.pint), p2 = p1 + 1;
                    double xg1 = fabs(x - xi[x1]), xg2 = fabs(xi[x2] - x);
                    double pg1 = fabs(p - P[p1]), pg2 = fabs(P[p2] - p);
                    double weight = sqrt(1 + 0 * sq(iz) / (sq(D + dect_s) + sq(dect_t)));
                    long vb = (long)b * np * nx;
                    val = (xg2 * pg2 * rcov[vb + (long)x1 * np + p1] + xg1 * pg2 * rcov[vb + (long)x2 * np + p1]
                         + xg2 * pg1 * rcov[vb + (long)x1 * np + p2] + xg1 * pg1 * rcov[vb + (long)x2 * np + p2])
                         / (g.pint * g.xint) * sq(lr) * g.bint * weight;
                } else if (!sticky) {
                    val = 0;
                }
                long id = (long)zi * nt * ns + (long)si * nt + ti;
                disp[id] = (float)((double)disp[id] + val);
            }
        }
    }
}

/* full FDK chain as FDKpro (FDK.cu:129-611) */
OC_API void oc_fdk(float *disp, const float *R, const float *xi, const float *P, const float *beta,
                   double D, int nb, int np, int nx, const double *size, int nt, int ns, int nz,
                   int filter_mode, int sticky, int nthreads)
{
    float *rcov = (float *)malloc(sizeof(float) * (size_t)nb * np * nx);
    oc_fdk_filter(rcov, R, xi, P, nb, np, nx, D, filter_mode, nthreads);
    oc_fdk_bp(disp, rcov, xi, P, beta, D, nb, np, nx, size, nt, ns, nz, sticky, nthreads);
    free(rcov);
}

/* ------------------------------------------------------------------------ */
/* 2D fan-beam Siddon forward projection, ProjectionFan (ProjectionFan_2D.cu:8-220). */
/* ------------------------------------------------------------------------ */
static double fan_ray(const float *pic, int nt, int ns, double ct, double cs, const double res[2],
                      double P, double beta, double D)
{
    const double r1 = res[0], r2 = res[1];
    double src_t = ct + D * sin(-beta);
    double src_s = cs + D * cos(-beta);
    double theta = atan(P / D);
    double smax = 2 * D;
    double end_t = ct + smax * sin(theta) * cos(-beta) + (D - smax * cos(theta)) * sin(-beta);
    double end_s = cs - smax * sin(theta) * sin(-beta) + (D - smax * cos(theta)) * cos(-beta);
    double dt = end_t - src_t, ds = end_s - src_s;
    double t2s = (dt == 0) ? ds / (dt + OC_EPS15) : ds / dt;
    double s2t = (ds == 0) ? dt / (ds + OC_EPS15) : dt / ds;
    t2s = slope_clamp(t2s); s2t = slope_clamp(s2t);
    int sig_t = end_t >= src_t ? 1 : -1;
    int sig_s = end_s >= src_s ? 1 : -1;
    double tlo = 0, thi = nt * r1, slo = 0, shi = ns * r2;
    double tlo_s = src_s + (tlo - src_t) * t2s, thi_s = src_s + (thi - src_t) * t2s;
    double slo_t = src_t + (slo - src_s) * s2t, shi_t = src_t + (shi - src_s) * s2t;
    int ok[4] = {tlo_s >= 0 && tlo_s <= shi, thi_s >= 0 && thi_s <= shi,
                 slo_t >= 0 && slo_t <= thi, shi_t >= 0 && shi_t <= thi};
    double ft[4] = {tlo, thi, slo_t, shi_t}, fs[4] = {tlo_s, thi_s, slo, shi};
    int first = -1, second = -1;
    for (int f = 0; f < 4; ++f) if (ok[f]) { first = f; break; }
    if (first < 0 || first == 3) return 0.0;   /* :117-121 (shi alone is never a first face) */
    for (int f = first + 1; f < 4; ++f) if (ok[f]) { second = f; break; }
    double T1 = ft[first], S1 = fs[first], T2 = 0, S2 = 0;
    if (second >= 0) { T2 = ft[second]; S2 = fs[second]; }
    double Ts, Ss;
    if (dist2sq(T1, S1, src_t, src_s) >= dist2sq(T2, S2, src_t, src_s)) { Ts = T2; Ss = S2; }
    else { Ts = T1; Ss = S1; }
    double ray = 0;
    double tc = Ts / r1, sc = Ss / r2;
    int up_t = (1 + sig_t) / 2, up_s = (1 + sig_s) / 2;
    for (int i = 0; i < nt + ns - 1; ++i) {           /* :162-216 */
        short gt, gs;
        if (fabs(tc - round(tc)) < OC_EPS15) gt = (short)(round(tc) + sig_t);
        else gt = (short)(floor(tc) + up_t);
        double gt_s = (src_s + (gt * r1 - src_t) * t2s) / r2;
        if (fabs(sc - round(sc)) < OC_EPS15) gs = (short)(round(sc) + sig_s);
        else gs = (short)(floor(sc) + up_s);
        double gs_t = (src_t + (gs * r2 - src_s) * s2t) / r1;
        double w, nt_, ns_;
        if (dist2sq(gt, gt_s, tc, sc) <= dist2sq(gs_t, gs, tc, sc)) {
            w = sqrt(dist2sq(gt * r1, gt_s * r2, tc * r1, sc * r2));
            nt_ = gt; ns_ = gt_s;
        } else {
            w = sqrt(dist2sq(gs_t * r1, gs * r2, tc * r1, sc * r2));
            nt_ = gs_t; ns_ = gs;
        }
        short it = (short)floor((nt_ + tc) / 2), is = (short)floor((ns_ + sc) / 2);
        tc = nt_; sc = ns_;
        if (it >= 0 && it < nt && is >= 0 && is < ns) ray += w * pic[(long)is * nt + it];
        else break;
    }
    return ray;
}

OC_API void oc_fan_fp(const float *pic, double *proj, const double *beta, const double *P, int nt,
                      int ns, double ct, double cs, int nb, int np, double D, const double *res,
                      int nthreads)
{
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
    for (long r = 0; r < (long)nb * np; ++r) {
        int ip = (int)(r % np), ib = (int)(r / np);
        proj[r] = fan_ray(pic, nt, ns, ct, cs, res, P[ip], beta[ib], D);
    }
}

/* ------------------------------------------------------------------------ */
/* 2D parallel-beam Siddon, ProjectionParallel (ProjectionParallel_2D.cu:9-253). */
/* ------------------------------------------------------------------------ */
static double par_ray(const float *pic, int h, int wd, double cy, double cx, const double res[2],
                      double t, double theta, double smax)
{
    double xs = cx + t * cos(-theta) + (-smax) * sin(-theta);
    double ys = cy - t * sin(-theta) + (-smax) * cos(-theta);
    double xe = cx + t * cos(-theta) + smax * sin(-theta);
    double ye = cy - t * sin(-theta) + smax * cos(-theta);
    double x2y = (xe - xs == 0) ? (ye - ys) / (xe - xs + OC_EPS30) : (ye - ys) / (xe - xs);
    double y2x = (ye - ys == 0) ? (xe - xs) / (ye - ys + OC_EPS30) : (xe - xs) / (ye - ys);
    x2y = slope_clamp(x2y); y2x = slope_clamp(y2x);
    int sig_y = (ye >= ys) ? 1 : (ye < ys ? -1 : 0);
    int sig_x = (xe >= xs) ? 1 : (xe < xs ? -1 : 0);
    double xlo = 0, xhi = wd * res[1], ylo = 0, yhi = h * res[0];
    double ylo_x = xs + (ylo - ys) * y2x, yhi_x = xs + (yhi - ys) * y2x;
    double xlo_y = ys + (xlo - xs) * x2y, xhi_y = ys + (xhi - xs) * x2y;
    /* face search order of :77-121: ylo, yhi, xlo, xhi */
    int ok[4] = {ylo_x >= 0 && ylo_x <= xhi, yhi_x >= 0 && yhi_x <= xhi,
                 xlo_y >= 0 && xlo_y <= yhi, xhi_y >= 0 && xhi_y <= yhi};
    double fx[4] = {ylo_x, yhi_x, xlo, xhi}, fy[4] = {ylo, yhi, xlo_y, xhi_y};
    int first = -1;
    for (int f = 0; f < 4; ++f) if (ok[f]) { first = f; break; }
    if (first < 0 || first == 3) return 0.0;
    /* the reference looks for the second point among: after ylo -> xlo, xhi, yhi;
       after yhi -> xlo, xhi; after xlo -> xhi */
    static const int order[3][3] = {{2, 3, 1}, {2, 3, -1}, {3, -1, -1}};
    int second = -1;
    for (int k = 0; k < 3; ++k) {
        int f = order[first][k];
        if (f >= 0 && ok[f]) { second = f; break; }
    }
    double X1 = fx[first], Y1 = fy[first], X2 = 0, Y2 = 0;
    if (second >= 0) { X2 = fx[second]; Y2 = fy[second]; }
    double Xs, Ys;
    if (dist2sq(X1, Y1, xs, ys) >= dist2sq(X2, Y2, xs, ys)) { Xs = X2; Ys = Y2; }
    else { Xs = X1; Ys = Y1; }
    double ray = 0;
    double xc = Xs / res[1], yc = Ys / res[0];
    int up_x = (1 + sig_x) / 2, up_y = (1 + sig_y) / 2;
    for (int i = 0; i < h + wd - 1; ++i) {           /* :163-243 */
        short gx, gy;
        if (fabs(xc - round(xc)) < OC_ERR5) gx = (short)(round(xc) + sig_x);
        else gx = (short)(floor(xc) + up_x);
        double gx_y = (ys + (gx * res[1] - xs) * x2y) / res[0];
        if (fabs(yc - round(yc)) < OC_ERR5) gy = (short)(round(yc) + sig_y);
        else gy = (short)(floor(yc) + up_y);
        double gy_x = (xs + (gy * res[0] - ys) * y2x) / res[1];
        double w, nx_, ny_;
        if (dist2sq(gx, gx_y, xc, yc) >= dist2sq(gy_x, gy, xc, yc)) {
            w = sqrt(dist2sq(gy_x * res[1], gy * res[0], xc * res[1], yc * res[0]));
            nx_ = gy_x; ny_ = gy;
        } else {
            w = sqrt(dist2sq(gx * res[1], gx_y * res[0], xc * res[1], yc * res[0]));
            nx_ = gx; ny_ = gx_y;
        }
        short ix = (short)floor((nx_ + xc) / 2), iy = (short)floor((ny_ + yc) / 2);
        xc = nx_; yc = ny_;
        if (ix >= 0 && ix < wd && iy >= 0 && iy < h) ray += w * pic[(long)iy * wd + ix];
        else break;
    }
    return ray;
}

OC_API void oc_par_fp(const float *pic, double *proj, const double *theta, const double *trange,
                      int h, int wd, double cy, double cx, int nth, int nt, const double *res,
                      int nthreads)
{
    set_threads(nthreads);
    double a = fabs(trange[0]), b = fabs(trange[nt - 1]);
    double smax = a > b ? a : b;
#pragma omp parallel for schedule(dynamic, 64)
    for (long r = 0; r < (long)nth * nt; ++r) {
        int it = (int)(r % nt), ith = (int)(r / nt);
        proj[r] = par_ray(pic, h, wd, cy, cx, res, trange[it], theta[ith], smax);
    }
}

/* ------------------------------------------------------------------------ */
/* 2D fan voxel-driven backprojection with the reference's chord-like       */
/* weight, BackProjection (BackprojectionFan2D.cu:7-116).                   */
/* ------------------------------------------------------------------------ */
OC_API void oc_fan_bp(float *disp, const float *R, const float *P, const float *beta, int nb,
                      int np, const double *size, int nt, int ns, double rscan, int nthreads)
{
    set_threads(nthreads);
    det_range g = make_range(P, np, NULL, 0, beta, nb);
    const double rt = 1.0 * size[0] / nt, rs = 1.0 * size[1] / ns;
    const double ct = size[0] / 2, cs = size[1] / 2;
    memset(disp, 0, sizeof(float) * (size_t)nt * ns);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
    for (int si = 0; si < ns; ++si)
    for (int ti = 0; ti < nt; ++ti) {
        for (int b = 0; b < nb; ++b) {
            const float bet = beta[b];
            double it = (ti + 0.5) * rt - ct, is = (si + 0.5) * rs - cs;
            const double sb = sinf(bet), cb = cosf(bet);   /* float overloads, as in the reference */
            double p = it * cb + is * sb;
            double s = -it * sb + is * cb;
            double u = (rscan - s) / rscan;
            double pd = p / u;
            double val = 0;
            if ((pd >= g.minp) && (pd < g.maxp)) {
                unsigned int p1 = (unsigned int)floor(fabs(pd - P[0]) / g.pint), p2 = p1 + 1;
                double pg1 = fabs(pd - P[p1]), pg2 = fabs(P[p2] - pd);
                val = (pg2 * R[(long)b * np + p1] + pg1 * R[(long)b * np + p2]) / g.pint;
            }
            double src_t = ct - rscan * sb, src_s = cs + rscan * cb;
            double th = atan(pd / rscan);
            double smax = 2 * rscan;
            double end_t = ct + smax * sin(th) * cb - (rscan - smax * cos(th)) * sb;
            double end_s = cs + smax * sin(th) * sb + (rscan - smax * cos(th)) * cb;
            double dt = end_t - src_t, ds = end_s - src_s;
            double t2s = (dt == 0) ? ds / (dt + OC_EPS15) : ds / dt;
            double s2t = (ds == 0) ? dt / (ds + OC_EPS15) : dt / ds;
            t2s = slope_clamp(t2s); s2t = slope_clamp(s2t);
            double tlo = ti * rt, thi = (ti + 1) * rt, slo = si * rs, shi = (si + 1) * rs;
            double tlo_s = src_s + (tlo - src_t) * t2s;
            double slo_t = src_t + (slo - src_s) * s2t;
            double T1, S1;
            if (tlo_s >= 0 && tlo_s <= shi) { T1 = tlo; S1 = tlo_s; }       /* :95-107 */
            else if (slo_t >= 0 && slo_t <= thi) { T1 = slo_t; S1 = slo; }
            else continue;
            double len = 2 * sqrt(dist2sq(T1, S1, end_t, end_s));
            long id = (long)si * nt + ti;
            disp[id] = (float)((double)disp[id] + val * len);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* FBPfan: weight + S-L filter + 1/U^2 weighted BP (FBPfan.cu:21-96).       */
/* ------------------------------------------------------------------------ */
OC_API void oc_fbpfan_filter_ex(float *rcov, const float *R, const float *P, const float *beta, int nb,
                                int np, double rscan, int mode, int kind, int wlen, int short_scan,
                                int nthreads)
{
    set_threads(nthreads);
    float pint = fabsf(P[1] - P[0]);
    float *g = (float *)malloc(sizeof(float) * (2 * np - 1));
    oc_ramp_taps(g, kind, pint, np);
    double *w = (double *)malloc(sizeof(double) * np);
    for (int p = 0; p < np; ++p) w[p] = rscan / sqrt(sq(rscan) + sq(P[p]));
    filt_opts o;
    float *pwb;
    double *winb;
    make_opts(&o, &pwb, &winb, beta, nb, P, np, rscan, 1, wlen, short_scan);
    filter_rows(rcov, R, nb, np, pint, g, w, 1, 128, 1024, 128, nb, mode, &o);   /* FBPfan.h:24-26 */
    free(pwb);
    free(winb);
    free(w);
    free(g);
}

OC_API void oc_fbpfan_filter(float *rcov, const float *R, const float *P, int nb, int np,
                             double rscan, int mode, int nthreads)
{
    oc_fbpfan_filter_ex(rcov, R, P, NULL, nb, np, rscan, mode, 0, 0, 0, nthreads);
}

OC_API void oc_fbpfan_bp(float *disp, const float *rcov, const float *P, const float *beta, int nb,
                         int np, const double *size, int nt, int ns, double rscan, int nthreads)
{
    set_threads(nthreads);
    det_range g = make_range(P, np, NULL, 0, beta, nb);
    const double rt = 1.0 * size[0] / nt, rs = 1.0 * size[1] / ns;
    const double ct = size[0] / 2, cs = size[1] / 2;
    memset(disp, 0, sizeof(float) * (size_t)nt * ns);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
    for (int si = 0; si < ns; ++si)
    for (int ti = 0; ti < nt; ++ti) {
        for (int b = 0; b < nb; ++b) {
            const float bet = beta[b];
            double it = (ti + 0.5) * rt - ct, is = (si + 0.5) * rs - cs;
            const double sb = sinf(bet), cb = cosf(bet);   /* float overloads, as in the reference */
            double p = it * cb + is * sb;
            double s = -it * sb + is * cb;
            double u = (rscan - s) / rscan;
            double pd = p / u;
            double val = 0;
            if ((pd >= g.minp) && (pd < g.maxp)) {
                unsigned int p1 = (unsigned int)floor(fabs(pd - P[0]) / g.pint), p2 = p1 + 1;
                double pg1 = fabs(pd - P[p1]), pg2 = fabs(P[p2] - pd);
                val = (pg2 * rcov[(long)b * np + p1] + pg1 * rcov[(long)b * np + p2]) / (sq(u) * g.pint) * g.bint;
            }
            long id = (long)si * nt + ti;
            disp[id] = (float)((double)disp[id] + val);
        }
    }
}

OC_API void oc_fbpfan(float *disp, const float *R, const float *P, const float *beta, int nb, int np,
                      const double *size, int nt, int ns, double rscan, int filter_mode, int nthreads)
{
    float *rcov = (float *)malloc(sizeof(float) * (size_t)nb * np);
    oc_fbpfan_filter(rcov, R, P, nb, np, rscan, filter_mode, nthreads);
    oc_fbpfan_bp(disp, rcov, P, beta, nb, np, size, nt, ns, rscan, nthreads);
    free(rcov);
}

/* ------------------------------------------------------------------------ */
/* FBPparallel: S-L filter (no weight) + linear-interpolation BP            */
/* (FBPparallel.cu:21-89).                                                   */
/* ------------------------------------------------------------------------ */
OC_API void oc_fbppar(float *disp, const float *R, const float *T, const float *theta, int nth,
                      int nt_det, const double *size, int nt, int ns, int nthreads)
{
    set_threads(nthreads);
    float tint = fabsf(T[1] - T[0]);
    float thint = nth > 1 ? fabsf(theta[1] - theta[0]) : 0.0f;
    float maxt = T[0] > T[nt_det - 1] ? T[0] : T[nt_det - 1];
    float mint = T[0] < T[nt_det - 1] ? T[0] : T[nt_det - 1];
    float *g = (float *)malloc(sizeof(float) * (2 * nt_det - 1));
    oc_sl_filter(g, tint, nt_det);
    float *rcov = (float *)malloc(sizeof(float) * (size_t)nth * nt_det);
    const int limit = 2048;   /* FBPparallel.h:26 */
    int gtime = (int)ceil(1.0 * nt_det / limit);
#pragma omp parallel for schedule(dynamic, 4)
    for (int row = 0; row < nth; ++row) {
        const float *in = R + (long)row * nt_det;
        float *out = rcov + (long)row * nt_det;
        for (int p = 0; p < nt_det; ++p) out[p] = 0.0f;
        for (int c = 0; c < gtime; ++c) {
            int g0 = c * limit, g1 = (c == gtime - 1) ? nt_det : (c + 1) * limit;
            for (int p = 0; p < nt_det; ++p) {
                double acc = 0;
                for (int q = g0; q < g1; ++q) acc += in[q] * g[(nt_det - 1) + p - q];
                out[p] = (float)((double)out[p] + tint * acc);
            }
        }
    }
    const double rt = 1.0 * size[0] / nt, rs = 1.0 * size[1] / ns;
    const double ct = size[0] / 2, cs = size[1] / 2;
    memset(disp, 0, sizeof(float) * (size_t)nt * ns);
#pragma omp parallel for collapse(2) schedule(dynamic, 16)
    for (int si = 0; si < ns; ++si)
    for (int ti = 0; ti < nt; ++ti) {
        for (int b = 0; b < nth; ++b) {
            const float th = theta[b];
            double it = (ti + 0.5) * rt - ct, is = (si + 0.5) * rs - cs;
            double t = it * (double)cosf(th) + is * (double)sinf(th);   /* float Theta */
            double val = 0;
            if ((t >= mint) && (t < maxt)) {
                unsigned int t1 = (unsigned int)floor(fabs(t - T[0]) / tint), t2 = t1 + 1;
                double d1 = fabs(t - T[t1]), d2 = fabs(T[t2] - t);
                val = (d2 * rcov[(long)b * nt_det + t1] + d1 * rcov[(long)b * nt_det + t2]) / tint * thint;
            }
            long id = (long)si * nt + ti;
            disp[id] = (float)((double)disp[id] + val);
        }
    }
    free(rcov);
    free(g);
}

/* ------------------------------------------------------------------------ */
/* Curved-detector (equiangular) FDK of ImplementUI.cu: per-xi-row S-L taps   */
/* of the equiangular detector (GFunction :6-22), Parker short-scan weight     */
/* with the cone-tilt proportion, cosine weight and convolution               */
/* (PreWeightFiltration :25-86), and the 1/L2 weighted backprojection         */
/* (BackProjection :88-150).  All double, as the reference (R is double).      */
/* Layouts: R and rcov [view][xi][gamma], display [z][s][t]; Size holds the   */
/* integer extents of the display in pixels (t, s) and mm (z).                */
/* ------------------------------------------------------------------------ */
static double ui_prop(double ds2d, double xi) { return ds2d / sqrt(1.0 * ds2d * ds2d + 1.0 * xi * xi); }

OC_API void oc_fdkui_taps(double *G, double gint, const double *xi, int lx, int lg, double ds2d)
{
    const long fs = 2L * lg - 1;
    for (int x = 0; x < lx; ++x) {
        const double gp = gint * ui_prop(ds2d, xi[x]);
        double *g = G + x * fs;
        g[lg - 1] = 2.0 / (1.0 * (OC_PI * gp) * (OC_PI * gp));
        for (int n = 1; n < lg; ++n) {
            const double sn = sin(n * gp);
            const double v = -2.0 * (1.0 * n * n) / (1.0 * OC_PI * OC_PI) / (4 * (1.0 * n * n) - 1) / (1.0 * sn * sn);
            g[lg - 1 - n] = v;
            g[lg - 1 + n] = v;
        }
    }
}

OC_API void oc_fdkui_filter(double *rcov, const double *R, const double *xi, const double *gama,
                            const double *beta, double b0, double maxg, double D, double ds2d, int lg, int nb,
                            int lx, int nthreads)
{
    set_threads(nthreads);
    const double gint = fabs(gama[1] - gama[0]);
    const long fs = 2L * lg - 1;
    double *G = (double *)malloc(sizeof(double) * fs * lx);
    oc_fdkui_taps(G, gint, xi, lx, lg, ds2d);
#pragma omp parallel
    {
        double *w = (double *)malloc(sizeof(double) * lg);
#pragma omp for schedule(dynamic, 4)
        for (long row = 0; row < (long)nb * lx; ++row) {
            const int b = (int)(row / lx), x = (int)(row % lx);
            const double pr = ui_prop(ds2d, xi[x]);
            const double bp = beta[b] * pr, b0p = b0 * pr, mgp = maxg * pr;
            const double gip = gint * pr, dp = D / pr;
            const double *in = R + row * lg;
            for (int g = 0; g < lg; ++g) {
                const double gp = gama[g] * pr;
                double W;
                if (bp >= b0p && bp < b0p + mgp - 2 * gp) {
                    const double sn = sin(OC_PI / 4 * bp / (mgp / 2 - gp));
                    W = 1.0 * sn * sn;
                } else if (bp >= b0p + mgp - 2 * gp && bp <= b0p + OC_PI - 2 * gp) {
                    W = 1;
                } else if (bp > b0p + OC_PI - 2 * gp && bp <= b0p + OC_PI + mgp) {
                    const double sn = sin(OC_PI / 4 * (OC_PI + mgp - bp) / (mgp / 2 + gp));
                    W = 1.0 * sn * sn;
                } else {
                    W = 0;
                }
                w[g] = in[g] * dp * cos(gp) * W;
            }
            const double *tap = G + x * fs;
            double *out = rcov + row * lg;
            for (int g = 0; g < lg; ++g) {
                double acc = 0;
                for (int q = 0; q < lg; ++q) acc += w[q] * tap[(lg - 1) + g - q];
                out[g] = gip * acc;
            }
        }
        free(w);
    }
    free(G);
}

OC_API void oc_fdkui_bp(double *display, const double *rcov, const int *size, int nz, const double *beta, int nb,
                        double D, double ds2d, const double *gama, int lg, const double *xi, int lx, int nthreads)
{
    set_threads(nthreads);
    const double gint = fabs(gama[1] - gama[0]), xint = fabs(xi[1] - xi[0]);
    const double bint = fabs(beta[1] - beta[0]);
    const double maxg = gama[0] > gama[lg - 1] ? gama[0] : gama[lg - 1];
    const double ming = gama[0] < gama[lg - 1] ? gama[0] : gama[lg - 1];
    const double maxx = xi[0] > xi[lx - 1] ? xi[0] : xi[lx - 1];
    const double minx = xi[0] < xi[lx - 1] ? xi[0] : xi[lx - 1];
    const int nt = size[0], ns = size[1];
    const double rz = 1.0 * size[2] / nz;
    /* integer halves, as the reference divides its int extents (:103-105) */
    const double ct = size[0] / 2, cs = size[1] / 2, cz = size[2] / 2;
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
    for (int z = 0; z < nz; ++z)
        for (int s = 0; s < ns; ++s)
            for (int t = 0; t < nt; ++t) {
                double acc = 0;
                const double it = (t - 0.5) - ct, is = (s - 0.5) - cs, iz = (z - 0.5) * rz - cz;
                for (int b = 0; b < nb; ++b) {
                    const double bt = beta[b];
                    const double st = D * cos(bt + OC_PI / 2), ss = D * sin(bt + OC_PI / 2), sz = 0;
                    const double L2 = 1.0 * (it - st) * (it - st) + 1.0 * (is - ss) * (is - ss) + 1.0 * (iz - sz) * (iz - sz);
                    const double dt = it * cos(bt) + is * sin(bt);
                    const double ds = -it * sin(bt) + is * cos(bt);
                    const double dz = iz;
                    const double X = ds2d * tan(asin(dz / sqrt(L2)));
                    const double Gm = atan(dt / (D - ds));
                    const double pr = sqrt(L2) / sqrt(L2 - 1.0 * dz * dz);
                    double val = 0;
                    if (Gm >= ming && Gm < maxg && X >= minx && X < maxx) {
                        unsigned int x1 = (unsigned int)floor(fabs(X - xi[0]) / xint), x2 = x1 + 1;
                        unsigned int g1 = (unsigned int)floor(fabs(Gm - gama[0]) / gint), g2 = g1 + 1;
                        if (x2 > (unsigned)(lx - 1)) { x2 = lx - 1; if (x1 > x2) x1 = x2; }   /* read-past-end guard */
                        if (g2 > (unsigned)(lg - 1)) { g2 = lg - 1; if (g1 > g2) g1 = g2; }
                        const double xg1 = fabs(X - xi[x1]), xg2 = fabs(xi[x2] - X);
                        const double gg1 = fabs(Gm - gama[g1]), gg2 = fabs(gama[g2] - Gm);
                        const double *rb = rcov + (long)b * lg * lx;
                        val = (xg2 * gg2 * rb[(long)x1 * lg + g1] + xg1 * gg2 * rb[(long)x2 * lg + g1]
                               + xg2 * gg1 * rb[(long)x1 * lg + g2] + xg1 * gg1 * rb[(long)x2 * lg + g2])
                              / (gint * xint) / L2 * (bint / pr);
                    }
                    acc += val;
                }
                display[((long)z * ns + s) * nt + t] = acc;
            }
}

/* ------------------------------------------------------------------------ */
/* IterativeFDK error slice (IterativeFDKerrCompute.cu:12-76): for the image  */
/* slice t, every (view, z, s) gathers, over the U samples along each ray of  */
/* the view and every detector bin P, the weighted difference between the     */
/* prior image at the ray point's depth and at the voxel's own z.  Output     */
/* [beta][z][s]; the sum is a float accumulator updated in double, U major    */
/* and P minor, as the reference's per-(view, U) launches add into it.        */
/* Arguments are those of the MEX gateway (IterativeFDKerrCompute.cpp:5-31): */
/* BetaScanInt = |b1 - b0| and dU = |U1 - U0| in float, PInt = |P1 - P0|.     */
/* ------------------------------------------------------------------------ */
OC_API void oc_iterfdk_err(const float *pic, float *err, const float *beta, const float *U,
                           const double *P, const double *G, const double *size, int nt, int ns, int nz,
                           int nb, int np, int nu, int lg, double D, int t, int nthreads)
{
    set_threads(nthreads);
    const double res[3] = {size[0] / nt, size[1] / ns, size[2] / nz};
    const double ct = size[0] / 2, cs = size[1] / 2, cz = size[2] / 2;
    const float bint = fabsf(beta[1] - beta[0]);
    const float du = fabsf(U[1] - U[0]);
    const double pint = fabs(P[1] - P[0]);
    const long plane = (long)nt * ns;
#pragma omp parallel for collapse(2) schedule(dynamic, 8)
    for (int b = 0; b < nb; ++b)
        for (int z = 0; z < nz; ++z) {
            const float sb = sinf(beta[b]), cb = cosf(beta[b]);
            for (int s = 0; s < ns; ++s) {
                const float it = (float)((t + 0.5) * res[0] - ct);
                const float is = (float)((s + 0.5) * res[1] - cs);
                const float iz = (float)((z + 0.5) * res[2] - cz);
                const float dt = it * cb + is * sb;      /* rotated frame */
                const float ds = -it * sb + is * cb;
                const float dz = iz;
                const float lr = (float)(D / (D - ds));
                const float a = dt * lr;
                float acc = 0.0f;
                for (int u = 0; u < nu; ++u) {
                    const float uu = U[u];
                    const float zr = (float)(dz + (ds - uu) * dz / (D - ds));
                    const int zi = (int)floor((zr + cz) / res[2]);
                    for (int p = 0; p < np; ++p) {
                        const double pv = P[p];
                        const int fi = (int)(floor((a - pv) / pint) + np);
                        if (fi < 0 || fi >= lg) continue;
                        const float tr = (float)(pv * (D - uu) / D);
                        const float xr = tr * cb - uu * sb;
                        const float yr = tr * sb + uu * cb;
                        const int xi = (int)floor((xr + ct) / res[0]);
                        const int yi = (int)floor((yr + cs) / res[1]);
                        if (xi < 0 || xi >= nt || yi < 0 || yi >= ns || zi < 0 || zi >= nz) continue;
                        const long col = (long)yi * nt + xi;
                        const float diff = pic[zi * plane + col] - pic[z * plane + col];
                        const double term = 0.5 * (1.0 * lr * lr) * diff * sqrt(1 + 1.0 * (pv / D) * (pv / D))
                                            * G[fi] * D / sqrt(1.0 * D * D + 1.0 * pv * pv) * du * pint * bint;
                        acc = (float)(acc + term);
                    }
                }
                err[((long)b * nz + z) * ns + s] = acc;
            }
        }
}

/* ------------------------------------------------------------------------ */
/* Independent check: textbook alpha-Siddon line integral through a t,s,z   */
/* grid (the merge-of-plane-crossings form of Siddon3D.m /                  */
/* GenSysMatCircular3D.m), FP64.  Used by the tests as a second oracle that */
/* shares no code with the reference walk above.                            */
/* ------------------------------------------------------------------------ */
OC_API double oc_siddon_line(const float *vol, int nt, int ns, int nz, const double res[3],
                             const double src[3], const double dst[3])
{
    int n[3] = {nt, ns, nz};
    double d[3] = {dst[0] - src[0], dst[1] - src[1], dst[2] - src[2]};
    double a_in = 0.0, a_out = 1.0;
    for (int k = 0; k < 3; ++k) {
        double lo = 0.0, hi = n[k] * res[k];
        if (d[k] == 0.0) {
            if (src[k] <= lo || src[k] >= hi) return 0.0;
            continue;
        }
        double a1 = (lo - src[k]) / d[k], a2 = (hi - src[k]) / d[k];
        double amin = a1 < a2 ? a1 : a2, amax = a1 < a2 ? a2 : a1;
        if (amin > a_in) a_in = amin;
        if (amax < a_out) a_out = amax;
    }
    if (a_out <= a_in) return 0.0;
    double len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    /* next crossing alphas */
    double anext[3], astep[3];
    int idx[3], step[3];
    double amid = a_in + 1e-9 * (a_out - a_in);
    for (int k = 0; k < 3; ++k) {
        double p = (src[k] + amid * d[k]) / res[k];
        int i = (int)floor(p);
        if (i < 0) i = 0;
        if (i > n[k] - 1) i = n[k] - 1;
        idx[k] = i;
        if (d[k] > 0) { step[k] = 1; anext[k] = ((i + 1) * res[k] - src[k]) / d[k]; astep[k] = res[k] / d[k]; }
        else if (d[k] < 0) { step[k] = -1; anext[k] = (i * res[k] - src[k]) / d[k]; astep[k] = -res[k] / d[k]; }
        else { step[k] = 0; anext[k] = INFINITY; astep[k] = INFINITY; }
    }
    double acc = 0.0, a = a_in;
    for (;;) {
        int k = 0;
        if (anext[1] < anext[k]) k = 1;
        if (anext[2] < anext[k]) k = 2;
        double an = anext[k] < a_out ? anext[k] : a_out;
        if (an > a) acc += (an - a) * vol[(long)idx[2] * nt * ns + (long)idx[1] * nt + idx[0]];
        a = an;
        if (a >= a_out) break;
        idx[k] += step[k];
        anext[k] += astep[k];
        if (idx[k] < 0 || idx[k] >= n[k]) break;
    }
    return acc * len;
}

/* Count of Siddon segments of each cone ray (the unit of the algorithmic
   byte count of the forward projector).  Returns the total over all rays. */
OC_API long long oc_cone_segments(int nt, int ns, int nz, const double *res, double ct, double cs,
                                  double cz, const float *beta, const float *P, const float *xi,
                                  int nb, int np, int nx, double D, int stride, int nthreads)
{
    set_threads(nthreads);
    long long total = 0;
    long nray = (long)nb * nx * np;
    if (stride < 1) stride = 1;
#pragma omp parallel for reduction(+:total) schedule(dynamic, 256)
    for (long r = 0; r < nray; r += stride) {
        int ip = (int)(r % np), ix = (int)((r / np) % nx), ib = (int)(r / ((long)np * nx));
        double sb = sin((double)beta[ib]), cb = cos((double)beta[ib]);
        double src[3] = {ct - D * sb, cs + D * cb, cz};
        double d[3] = {P[ip] * cb + D * sb, P[ip] * sb - D * cb, (double)xi[ix]};
        int n[3] = {nt, ns, nz};
        double a_in = -1e300, a_out = 1e300;
        int miss = 0;
        for (int k = 0; k < 3; ++k) {
            double lo = 0.0, hi = n[k] * res[k];
            if (d[k] == 0.0) { if (src[k] <= lo || src[k] >= hi) miss = 1; continue; }
            double a1 = (lo - src[k]) / d[k], a2 = (hi - src[k]) / d[k];
            double amin = a1 < a2 ? a1 : a2, amax = a1 < a2 ? a2 : a1;
            if (amin > a_in) a_in = amin;
            if (amax < a_out) a_out = amax;
        }
        if (miss || a_out <= a_in) continue;
        /* voxels traversed = 1 + plane crossings per axis; on the entry / exit
           face the voxel is exact, elsewhere the floor of the coordinate */
        long long c = 1;
        for (int k = 0; k < 3; ++k) {
            if (d[k] == 0.0) continue;
            double g0 = (src[k] + a_in * d[k]) / res[k], g1 = (src[k] + a_out * d[k]) / res[k];
            double lo_k = fmin((0 - src[k]) / d[k], (n[k] * res[k] - src[k]) / d[k]);
            double hi_k = fmax((0 - src[k]) / d[k], (n[k] * res[k] - src[k]) / d[k]);
            long long s0 = (lo_k == a_in) ? (d[k] > 0 ? 0 : n[k] - 1) : (long long)floor(g0);
            long long e0 = (hi_k == a_out) ? (d[k] > 0 ? n[k] - 1 : 0) : (long long)floor(g1);
            if (s0 < 0) s0 = 0;
            if (s0 > n[k] - 1) s0 = n[k] - 1;
            if (e0 < 0) e0 = 0;
            if (e0 > n[k] - 1) e0 = n[k] - 1;
            c += s0 > e0 ? s0 - e0 : e0 - s0;
        }
        total += c;
    }
    return total * stride;
}
