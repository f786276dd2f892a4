// kernels.cuh -- kernel launchers of libctgb and the geometry they take.
#pragma once
#include "cone_geom.cuh"

namespace ct {

// 2D fan / parallel geometry (ProjectionFan_2D.cpp, BackprojectionFan2D.cpp,
// FBPfan.cpp, ProjectionParallel_2D.cpp, FBPparallel.cpp argument sets).
struct FanGeom {
    int nt, ns;              // image size (t fastest)
    int nb, np;              // views, detector bins
    double size[2];          // image extent in mm along t and s
    double res[2];           // pixel pitch
    double D;                // source to centre (Rscan); unused for parallel beam
    const double2 *trig_d;   // per view (sin, cos) of the double angles (forward projectors)
    const double *Pd;        // double detector coordinates (forward projectors)
    const float2 *trig_f;    // per view (sinf, cosf) of the float angles (backprojectors)
    const float *Pf;         // float detector coordinates (backprojectors)
    float pint, bint, minp, maxp, p0, psgn;
    int parallel;            // 1: parallel-beam geometry
    double smax;             // parallel: max |t| (ProjectionParallel_2D.cu:25)
    // derived on the host before each launch (fan_geom_derive): 1 / res and n * res
    // per axis, so the per-ray set-up divides nothing; and float-float (hi, lo)
    // copies of res, size / 2, D and 1 / pint for the backprojector's
    // near-boundary recompute, so that it runs no FP64
    double ires[2], ext[2];
    float2 res_ff[2], hsize_ff[2], D_ff, ipint_ff;
    // the walk set-up of every ray (fan_ray_table_launch), or null: computed per ray
    const struct FanRay *ray_tab;
};

// The forward walk's set-up of one 2D ray, as the FP64 slab test makes it
// (siddon.cuh): first crossings and steps per axis, exit parameter, |d|,
// entry pixel, segment count, index steps and flags (bit 0 hit, bit 1 grazing).
struct __align__(16) FanRay {
    float a0t, a0s, dat, das;
    float L, scale;
    int idx, nseg;
    int st, ss, flags, pad_;
};
static_assert(sizeof(FanRay) == 48, "FanRay: 48 bytes");

inline float2 ff_split_host(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

inline void fan_geom_derive(FanGeom &g) {
    const int n[2] = {g.nt, g.ns};
    for (int a = 0; a < 2; ++a) {
        g.ires[a] = 1.0 / g.res[a];
        g.ext[a] = n[a] * g.res[a];
        g.res_ff[a] = ff_split_host(g.res[a]);
        g.hsize_ff[a] = ff_split_host(0.5 * g.size[a]);
    }
    g.D_ff = ff_split_host(g.D);
    g.ipint_ff = ff_split_host(1.0 / (double)g.pint);
}

// Detector-row filter job (filter.cu).
struct RowFilter {
    int nrow, np;
    float pint;
    const float *G;          // 2*np-1 taps
    const double *w;         // pre-weight table [wrows][np], or nullptr
    int wrows;               // weight row = row % wrows
    int launch_order;        // 0 clean, 1 reference launch order
    int tile, limit, row_block, rowmod;   // reference tiling
    const float *pw;         // short-scan weights [view][np] multiplied into the raw row, or nullptr
    int pw_div;              // view of a row = row / pw_div
    const double *win;       // smoothing window of wlen taps applied to the filtered row, or nullptr
    int wlen;
    double wsum;             // sum of the window taps (the divisor)
};

// Rays that graze a grid plane, listed by the fast projectors for the FP64
// re-walk of ref_walk.cu.  count is reset by the launcher and counts every
// grazing ray, listed or not.  The first cap rays go to the list; the rest
// set their bit in `bits` (one bit per ray of the launch, nbits of them),
// which the re-walk drains and clears, so no grazing ray is ever left with
// the FP32 walk's value.  bits may be null (system-matrix export): the host
// then reads count and re-runs with a list that holds every ray.
struct GrazeList {
    unsigned long long *rays;
    unsigned long long *count;
    int cap;
    unsigned int *bits;
    long long nbits;
};

#ifdef __CUDACC__
// Record a grazing ray: `entry` in the list, or bit `bit` once the list is full.
__device__ __forceinline__ void graze_push(const GrazeList &gl, unsigned long long entry, unsigned long long bit) {
    const unsigned long long slot = atomicAdd(gl.count, 1ULL);
    if (slot < (unsigned long long)gl.cap) gl.rays[slot] = entry;
    else if (gl.bits) atomicOr(gl.bits + (bit >> 5), 1u << (bit & 31));
}
#endif

// The in-plane part of the forward projector's walk set-up for one detector
// column (view v, column p): the rays of a column share the source and the
// (t, s) part of d, so they enter the volume's (t, s) square at the same
// parameter and cross the same t and s planes at the same parameters,
// whatever their row.  Built once per geometry (cone_fp_columns); parameters
// after a_in are relative to a_in.
struct __align__(16) FpColumn {
    double a_in;       // in-plane entry parameter along d (FP64)
    float a0t, a0s;    // first t / s plane crossing after the entry (+inf: the axis does not move)
    float dat, das;    // parameter between t / s planes
    float L;           // in-plane exit
    float gint, gins;  // entry coordinates along t and s in voxel units
    float dtf, dsf;    // t and s components of d (FP32)
    int s0t, s0s;      // entry voxel
    int cntt, cnts;    // t / s crossings up to the in-plane exit (cntt < 0: the column misses the volume)
    int flags;         // grazing along a t or s plane; the signs of the t and s components of d
};
static_assert(sizeof(FpColumn) == 64, "FpColumn: 64 bytes");

// vol is [z][s][t] and volT the same volume as [z][t][s], read for views whose
// detector rows run closer to the s axis; both point kFpPadSlices slices into
// zero-padded copies (the walk reads unclamped, see siddon.cuh).  volU is the
// caller's volume, read by the FP64 re-walk of grazing rays.  cols is the
// column table of cone_fp_columns.  mode 0: out = A vol; mode 1:
// out = (b - A vol) * scale, norms += (|r|^2, |b|^2).
// v0, nv: a range of the launch order ConeGeom::vorder (chunks of kFpViewChunk
// views, each chunk grouped by volume copy); nv = 0: from v0 to the end.
constexpr int kFpPadSlices = 4;
constexpr int kFpViewChunk = 90;
int cone_fp_columns(const ConeGeom &g, FpColumn *cols, cudaStream_t st);
int cone_fp_launch(const ConeGeom &g, const FpColumn *cols, const float *vol, const float *volT, const float *volU,
                   float *out, const float *b, const float *rowsum, float eps, double *norms, int mode,
                   const GrazeList &gl, cudaStream_t st, int v0 = 0, int nv = 0);
int cone_transpose_ts(const ConeGeom &g, const float *vol, float *volT, cudaStream_t st);
// Number of walk segments over all rays into *count (as double), with the
// per-ray set-up the system-matrix export shares (cone_setup.cuh).
int cone_count_launch(const ConeGeom &g, double *count, cudaStream_t st);
int cone_fixup_launch(const ConeGeom &g, const float *vol, float *out, const float *b, const float *rowsum,
                      float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st);
int fan_fixup_launch(const FanGeom &g, const float *img, void *out, bool out_double, const float *b,
                     const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st);
// Backprojection in view chunks: the quads of views [v0, v0 + nv) of the full
// sinogram R are packed into Q, then backprojected; each voxel's chunk sum plus
// prev (optional) goes to out, or, with update, into out = vol as
// clamp(vol + lambda * sum / (colsum + eps), lo, hi).
size_t cone_quads_bytes(const ConeGeom &g, int nviews);
int cone_pack_quads(const ConeGeom &g, const float *R, float4 *Q, int v0, int nv, cudaStream_t st);
// zt0, nzt: a range of z tiles of cone_bp_ztile() slices (nzt = 0: from zt0 to the top).
int cone_bp_launch(const ConeGeom &g, const float4 *Q, int v0, int nv, const float *prev, float *out, int weighting,
                   const float *colsum, float eps, float lambda, float lo, float hi, bool update, cudaStream_t st,
                   int zt0 = 0, int nzt = 0);
int cone_bp_ztile();
int row_filter_launch(const RowFilter &f, const float *R, float *out, cudaStream_t st);
// The set-up table of every ray of g (nb * np records), for g.ray_tab.
int fan_ray_table_launch(const FanGeom &g, FanRay *tab, cudaStream_t st);
int fan_fp_launch(const FanGeom &g, const float *img, void *out, const float *b, const float *rowsum,
                  float eps, double *norms, int mode, const GrazeList &gl, cudaStream_t st);
int fan_bp_launch(const FanGeom &g, const float *R, float *img, int wmode, const float *colsum, float eps,
                  float lambda, float lo, float hi, bool update, cudaStream_t st);
// System-matrix export (sysmat.cu, ref_walk.cu): CSR rows of rays in
// sinogram order, columns the voxel index; counts go to row_ptr[row + 1].
int cone_sysmat_launch(const ConeGeom &g, int v0, int nv, long long *row_ptr, int *col, float *val, bool fill,
                       const GrazeList &gl, cudaStream_t st);
int fan_sysmat_launch(const FanGeom &g, long long *row_ptr, int *col, float *val, bool fill, const GrazeList &gl,
                      cudaStream_t st);
int cone_sysmat_ref_launch(const ConeGeom &g, long long r0, long long *row_ptr, int *col, float *val, bool fill,
                           const GrazeList &gl, cudaStream_t st);
int fan_sysmat_ref_launch(const FanGeom &g, long long *row_ptr, int *col, float *val, bool fill, const GrazeList &gl,
                          cudaStream_t st);
// row_ptr[1..n] <- inclusive prefix sum of itself, row_ptr[0] <- 0; tmp is CUB scratch
int csr_scan(long long *row_ptr, int n, void **tmp, size_t *tmp_bytes, cudaStream_t st);
int tv_flow_launch(float *x, float *work, double *scratch, int nx, int ny, int nz, int iters, float step,
                   float eps, float lo, cudaStream_t st);
int sq_diff_sum_launch(const float *a, const float *b, long long n, double *out, cudaStream_t st);
// Free the device buffers the IterativeFDK / curved-FDK drop-ins cache between calls.
void iterfdk_release_cache();
void fdkui_release_cache();

}  // namespace ct

namespace ct {

// One slice of a batch of uneven 2D fan scans (fan_batch.cu).
struct BatchSlice {
    FanGeom g;
    long long img_off, sino_off;   // offsets into the packed image / sinogram buffers
    int ray_blk0, pix_blk0;        // first block of the slice in the FP / BP grids
};

int fan_batch_fp_launch(const BatchSlice *d_sl, int nsl, int nblocks, int block, const float *img, float *out,
                        const float *b, const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl,
                        cudaStream_t st);
int fan_batch_bp_launch(const BatchSlice *d_sl, int nsl, int nblocks, int block, const float *R, float *img, int wmode,
                        const float *colsum, float eps, float lambda, float lo, float hi, bool update,
                        cudaStream_t st);
int fan_batch_fixup_launch(const BatchSlice *d_sl, int nsl, const float *img, float *out, const float *b,
                           const float *rowsum, float eps, double *norms, int mode, const GrazeList &gl,
                           cudaStream_t st);

}  // namespace ct
