/*
 * ctgb.h -- C ABI of the GB300 (sm_103a) CT projector / backprojector library
 * (libctgb.so).  A drop-in for the host helpers behind the CT-Research MEX
 * operators, plus device-pointer entry points for reconstruction loops that
 * keep all data in HBM.
 *
 * Conventions (identical to the reference operators):
 *   volume     float [z][s][t], t fastest      (ProjectionCone_3D.cu:366)
 *   cone sino  float [beta][xi][P], P fastest  (ProjectionCone_3D.cu:16)
 *   2D image   float [s][t], t fastest         (ProjectionFan_2D.cu:207)
 *   2D sino    [beta][P], P fastest            (ProjectionFan_2D.cu:15)
 *   angles in radians; world coordinates run 0..Size (mm), rotation centre
 *   Size/2; the source sits at (C_t - D sin(beta), C_s + D cos(beta), C_z);
 *   P and xi are coordinates on a virtual flat detector through the centre.
 *
 * Every entry point returns a ct_status (0 = success) instead of the
 * reference's cudaError_t; ct_last_error() gives a message for the last
 * failure on the calling thread.  No entry point resets the device.
 */
#ifndef CTGB_H
#define CTGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CT_OK = 0,
    CT_ERR_ARG = 1,      /* invalid size, geometry or pointer */
    CT_ERR_OOM = 2,      /* device allocation failed */
    CT_ERR_LAUNCH = 3,   /* kernel launch failed */
    CT_ERR_CUDA = 4,     /* other CUDA runtime error (copy, sync, ...) */
    CT_ERR_TIMEOUT = 5   /* a bounded device wait gave up */
} ct_status;

/* Message of the last failure on this thread ("" when none). */
const char *ct_last_error(void);
/* Library version string. */
const char *ct_version(void);
/* Frees the device memory that the host-pointer entry points below keep
 * between calls (the cone plan of the last geometry and its staging buffers,
 * the IterativeFDK and curved-FDK buffers).  Call it before cudaDeviceReset,
 * which the reference's gateways run after every call (ProjectionCone_3D.cpp:53):
 * a reset frees those buffers behind the library's back.  No counterpart in
 * the reference, whose helpers allocate and free on every call. */
int ct_dropin_release(void);

/* ===================================================================== */
/* Drop-in host-pointer entry points.  Arguments, their meaning and the   */
/* output layout are those of the reference host helpers named in each   */
/* comment; device buffers are managed inside (cached between calls).     */
/* ===================================================================== */

/* Cone-beam Siddon forward projection.
 * Replaces ProjectionCone_3D() (GPU_accelerated_Operator/ProjectionCone_3D/
 * ProjectionCone_3D.h:32-35, body ProjectionCone_3D.cu:382-645).
 * resolution = {Size_t/t_length, Size_s/s_length, Size_z/z_length}. */
int ct_ProjectionCone_3D(const float *Pic, float *Projection, const float *BetaScanRange,
                         const float *Pdomain, const float *Xigamadomain, int t_length, int s_length,
                         int z_length, double Center_t, double Center_s, double Center_z, int LBeta,
                         int LP, int LXigama, double Distance, const double *resolution);

/* Cone-beam voxel-driven backprojection with chord weight (the A^T of the
 * cone iterative methods).  Replaces BackPro() (GPU_accelerated_Operator/
 * BackprojectionCone_3D/Backprojection3D.h:31-33, body Backprojection3D.cu:294-557). */
int ct_BackPro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
               const float *BetaScanRange, double Distance, int LBeta, int LP, int LXigama,
               const double *Size, int t_length, int s_length, int z_length);

/* FDK: cosine pre-weight, Shepp-Logan ramp, weighted bilinear backprojection.
 * Replaces FDKpro() (Analytic_Algorithm/FBP_type_analytic_algorithm_GPU_cpp_sourcecode/
 * FDK_GPU/FDK.h:29-31, body FDK.cu:129-611).  R is not modified. */
int ct_FDKpro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
              const float *BetaScanRange, double Distance, int LBeta, int LP, int LXigama,
              const double *Size, int t_length, int s_length, int z_length);

/* 2D fan-beam Siddon forward projection (double output, double angles/bins).
 * Replaces ProjectionFan_2D() (GPU_accelerated_Operator/ProjectionFan_2D/
 * ProjectionFan_2D.h:32-34, body ProjectionFan_2D.cu:223-475). */
int ct_ProjectionFan_2D(const float *Pic, double *Projection, const double *BetaScanRange,
                        const double *Pdomain, int t_length, int s_length, double Center_t,
                        double Center_s, int LBeta, int LP, double Distance, const double *resolution);

/* 2D parallel-beam Siddon forward projection.
 * Replaces ProjectionParallel_2D() (GPU_accelerated_Operator/ProjectionParallel_2D/
 * ProjectionParallel_2D.h:33-35, body ProjectionParallel_2D.cu:256-483). */
int ct_ProjectionParallel_2D(const float *Pic, double *Projection, const double *thetaRange,
                             const double *t_Range, int height, int width, double Center_y,
                             double Center_x, int Ltheta, int Lt, const double *resolution);

/* 2D fan voxel-driven backprojection (unfiltered; the A^T of 2D SIRT).
 * Replaces FBPfan() of GPU_accelerated_Operator/BackprojectionFan_2D
 * (BackprojectionFan2D.h:35-36, body BackprojectionFan2D.cu:119-349). */
int ct_BackprojectionFan2D(float *Display, const float *R, const float *Pdomain,
                           const float *BetaScanRange, int LBeta, int LP, const double *Size,
                           int t_length, int s_length, double Rscan);

/* 2D fan FBP: pre-weight, S-L ramp, 1/U^2 weighted backprojection.
 * Replaces FBPfan() of Analytic_Algorithm/.../FBP_fan_GPU (FBPfan.h:31-32,
 * body FBPfan.cu:99-557).  R is not modified. */
int ct_FBPfan(float *Display, const float *R, const float *Pdomain, const float *BetaScanRange,
              int LBeta, int LP, const double *Size, int t_length, int s_length, double Rscan);

/* 2D parallel FBP: S-L ramp and linear-interpolation backprojection.
 * Replaces FBPpara() (Analytic_Algorithm/.../FBP_parallel_GPU/FBPparallel.h:31-32). */
int ct_FBPpara(float *Display, const float *R, const float *Tdomain, const float *ThetaScanRange,
               int LTheta, int LT, const double *Size, int t_length, int s_length);

/* 2D fan FBP (as ct_FBPfan) that allocates no device memory; no counterpart in
 * the reference.  For callers that may not call cudaMalloc / cudaFree while they
 * run (memory reserved once at start-up, or a framework-owned device pool).
 * d_R (LBeta x LP sinogram) and d_Display (t x s image, < 2^31 pixels) are
 * device buffers of the caller; Pdomain, BetaScanRange and Size are host arrays,
 * copied into the library's array with cudaMemcpyAsync on `stream`.  All other
 * data sits in that one library-owned 8 MiB device array: sizes whose tables and
 * filtered sinogram (about 4 * LBeta * LP bytes) do not fit return CT_ERR_ARG.
 * The first call on a device looks up that array's address; make it before any
 * stream capture.  Under CUDA's lazy module loading (the default) the array's
 * 8 MiB are committed on a device by that first call, so a caller that reserves
 * all remaining device memory should make one call before reserving.  Calls
 * share the array, so calls that overlap on the GPU race: serialise them.  Work
 * is queued on `stream` (cudaStream_t). */
int ct_FBPfan_noalloc(float *d_Display, const float *d_R, const float *Pdomain,
                      const float *BetaScanRange, int LBeta, int LP, const double *Size, int t_length,
                      int s_length, double Rscan, void *stream);

/* ===================================================================== */
/* Plans and device-pointer entry points (data stays in HBM).             */
/* ===================================================================== */

typedef struct ct_cone_plan ct_cone_plan;
typedef struct ct_fan_plan ct_fan_plan;

/* Behaviour switches of the plans.  Every plan starts with the settings that
 * reproduce the reference exactly, data-dependent quirks included
 * (LAUNCH_ORDER, STICKY, Shepp-Logan taps, no window, full scan). */
enum {
    CT_FDK_FILTER_CLEAN = 0,       /* weight the whole row, then filter */
    CT_FDK_FILTER_LAUNCH_ORDER = 1,/* reference: in-place weight seen in launch order (FDK.cu:36-44) */
    CT_FDK_BP_ZERO = 0,            /* off-detector voxels add 0 */
    CT_FDK_BP_STICKY = 1           /* reference: they re-add the last in-range value (FDK.cu:73,100-123) */
};

/* Ramp filters of the FDK / FBP filter stage. */
enum {
    CT_FILTER_SHEPP_LOGAN = 0,     /* GFunction taps (FDK.cu:6-19), the reference's GPU filter */
    CT_FILTER_RAM_LAK = 1          /* FBP_parallel.m:241-251, scaled by 1/2 to the Shepp-Logan amplitude */
};

/* Cone geometry; arrays are host pointers copied into the plan.  Angles,
 * P and xi domains as the reference's BetaScanRange / Pdomain / Xigamadomain
 * (uniform spacing required by the backprojectors, as in the reference). */
int ct_cone_plan_create(ct_cone_plan **plan, int t_length, int s_length, int z_length,
                        const double *Size, const float *BetaScanRange, int LBeta,
                        const float *Pdomain, int LP, const float *Xigamadomain, int LXigama,
                        double Distance);
int ct_cone_plan_destroy(ct_cone_plan *plan);
/* FDK behaviour (CT_FDK_FILTER_*, CT_FDK_BP_*). Defaults: LAUNCH_ORDER, STICKY. */
int ct_cone_plan_set_fdk_mode(ct_cone_plan *plan, int filter_mode, int bp_mode);
/* Filter stage options; none has a counterpart in the reference's GPU code.
 * kind: CT_FILTER_*.  window_len > 0 smooths every filtered row with a
 * Hamming window of that many taps, out[p] = sum_i h[i] x[p + i - len/2] / sum(h)
 * (the commented post-filter of FanProjection.m:265-270); 0 = none. */
int ct_cone_plan_set_filter(ct_cone_plan *plan, int kind, int window_len);
/* enable = 1: multiply the projections by 2x the short-scan weights of
 * ParkFunction.m:6-16 (gama = atan(P / Distance), fan angle from the detector
 * ends, start angle = BetaScanRange[0]) before the pre-weight and filter. */
int ct_cone_plan_set_short_scan(ct_cone_plan *plan, int enable);
/* Device bytes of plan-owned workspace (packed sinogram, filter rows). */
size_t ct_cone_plan_workspace_bytes(const ct_cone_plan *plan);
/* Views per chunk of the backprojectors (ct_cone_bp, ct_cone_bp_update,
 * ct_cone_fdk_bp): each chunk's detector data is packed and backprojected on
 * its own and its sums added to the volume; the packed data needs 16 bytes per
 * detector sample of one chunk.  0 (the default): automatic, chunks of about
 * 768 MiB of packed data evened out over the scan (shorter launches keep the
 * packed views in L2); a value >= the view count: one pass.  Results differ
 * from one pass only by float rounding of the partial sums.  get returns the
 * chunk in effect.  No counterpart in the reference. */
int ct_cone_plan_set_bp_chunk(ct_cone_plan *plan, int views);
int ct_cone_plan_get_bp_chunk(const ct_cone_plan *plan, int *views);

/* proj[beta][xi][P] = Siddon line integrals of vol.  All pointers are device
 * pointers; work is queued on `stream` (cudaStream_t, 0 = legacy default). */
int ct_cone_fp(ct_cone_plan *plan, const float *d_vol, float *d_proj, void *stream);
/* Forward projection fused with the SIRT residual: out = (b - A vol) * scale,
 * with scale = 1/(rowsum + eps) when d_rowsum is non-NULL (else 1), and
 * adds sum((b - A vol)^2) and sum(b^2) into d_norms[0..1] (double, device). */
int ct_cone_fp_residual(ct_cone_plan *plan, const float *d_vol, const float *d_b,
                        const float *d_rowsum, float eps, float *d_out, double *d_norms, void *stream);
/* vol = BackPro(proj): chord-weighted voxel-driven backprojection. */
int ct_cone_bp(ct_cone_plan *plan, const float *d_proj, float *d_vol, void *stream);
/* SIRT update fused into the backprojection:
 * vol = clamp(vol + lambda * BackPro(proj) / (colsum + eps), lo, hi). */
int ct_cone_bp_update(ct_cone_plan *plan, const float *d_proj, const float *d_colsum, float eps,
                      float lambda, float lo, float hi, float *d_vol, void *stream);
/* FDK reconstruction of d_proj into d_vol (modes from ct_cone_plan_set_fdk_mode). */
int ct_cone_fdk(ct_cone_plan *plan, const float *d_proj, float *d_vol, void *stream);
/* The two FDK stages on their own: cosine pre-weight + S-L ramp into
 * d_filtered (sinogram layout), and the LR^2-weighted backprojection of an
 * already filtered sinogram. */
int ct_cone_fdk_filter(ct_cone_plan *plan, const float *d_proj, float *d_filtered, void *stream);
int ct_cone_fdk_bp(ct_cone_plan *plan, const float *d_filtered, float *d_vol, void *stream);
/* The projector's system matrix as CSR (GenSysMatCircular3D.m computes it in
 * MATLAB; no GPU counterpart in the reference).  Rows: the rays of views
 * view0 .. view0 + nviews - 1 in sinogram order ([beta][xi][P], row 0 = the
 * first ray of view0); columns: voxel index of the [z][s][t] volume; values:
 * segment lengths in mm, from the forward projector's own walk, so A vol
 * equals ct_cone_fp to float rounding.  Call with d_col = d_val = NULL to get
 * d_row_ptr (rows + 1 int64, device) and *nnz; call again with device arrays
 * of cap >= *nnz entries to fill them. */
int ct_cone_sysmat(ct_cone_plan *plan, int view0, int nviews, long long *d_row_ptr, int *d_col,
                   float *d_val, long long cap, long long *nnz, void *stream);
/* Exact number of Siddon segments over all rays of the plan (host result). */
int ct_cone_count_segments(ct_cone_plan *plan, long long *segments, void *stream);

/* Rays that run along a grid plane to FP64 precision are re-walked with the
 * reference's own FP64 walk (ProjectionCone_3D.cu:44-84 clamps their slopes
 * at 1e16, and their charge follows that rounding).  The fast projector lists
 * them for the re-walk; past the list's capacity (65536 by default) it marks
 * them in a one-bit-per-ray overflow map that the re-walk drains, so every
 * such ray gets the reference's value at any count.  These report how many
 * rays of the plan's last forward projection took the re-walk (host result;
 * synchronises `stream`).  No counterpart in the reference. */
int ct_cone_plan_grazing_rays(const ct_cone_plan *plan, long long *n, void *stream);
int ct_fan_plan_grazing_rays(const ct_fan_plan *plan, long long *n, void *stream);
/* List capacity of grazing-ray buffers allocated from now on (process-wide;
 * >= 1).  Memory tuning and tests; the results do not depend on it. */
int ct_set_graze_list_capacity(int cap);

/* 2D fan plan (ProjectionFan_2D / BackprojectionFan2D / FBPfan geometry). */
int ct_fan_plan_create(ct_fan_plan **plan, int t_length, int s_length, const double *Size,
                       const double *BetaScanRange, int LBeta, const double *Pdomain, int LP,
                       double Distance);
int ct_fan_plan_destroy(ct_fan_plan *plan);
/* Parallel-beam plan (ProjectionParallel_2D geometry): image height x width,
 * resolution[0] along the height, resolution[1] along the width; works with
 * ct_fan_fp / ct_fan_fp_residual / ct_fan_sysmat. */
int ct_par_plan_create(ct_fan_plan **plan, int height, int width, const double *resolution,
                       const double *thetaRange, int Ltheta, const double *t_Range, int Lt);
/* The 2D projector's system matrix as CSR (GenSysMatFan.m / GenSysMatParal.m
 * compute it in MATLAB), as ct_cone_sysmat: rows [beta][P], columns s * t_length + t. */
int ct_fan_sysmat(ct_fan_plan *plan, long long *d_row_ptr, int *d_col, float *d_val, long long cap,
                  long long *nnz, void *stream);
/* FBP filter options, as ct_cone_plan_set_filter / ct_cone_plan_set_short_scan. */
int ct_fan_plan_set_filter(ct_fan_plan *plan, int kind, int window_len);
int ct_fan_plan_set_short_scan(ct_fan_plan *plan, int enable);
int ct_fan_fp(ct_fan_plan *plan, const float *d_img, float *d_proj, void *stream);
int ct_fan_fp_residual(ct_fan_plan *plan, const float *d_img, const float *d_b, const float *d_rowsum,
                       float eps, float *d_out, double *d_norms, void *stream);
int ct_fan_bp(ct_fan_plan *plan, const float *d_proj, float *d_img, void *stream);
int ct_fan_bp_update(ct_fan_plan *plan, const float *d_proj, const float *d_colsum, float eps,
                     float lambda, float lo, float hi, float *d_img, void *stream);
int ct_fan_fbp(ct_fan_plan *plan, const float *d_proj, float *d_img, int filter_mode, void *stream);

/* ===================================================================== */
/* Batches of uneven 2D fan slices: every operator runs all slices in one */
/* launch.  Images and sinograms are packed back to back in two device    */
/* buffers at the offsets ct_fan_batch_layout returns.                    */
/* ===================================================================== */

typedef struct ct_fan_batch ct_fan_batch;

/* Slice k: image t_length[k] x s_length[k], extent Size[2k..2k+1], views
 * BetaScanRange[k][0..LBeta[k]), bins Pdomain[k][0..LP[k]), Distance[k]. */
int ct_fan_batch_create(ct_fan_batch **batch, int nslices, const int *t_length, const int *s_length,
                        const double *Size, const double *const *BetaScanRange, const int *LBeta,
                        const double *const *Pdomain, const int *LP, const double *Distance);
int ct_fan_batch_destroy(ct_fan_batch *batch);
/* Offsets (in floats) of each slice in the packed image / sinogram buffers;
 * element nslices holds the totals.  Arrays of nslices + 1. */
int ct_fan_batch_layout(const ct_fan_batch *batch, long long *img_offsets, long long *sino_offsets);
/* Threads per block of the forward / back projection launches (tuning). */
int ct_fan_batch_set_blocks(ct_fan_batch *batch, int fp_block, int bp_block);
int ct_fan_batch_fp(ct_fan_batch *batch, const float *d_img, float *d_proj, void *stream);
/* d_norms: 2 doubles per slice, (|b - A x|^2, |b|^2) added. */
int ct_fan_batch_fp_residual(ct_fan_batch *batch, const float *d_img, const float *d_b, const float *d_rowsum,
                             float eps, float *d_out, double *d_norms, void *stream);
int ct_fan_batch_bp(ct_fan_batch *batch, const float *d_proj, float *d_img, void *stream);
int ct_fan_batch_bp_update(ct_fan_batch *batch, const float *d_proj, const float *d_colsum, float eps,
                           float lambda, float lo, float hi, float *d_img, void *stream);
int ct_fan_batch_fbp(ct_fan_batch *batch, const float *d_proj, float *d_img, int filter_mode, void *stream);
/* FBP filter options of every slice (ct_fan_plan_set_filter, ct_fan_plan_set_short_scan). */
int ct_fan_batch_set_filter(ct_fan_batch *batch, int kind, int window_len, int short_scan);
/* Grazing rays of the batch's last forward projection (as ct_fan_plan_grazing_rays). */
int ct_fan_batch_grazing_rays(const ct_fan_batch *batch, long long *n, void *stream);

/* ===================================================================== */
/* IterativeFDK error slice                                               */
/* ===================================================================== */

/* Drop-in for IterativeFDKerrCompute() (IterativeFDKerrCompute.h:23-27): host
 * pointers, the reference's argument list and meaning.  Pic is the prior image
 * [z][s][t]; ErrorSlicecuda receives LBeta * s_length * z_length floats laid
 * out [beta][z][s] for image slice t (0-based).  Every (s, z) is computed once
 * at any size (the reference's residual launches cover s, z < 512 or
 * multiples of 512 only). */
int ct_IterativeFDKerrCompute(const float *Pic, float *ErrorSlicecuda, const float *BetaScanRange,
                              const float *Udomain, const double *Pdomain, const double *G,
                              const double *Size, int t_length, int s_length, int z_length,
                              double Center_t, double Center_s, double Center_z, int LBeta, int LP,
                              int LU, int LG, double Distance, const double *resolution2, int t,
                              float BetaScanInt, float dU, double PInt);
/* Device-pointer form: d_Pic and d_Err on the device, the domains on the host;
 * centres, resolution and intervals derived as the MEX gateway does
 * (IterativeFDKerrCompute.cpp:10-31).  t is 0-based. */
int ct_iterfdk_err(const float *d_Pic, float *d_Err, const float *BetaScanRange, int LBeta,
                   const float *Udomain, int LU, const double *Pdomain, int LP, const double *G, int LG,
                   const double *Size, int t_length, int s_length, int z_length, double Distance, int t,
                   void *stream);

/* ===================================================================== */
/* Curved-detector (equiangular) short-scan FDK                           */
/* ===================================================================== */

/* Drop-in for FDKUI() (ImplementUI.h:31-33): R [beta][xi][gamma] (double,
 * LBeta x LXigama x LGama, host) -> Display [z][s][t] (double, Size[0] x
 * Size[1] x z_length, host).  Size holds the integer extents (pixels in t
 * and s, mm in z); betaStartAngle and MaxGama feed the Parker weights.  The
 * reference fixes LGama = 936, LXigama = 80, LBeta = 800 in its filter
 * launch (ImplementUI.h:16-20); any sizes are accepted here. */
int ct_FDKUI(double *Display, const double *R, const double *Xigamadomain, const double *Gamadomain,
             const double *BetaScanRange, double betaStartAngle, double MaxGama, double Distance,
             double Distance_s2d, int LGama, int LBeta, int LXigama, const int *Size, int z_length);
/* The two stages on device buffers: weighted, filtered rows of d_R into d_Rcov
 * (float, same layout), and the backprojection of d_Rcov into d_Display. */
int ct_fdkui_filter(const double *d_R, float *d_Rcov, const double *Xigamadomain, const double *Gamadomain,
                    const double *BetaScanRange, double betaStartAngle, double MaxGama, double Distance,
                    double Distance_s2d, int LGama, int LBeta, int LXigama, void *stream);
int ct_fdkui_bp(const float *d_Rcov, double *d_Display, const double *Xigamadomain, const double *Gamadomain,
                const double *BetaScanRange, double Distance, double Distance_s2d, int LGama, int LBeta,
                int LXigama, const int *Size, int z_length, void *stream);

/* ===================================================================== */
/* Row-action reconstruction on an exported system matrix                 */
/* ===================================================================== */

/* One ART (Kaczmarz) sweep over CSR rows row_begin .. row_end - 1 in order
 * (Iterative_algorithm/ART.m:57-75): x <- x - lambda a_j (a_j.x - b_j) / (a_j.a_j),
 * rows with a_j.a_j = 0 skipped.  CSR as ct_*_sysmat exports it; device pointers. */
int ct_csr_kaczmarz(const long long *d_row_ptr, const int *d_col, const float *d_val, const float *d_b,
                    float *d_x, int row_begin, int row_end, float lambda, void *stream);

/* ===================================================================== */
/* Elementwise and regulariser kernels of the SIRT(-TV) loops.            */
/* ===================================================================== */

/* Isotropic TV gradient-flow sub-iterations on a [nz][ny][nx] volume
 * (nz = 1 for 2D):  x <- max(x - step * g / rms(g), lo) with g the gradient
 * of sum sqrt(|forward-difference grad x|^2 + eps^2); `iters` steps.  d_work
 * must hold nx*ny*nz floats; d_scratch 2 doubles. */
int ct_tv_flow(float *d_x, float *d_work, double *d_scratch, int nx, int ny, int nz, int iters,
               float step, float eps, float lo, void *stream);
/* The regularisation phase of one ASD-POCS iteration (SIRT-TV with the TV
 * step tied to the data step), all on the device so iterations can be captured
 * in a CUDA graph.  d_prev holds x before the data step; d_state = double[3]
 * (alpha, scratch, scratch) with alpha carried across calls.  Computes
 * dp = ||x - prev||, copies x to d_prev, runs `iters` TV sub-steps (as
 * ct_tv_flow) of RMS size alpha * dp / sqrt(n), and multiplies alpha by
 * alpha_red when the sub-steps moved x by more than r_max * dp. */
int ct_tv_flow_asd(float *d_x, float *d_prev, float *d_work, double *d_scratch, double *d_state, int nx, int ny,
                   int nz, int iters, float eps, float lo, float alpha_red, float r_max, void *stream);
/* d_norm[0] += sum((a - b)^2) over n floats (FP32 partial sums of 16 terms,
 * accumulated in double). */
int ct_sq_diff_sum(const float *d_a, const float *d_b, long long n, double *d_norm, void *stream);

/* ===================================================================== */
/* Learned warm start for SIRT-TV: the BF16 3D U-Net's kernels.           */
/* No reference counterpart (the reference has no learned component); the */
/* network feeds the SIRT-TV loop above its starting image.  Activations   */
/* are bf16, channels-last [n][z][y][x][c]; weights bf16 [cout][taps][cin];*/
/* sums FP32.  All pointers are device pointers, 16-byte aligned.         */
/* ===================================================================== */

/* out[v][co] = act(bias[co] + sum_tap sum_ci X[v + off(tap)][ci] W[co][tap][ci])
 * with X = concat(x1 (c1 channels), x2 (c2 channels)) along channels, zero
 * padding, ntaps 27 (3x3x3, tap = 9 (dz+1) + 3 (dy+1) + (dx+1)) or 1.  Output
 * channels [0, co1) go to out1 ([v][co1]) and [co1, co1 + co2) to out2; act is
 * ReLU when relu != 0, and an output value is zeroed where its mask (same
 * layout as its output, may be null) is not > 0.  co1 + co2 in {32, 64, 128,
 * 256}; c1, c2 multiples of 32; x a divisor or multiple of 128, and y, z such
 * that 128-voxel x-y-z blocks tile the volume.  tcgen05 tensor cores. */
int ct_unet_conv3d(const void *d_x1, int c1, const void *d_x2, int c2, int nb, int nz, int ny, int nx,
                   const void *d_w, int ntaps, const float *d_bias, int relu, void *d_out1, int co1, void *d_out2,
                   int co2, const void *d_mask1, const void *d_mask2, void *stream);
/* dW[co][tap][ci] += sum_v dY[v][co] X[v + off(tap)][ci] (FP32 dW).  X is
 * given channel-major [n][cin][z][y][x] as three copies shifted along x
 * (d_xm[x] = X[x - 1], d_x0, d_xp[x] = X[x + 1]; ct_unet_shift_t makes them;
 * d_xm / d_xp unused for ntaps 1); dY channel-major [n][cout][z][y][x].
 * x a multiple of 8.  Split-K: one CTA per kper 64-voxel slices of the y*x
 * planes. */
int ct_unet_conv3d_wgrad(const void *d_xm, const void *d_x0, const void *d_xp, int cin, const void *d_dy, int cout,
                         int nb, int nz, int ny, int nx, int ntaps, int kper, float *d_dw, void *stream);
/* Reads and clears the device flag of the convolutions' bounded waits:
 * CT_ERR_TIMEOUT (flags != 0) when a wait gave up since the last call.  Flag
 * bits: 1 a free ring stage, 2 a loaded stage, 4 the last MMA, 8 the self-test. */
int ct_unet_status(int *flags);
/* Runs the convolutions' bounded mbarrier wait, with a limit of limit_ns
 * (1 us .. 1 s), on a barrier that nothing arrives on: the wait gives up and
 * sets flag 8, which ct_unet_status then reports as CT_ERR_TIMEOUT.  Shows that
 * the bounded waits end and report; the context stays usable. */
int ct_unet_wait_selftest(long long limit_ns, void *stream);
/* out[v][k] = vol[v + off(k)] (k < 27, zero outside), 0 for k = 27..31: the
 * one-channel input as 32 channels for a 1-tap convolution. */
int ct_unet_im2col27(const float *d_vol, int nb, int nz, int ny, int nx, void *d_out, void *stream);
/* 2x2x2 max pooling and its gradient (to the first maximum of each window,
 * when that maximum is > 0: the pooled tensors are ReLU outputs);
 * nearest 2x upsampling and its gradient (sum of the 8 children).  Sizes are
 * the coarse volume's; c a multiple of 8. */
int ct_unet_pool2(const void *d_in, void *d_out, int c, int nb, int nz, int ny, int nx, void *stream);
int ct_unet_pool2_bwd(const void *d_x, const void *d_y, const void *d_dy, void *d_dx, int c, int nb, int nz, int ny,
                      int nx, void *stream);
int ct_unet_up2(const void *d_in, void *d_out, int c, int nb, int nz, int ny, int nx, void *stream);
int ct_unet_up2_bwd(const void *d_dout, void *d_din, int c, int nb, int nz, int ny, int nx, void *stream);
/* Channel-major copies of a channels-last activation at channel offset coff
 * of a ctot-channel buffer, shifted along x by -1 / 0 / +1 (null: skipped). */
int ct_unet_shift_t(const void *d_in, int c, int nb, int nz, int ny, int nx, void *d_om, void *d_o0, void *d_op,
                    int ctot, int coff, void *stream);
/* Output head: out[v] = base[v] + b + sum_c w[c] f[v][c] (32 channels, FP32
 * out; base may be null), and its gradient: df = w dout (f > 0),
 * dw += sum_v dout f, db += sum_v dout. */
int ct_unet_head(const void *d_f, const float *d_w, const float *d_b, const float *d_base, float *d_out,
                 long long nvox, void *stream);
int ct_unet_head_bwd(const float *d_dout, const void *d_f, const float *d_w, void *d_df, float *d_dw, float *d_db,
                     long long nvox, void *stream);
/* db[c] += sum_v dy[v][c] (bias gradient); c divides 256. */
int ct_unet_colsum(const void *d_dy, int c, long long nvox, float *d_db, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CTGB_H */
