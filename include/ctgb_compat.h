/*
 * ctgb_compat.h -- the reference's own host-helper names and signatures, with
 * C++ linkage and cudaError_t results, so that the reference's MEX gateways
 * (X.cpp, unchanged) link against this library instead of X.cu.
 *
 * Two libraries carry these definitions, because the reference has two
 * different helpers named FBPfan with one signature:
 *   libctgb_compat.so        every helper below; FBPfan is the filtered fan FBP
 *                            of FBP_fan_GPU (FBPfan.h:31-32)
 *   libctgb_compat_bpfan.so  only FBPfan, the unfiltered fan backprojection of
 *                            BackprojectionFan_2D (BackprojectionFan2D.h:35-36)
 * A gateway links the one whose FBPfan it calls (BackprojectionFan2D.cpp links
 * the second; every other gateway the first).
 *
 * Each helper runs the library's drop-in entry point (include/ctgb.h), then
 * frees what that entry point caches, so that the cudaDeviceReset the
 * gateways call after every helper (ProjectionCone_3D.cpp:53) finds nothing of
 * the library's on the device.  Status mapping: CT_ERR_ARG ->
 * cudaErrorInvalidValue, CT_ERR_OOM -> cudaErrorMemoryAllocation,
 * CT_ERR_LAUNCH -> cudaErrorLaunchFailure, CT_ERR_TIMEOUT -> cudaErrorTimeout,
 * other failures -> cudaErrorUnknown; the library's message goes to stderr,
 * as the reference helpers print theirs.
 */
#ifndef CTGB_COMPAT_H
#define CTGB_COMPAT_H

#include <cuda_runtime.h>

/* ProjectionCone_3D.h:32-35 */
cudaError_t ProjectionCone_3D(const float *Pic, float *Projection, const float *BetaScanRange, const float *Pdomain,
                              const float *Xigamadomain, const int t_length, const int s_length, const int z_length,
                              const double Center_t, const double Center_s, const double Center_z, const int LBeta,
                              const int LP, const int LXigama, const double Distance, const double *resolution);

/* Backprojection3D.h:31-33 */
cudaError_t BackPro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
                    const float *BetaScanRange, const double Distance, const int LBeta, const int LP,
                    const int LXigama, const double *Size, const int t_length, const int s_length,
                    const int z_length);

/* FDK.h:29-31 */
cudaError_t FDKpro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
                   const float *BetaScanRange, const double Distance, const int LBeta, const int LP,
                   const int LXigama, const double *Size, const int t_length, const int s_length,
                   const int z_length);

/* ProjectionFan_2D.h:32-34 */
cudaError_t ProjectionFan_2D(const float *Pic, double *Projection, const double *BetaScanRange,
                             const double *Pdomain, const int t_length, const int s_length, const double Center_t,
                             const double Center_s, const int LBeta, const int LP, const double Distance,
                             const double *resolution);

/* ProjectionParallel_2D.h:33-35 */
cudaError_t ProjectionParallel_2D(const float *Pic, double *Projection, const double *thetaRange,
                                  const double *t_Range, const int height, const int width, const double Center_y,
                                  const double Center_x, const int Ltheta, const int Lt, const double *resolution);

/* FBPfan.h:31-32 (libctgb_compat.so) or BackprojectionFan2D.h:35-36 (libctgb_compat_bpfan.so) */
cudaError_t FBPfan(float *Display, const float *R, const float *Pdomain, const float *BetaScanRange,
                   const int LBeta, const int LP, const double *Size, const int t_length, const int s_length,
                   const double Rscan);

/* FBPparallel.h:31-32 */
cudaError_t FBPpara(float *Display, const float *R, const float *Tdomain, const float *ThetaScanRange,
                    const int LTheta, const int LT, const double *Size, const int t_length, const int s_length);

/* IterativeFDKerrCompute.h:24-28 */
cudaError_t IterativeFDKerrCompute(const float *Pic, float *ErrorSlicecuda, const float *BetaScanRange,
                                   const float *Udomain, const double *Pdomain, const double *G, const double *Size,
                                   const int t_length, const int s_length, const int z_length, const double Center_t,
                                   const double Center_s, const double Center_z, const int LBeta, const int LP,
                                   const int LU, const int LG, const double Distance, const double *resolution2,
                                   const int t, const float BetaScanInt, const float dU, const double PInt);

/* ImplementUI.h:31-33 */
cudaError_t FDKUI(double *Display, const double *R, const double *Xigamadomain, const double *Gamadomain,
                  const double *BetaScanRange, const double betaStartAngle, const double MaxGama,
                  const double Distance, const double Distance_s2d, const int LGama, const int LBeta,
                  const int LXigama, const int *Size, const int z_length);

#endif /* CTGB_COMPAT_H */
