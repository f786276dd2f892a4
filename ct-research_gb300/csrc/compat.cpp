// compat.cpp -- the reference helper names over the C ABI (include/ctgb_compat.h).
//
// Built twice: as libctgb_compat.so (every helper; FBPfan = the filtered fan
// FBP) and, with CTGB_COMPAT_BPFAN defined, as libctgb_compat_bpfan.so (only
// FBPfan = the unfiltered fan backprojection of BackprojectionFan_2D).  Both
// link libctgb.so.
#include <cstdio>

#include "ctgb.h"
#include "ctgb_compat.h"

namespace {

// ct_status -> cudaError_t, with the library's message on stderr; the drop-in
// caches are freed either way, so a cudaDeviceReset after the call is safe.
cudaError_t finish(int status, const char *name) {
    ct_dropin_release();
    switch (status) {
        case CT_OK: return cudaSuccess;
        case CT_ERR_ARG: break;
        default: break;
    }
    std::fprintf(stderr, "%s failed: %s\n", name, ct_last_error());
    switch (status) {
        case CT_ERR_ARG: return cudaErrorInvalidValue;
        case CT_ERR_OOM: return cudaErrorMemoryAllocation;
        case CT_ERR_LAUNCH: return cudaErrorLaunchFailure;
        case CT_ERR_TIMEOUT: return cudaErrorTimeout;
        default: return cudaErrorUnknown;
    }
}

}  // namespace

#ifdef CTGB_COMPAT_BPFAN

cudaError_t FBPfan(float *Display, const float *R, const float *Pdomain, const float *BetaScanRange,
                   const int LBeta, const int LP, const double *Size, const int t_length, const int s_length,
                   const double Rscan) {
    return finish(ct_BackprojectionFan2D(Display, R, Pdomain, BetaScanRange, LBeta, LP, Size, t_length, s_length,
                                         Rscan),
                  "FBPfan (BackprojectionFan_2D)");
}

#else

cudaError_t ProjectionCone_3D(const float *Pic, float *Projection, const float *BetaScanRange, const float *Pdomain,
                              const float *Xigamadomain, const int t_length, const int s_length, const int z_length,
                              const double Center_t, const double Center_s, const double Center_z, const int LBeta,
                              const int LP, const int LXigama, const double Distance, const double *resolution) {
    return finish(ct_ProjectionCone_3D(Pic, Projection, BetaScanRange, Pdomain, Xigamadomain, t_length, s_length,
                                       z_length, Center_t, Center_s, Center_z, LBeta, LP, LXigama, Distance,
                                       resolution),
                  "ProjectionCone_3D");
}

cudaError_t BackPro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
                    const float *BetaScanRange, const double Distance, const int LBeta, const int LP,
                    const int LXigama, const double *Size, const int t_length, const int s_length,
                    const int z_length) {
    return finish(ct_BackPro(Display, R, Xigamadomain, Pdomain, BetaScanRange, Distance, LBeta, LP, LXigama, Size,
                             t_length, s_length, z_length),
                  "BackPro");
}

cudaError_t FDKpro(float *Display, const float *R, const float *Xigamadomain, const float *Pdomain,
                   const float *BetaScanRange, const double Distance, const int LBeta, const int LP,
                   const int LXigama, const double *Size, const int t_length, const int s_length,
                   const int z_length) {
    return finish(ct_FDKpro(Display, R, Xigamadomain, Pdomain, BetaScanRange, Distance, LBeta, LP, LXigama, Size,
                            t_length, s_length, z_length),
                  "FDKpro");
}

cudaError_t ProjectionFan_2D(const float *Pic, double *Projection, const double *BetaScanRange,
                             const double *Pdomain, const int t_length, const int s_length, const double Center_t,
                             const double Center_s, const int LBeta, const int LP, const double Distance,
                             const double *resolution) {
    return finish(ct_ProjectionFan_2D(Pic, Projection, BetaScanRange, Pdomain, t_length, s_length, Center_t,
                                      Center_s, LBeta, LP, Distance, resolution),
                  "ProjectionFan_2D");
}

cudaError_t ProjectionParallel_2D(const float *Pic, double *Projection, const double *thetaRange,
                                  const double *t_Range, const int height, const int width, const double Center_y,
                                  const double Center_x, const int Ltheta, const int Lt, const double *resolution) {
    return finish(ct_ProjectionParallel_2D(Pic, Projection, thetaRange, t_Range, height, width, Center_y, Center_x,
                                           Ltheta, Lt, resolution),
                  "ProjectionParallel_2D");
}

cudaError_t FBPfan(float *Display, const float *R, const float *Pdomain, const float *BetaScanRange,
                   const int LBeta, const int LP, const double *Size, const int t_length, const int s_length,
                   const double Rscan) {
    return finish(ct_FBPfan(Display, R, Pdomain, BetaScanRange, LBeta, LP, Size, t_length, s_length, Rscan),
                  "FBPfan");
}

cudaError_t FBPpara(float *Display, const float *R, const float *Tdomain, const float *ThetaScanRange,
                    const int LTheta, const int LT, const double *Size, const int t_length, const int s_length) {
    return finish(ct_FBPpara(Display, R, Tdomain, ThetaScanRange, LTheta, LT, Size, t_length, s_length), "FBPpara");
}

cudaError_t IterativeFDKerrCompute(const float *Pic, float *ErrorSlicecuda, const float *BetaScanRange,
                                   const float *Udomain, const double *Pdomain, const double *G, const double *Size,
                                   const int t_length, const int s_length, const int z_length, const double Center_t,
                                   const double Center_s, const double Center_z, const int LBeta, const int LP,
                                   const int LU, const int LG, const double Distance, const double *resolution2,
                                   const int t, const float BetaScanInt, const float dU, const double PInt) {
    return finish(ct_IterativeFDKerrCompute(Pic, ErrorSlicecuda, BetaScanRange, Udomain, Pdomain, G, Size, t_length,
                                            s_length, z_length, Center_t, Center_s, Center_z, LBeta, LP, LU, LG,
                                            Distance, resolution2, t, BetaScanInt, dU, PInt),
                  "IterativeFDKerrCompute");
}

cudaError_t FDKUI(double *Display, const double *R, const double *Xigamadomain, const double *Gamadomain,
                  const double *BetaScanRange, const double betaStartAngle, const double MaxGama,
                  const double Distance, const double Distance_s2d, const int LGama, const int LBeta,
                  const int LXigama, const int *Size, const int z_length) {
    return finish(ct_FDKUI(Display, R, Xigamadomain, Gamadomain, BetaScanRange, betaStartAngle, MaxGama, Distance,
                           Distance_s2d, LGama, LBeta, LXigama, Size, z_length),
                  "FDKUI");
}

#endif
