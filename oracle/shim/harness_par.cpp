/* Launch loop for ProjectionParallel (ProjectionParallel_2D.cu:9) on the CPU. */
SHIM_EXPORT void ref_par_fp(const float *pic, double *proj, const double *theta,
                            const double *trange, int h, int w, double cy, double cx, int nth,
                            int nt, const double *res)
{
    SHIM_LAUNCH(nth, nt, ProjectionParallel(pic, proj, trange, theta, cy, cx, res, h, w, nt, 0, 0));
}
