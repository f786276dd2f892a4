/* Launch loop for ProjectionFan (ProjectionFan_2D.cu:8) on the CPU. */
SHIM_EXPORT void ref_fan_fp(const float *pic, double *proj, const double *beta, const double *P,
                            int nt, int ns, double ct, double cs, int nb, int np, double D,
                            const double *res)
{
    SHIM_LAUNCH(nb, np, ProjectionFan(pic, proj, P, beta, ct, cs, res, nt, ns, 0, 0, D, np, nb,
                                      (const double *)0));
}
