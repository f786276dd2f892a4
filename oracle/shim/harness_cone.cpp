/* Launch loops for ProjectionCone (ProjectionCone_3D.cu:8) and
 * BackProjection3D (Backprojection3D.cu:8) on the CPU.  Appended after the
 * reference kernel text by oracle/build_ref.py.  Checker only. */
SHIM_EXPORT void ref_cone_fp(const float *pic, float *proj, const float *beta, const float *P,
                             const float *xi, int nt, int ns, int nz, double ct, double cs,
                             double cz, int nb, int np, int nx, double D, const double *res)
{
    for (int b = 0; b < nb; ++b)
        SHIM_LAUNCH(nx, np, ProjectionCone(pic, proj, P, xi, ct, cs, cz, res, nt, ns, nz, beta[b], b,
                                           0, 0, D, np, nx, (const float *)0));
}
