/* Launch loop of BackPro (Backprojection3D.cu:294-557): one launch per view,
 * float range values computed on the host as the reference does (:304-311). */
SHIM_EXPORT void ref_cone_bp(float *disp, const float *R, const float *xi, const float *P,
                             const float *beta, double D, int nb, int np, int nx,
                             const double *size, int nt, int ns, int nz)
{
    float pint = fabs(P[1] - P[0]);
    float xint = fabs(xi[1] - xi[0]);
    float bint = nb > 1 ? fabs(beta[1] - beta[0]) : 0.0f;
    float maxp = P[0] > P[np - 1] ? P[0] : P[np - 1];
    float minp = P[0] < P[np - 1] ? P[0] : P[np - 1];
    float maxx = xi[0] > xi[nx - 1] ? xi[0] : xi[nx - 1];
    float minx = xi[0] < xi[nx - 1] ? xi[0] : xi[nx - 1];
    memset(disp, 0, sizeof(float) * (size_t)nt * ns * nz);
    for (int b = 0; b < nb; ++b)
        SHIM_LAUNCH(ns, nt, BackProjection3D(R, disp, size, nt, ns, nz, beta[b], D, P, xi, pint, xint,
                                             bint, minp, maxp, minx, maxx, b, np, nx, 0, 0));
}
