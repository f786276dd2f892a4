/* Drives the three kernels of FDK.cu (GFunction :6, PreWeightFilter :21,
 * BackProjection :50) on the CPU.  PreWeightFilter weights its input in place
 * while other threads read it; to keep that interleaving out of the fixtures
 * it is driven twice: with an all-zero filter (the output of interest is the
 * weighted input it leaves behind) and with Distance = 1e30, where the
 * weight rounds to exactly 1 in float so only the convolution acts. */
static void fdk_G(float *G, float pint, int np)
{
    SHIM_LAUNCH(1, np, GFunction(G, pint, 0, np));
}
SHIM_EXPORT void ref_fdk_G(float *G, float pint, int np) { fdk_G(G, pint, np); }

SHIM_EXPORT void ref_fdk_weight(float *R, const float *P, const float *xi, int nb, int np, int nx,
                                double D)
{
    float *G = (float *)calloc(2 * np - 1, sizeof(float));
    float *rcov = (float *)calloc((size_t)nb * np * nx, sizeof(float));
    float pint = fabs(P[1] - P[0]);
    for (int b = 0; b < nb; ++b)
        SHIM_LAUNCH(nx, np, PreWeightFilter(rcov, R, P, xi, D, G, pint, np, nx, 0, 0, b, 0, np));
    free(rcov);
    free(G);
}

SHIM_EXPORT void ref_fdk_conv(float *rcov, float *R, const float *P, const float *xi, int nb, int np,
                              int nx)
{
    float *G = (float *)calloc(2 * np - 1, sizeof(float));
    float pint = fabs(P[1] - P[0]);
    fdk_G(G, pint, np);
    memset(rcov, 0, sizeof(float) * (size_t)nb * np * nx);
    const int limit = Filterlengthlimit;
    int gtime = (int)ceil(1.0 * np / limit);
    for (int b = 0; b < nb; ++b)
        for (int c = 0; c < gtime; ++c) {
            int g0 = c * limit, g1 = (c != gtime - 1) ? (c + 1) * limit : np;
            SHIM_LAUNCH(nx, np, PreWeightFilter(rcov, R, P, xi, 1e30, G, pint, np, nx, 0, 0, b, g0, g1));
        }
    free(G);
}

SHIM_EXPORT void ref_fdk_bp(float *disp, const float *rcov, const float *xi, const float *P,
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
        SHIM_LAUNCH(ns, nt, BackProjection(rcov, disp, size, nt, ns, nz, beta[b], D, P, xi, pint, xint,
                                           bint, minp, maxp, minx, maxx, b, np, nx, 0, 0));
}
