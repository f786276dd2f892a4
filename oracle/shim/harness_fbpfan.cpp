/* Drives the kernels of FBPfan.cu (GFunction :6, PreWeightFilter :21,
 * BackProjection :45) on the CPU; the in-place weight is isolated the same
 * way as for FDK (zero filter / Rscan = 1e30). */
SHIM_EXPORT void ref_fbpfan_weight(float *R, const float *P, int nb, int np, double rscan)
{
    float *G = (float *)calloc(2 * np - 1, sizeof(float));
    float *rcov = (float *)calloc((size_t)nb * np, sizeof(float));
    float pint = fabs(P[1] - P[0]);
    SHIM_LAUNCH(nb, np, PreWeightFilter(rcov, R, G, pint, P, np, 0, 0, 0, np, rscan));
    free(rcov);
    free(G);
}

SHIM_EXPORT void ref_fbpfan_conv(float *rcov, float *R, const float *P, int nb, int np)
{
    float *G = (float *)calloc(2 * np - 1, sizeof(float));
    float pint = fabs(P[1] - P[0]);
    SHIM_LAUNCH(1, np, GFunction(G, pint, 0, np));
    memset(rcov, 0, sizeof(float) * (size_t)nb * np);
    const int limit = Filterlengthlimit;
    int gtime = (int)ceil(1.0 * np / limit);
    for (int c = 0; c < gtime; ++c) {
        int g0 = c * limit, g1 = (c != gtime - 1) ? (c + 1) * limit : np;
        SHIM_LAUNCH(nb, np, PreWeightFilter(rcov, R, G, pint, P, np, 0, 0, g0, g1, 1e30));
    }
    free(G);
}

SHIM_EXPORT void ref_fbpfan_bp(float *disp, const float *rcov, const float *P, const float *beta,
                               int nb, int np, const double *size, int nt, int ns, double rscan)
{
    float pint = fabs(P[1] - P[0]);
    float bint = nb > 1 ? fabs(beta[1] - beta[0]) : 0.0f;
    float maxp = P[0] > P[np - 1] ? P[0] : P[np - 1];
    float minp = P[0] < P[np - 1] ? P[0] : P[np - 1];
    memset(disp, 0, sizeof(float) * (size_t)nt * ns);
    for (int b = 0; b < nb; ++b)
        SHIM_LAUNCH(ns, nt, BackProjection(rcov, disp, size, nt, ns, beta[b], P, pint, bint, minp, maxp,
                                           b, np, nb, 0, 0, rscan));
}
