/* Drives FBPpara's kernels (FBPparallel.cu: GFunction :6, Filter :21,
 * BackProjection :41) on the CPU.  Filter has no in-place write, so the whole
 * chain runs as the reference host code orders it. */
SHIM_EXPORT void ref_fbppar(float *disp, const float *R, const float *T, const float *theta, int nth,
                            int ntd, const double *size, int nt, int ns)
{
    float tint = fabs(T[1] - T[0]);
    float thint = nth > 1 ? fabs(theta[1] - theta[0]) : 0.0f;
    float maxt = T[0] > T[ntd - 1] ? T[0] : T[ntd - 1];
    float mint = T[0] < T[ntd - 1] ? T[0] : T[ntd - 1];
    float *G = (float *)calloc(2 * ntd - 1, sizeof(float));
    float *rcov = (float *)calloc((size_t)nth * ntd, sizeof(float));
    float *Rw = (float *)malloc(sizeof(float) * (size_t)nth * ntd);
    memcpy(Rw, R, sizeof(float) * (size_t)nth * ntd);
    SHIM_LAUNCH(1, ntd, GFunction(G, tint, 0, ntd));
    const int limit = Filterlengthlimit;
    int gtime = (int)ceil(1.0 * ntd / limit);
    for (int c = 0; c < gtime; ++c) {
        int g0 = c * limit, g1 = (c != gtime - 1) ? (c + 1) * limit : ntd;
        SHIM_LAUNCH(nth, ntd, Filter(rcov, Rw, G, tint, ntd, 0, 0, g0, g1));
    }
    memset(disp, 0, sizeof(float) * (size_t)nt * ns);
    for (int b = 0; b < nth; ++b)
        SHIM_LAUNCH(ns, nt, BackProjection(rcov, disp, size, nt, ns, theta[b], T, tint, thint, mint, maxt,
                                           b, ntd, nth, 0, 0));
    free(Rw);
    free(rcov);
    free(G);
}
