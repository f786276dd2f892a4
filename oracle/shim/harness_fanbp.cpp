/* Launch loop of FBPfan in BackprojectionFan2D.cu (:119-349), one launch per view. */
SHIM_EXPORT void ref_fan_bp(float *disp, const float *R, const float *P, const float *beta, int nb,
                            int np, const double *size, int nt, int ns, double rscan)
{
    float pint = fabs(P[1] - P[0]);
    float bint = nb > 1 ? fabs(beta[1] - beta[0]) : 0.0f;
    float maxp = P[0] > P[np - 1] ? P[0] : P[np - 1];
    float minp = P[0] < P[np - 1] ? P[0] : P[np - 1];
    memset(disp, 0, sizeof(float) * (size_t)nt * ns);
    for (int b = 0; b < nb; ++b)
        SHIM_LAUNCH(ns, nt, BackProjection(R, disp, size, nt, ns, beta[b], P, pint, bint, minp, maxp, b,
                                           np, nb, 0, 0, rscan));
}
