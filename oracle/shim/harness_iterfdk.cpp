/* Launch loop of IterativeFDKerrCompute (IterativeFDKerrCompute.cu:78-331) on
   the CPU, with the argument derivation of its MEX gateway
   (IterativeFDKerrCompute.cpp:5-31).  For s_length, z_length < 512 the
   reference launches one grid of z_length blocks x s_length threads per
   (view, U) pair, views outermost; that is the only case driven here. */
SHIM_EXPORT int ref_iterfdk_err(const float *pic, float *err, const float *beta, const float *U,
                                const double *P, const double *G, const double *size, int nt, int ns,
                                int nz, int nb, int np, int nu, int lg, double D, int t_matlab)
{
    if (ns >= 512 || nz >= 512) return 1;
    const double res[3] = {size[0] / nt, size[1] / ns, size[2] / nz};
    const double ct = size[0] / 2, cs = size[1] / 2, cz = size[2] / 2;
    const float bint = fabsf(beta[1] - beta[0]);
    const float du = fabsf(U[1] - U[0]);
    const double pint = fabs(P[1] - P[0]);
    const int t = t_matlab - 1;
    memset(err, 0, sizeof(float) * (size_t)nb * ns * nz);
    for (int b = 0; b < nb; ++b)
        for (int u = 0; u < nu; ++u)
            SHIM_LAUNCH(nz, ns, IterativeFDKerr(pic, err, U[u], P, G, size, res, ct, cs, cz, nt, ns, nz, beta[b],
                                                b, 0, 0, D, nb, np, nu, lg, t, bint, du, pint));
    return 0;
}
