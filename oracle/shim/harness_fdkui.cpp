/* Drives the three kernels of ImplementUI.cu (GFunction :6, PreWeightFiltration
 * :25, BackProjection :88) on the CPU, with the launch configuration of FDKUI
 * (:160-340).  Built with SHIM_THREADED: PreWeightFiltration weights its own
 * sample in place, synchronises, then convolves the row, so each of its
 * blocks runs as THREAD_SIZE_X OS threads with a real barrier.  Its grid is
 * fixed at BLOCK_SIZE_X x BLOCK_SIZE_Y blocks of THREAD_SIZE_X threads
 * (ImplementUI.h:16-20); a caller picks which of those blocks to run. */

/* Taps of every xi row, LXigama x Filter_SIZE (GFunction, launched <<<LXigama, LGama>>>). */
SHIM_EXPORT void ref_fdkui_G(double *G, double gint, const double *xi, int lx, double ds2d)
{
    SHIM_LAUNCH(lx, THREAD_SIZE_X, GFunction(G, gint, xi, ds2d));
}

/* Filtered rows (xi index xs[k], view index bs[k]) of R [view][xi][gamma]
 * (BLOCK_SIZE_X xi rows of THREAD_SIZE_X samples per view); R is weighted in
 * place as the kernel does.  rcov receives nrows x THREAD_SIZE_X values. */
SHIM_EXPORT void ref_fdkui_filter_rows(double *rcov_rows, double *R, const double *xi, const double *gama,
                                       const double *beta, double b0, double maxg, double D, double ds2d,
                                       const int *xs, const int *bs, int nrows)
{
    const double gint = fabs(gama[1] - gama[0]);
    double *G = (double *)calloc((size_t)BLOCK_SIZE_X * Filter_SIZE, sizeof(double));
    ref_fdkui_G(G, gint, xi, BLOCK_SIZE_X, ds2d);
    int maxb = 0;
    for (int k = 0; k < nrows; ++k) maxb = bs[k] > maxb ? bs[k] : maxb;
    double *rcov = (double *)calloc((size_t)(maxb + 1) * BLOCK_SIZE_X * THREAD_SIZE_X, sizeof(double));
    gridDim.x = BLOCK_SIZE_X;
    gridDim.y = BLOCK_SIZE_Y;
    for (int k = 0; k < nrows; ++k) {
        shim_launch_block(xs[k], bs[k], THREAD_SIZE_X, [&](unsigned int) {
            PreWeightFiltration(rcov, R, G, gama, beta, xi, b0, maxg, D, ds2d, gint);
        });
        memcpy(rcov_rows + (size_t)k * THREAD_SIZE_X,
               rcov + ((size_t)bs[k] * BLOCK_SIZE_X + xs[k]) * THREAD_SIZE_X, sizeof(double) * THREAD_SIZE_X);
    }
    free(rcov);
    free(G);
}

/* Backprojection of filtered data rcov [view][xi][gamma] into display
 * [z][s][t] (Size[0] x Size[1] x z_length), one launch per view (:328-335). */
SHIM_EXPORT void ref_fdkui_bp(double *display, const double *rcov, const int *size, int z_length,
                              const double *beta, int nb, double D, double ds2d, const double *gama, int lg,
                              const double *xi, int lx)
{
    const double gint = fabs(gama[1] - gama[0]);
    const double xint = fabs(xi[1] - xi[0]);
    const double bint = fabs(beta[1] - beta[0]);
    const double maxg = gama[0] > gama[lg - 1] ? gama[0] : gama[lg - 1];
    const double ming = gama[0] < gama[lg - 1] ? gama[0] : gama[lg - 1];
    const double maxx = xi[0] > xi[lx - 1] ? xi[0] : xi[lx - 1];
    const double minx = xi[0] < xi[lx - 1] ? xi[0] : xi[lx - 1];
    memset(display, 0, sizeof(double) * (size_t)size[0] * size[1] * z_length);
    for (int b = 0; b < nb; ++b)
        SHIM_LAUNCH2(size[1], z_length, size[0],
                     BackProjection(rcov, display, size, z_length, beta[b], D, ds2d, gama, xi, gint, xint, bint,
                                    ming, maxg, minx, maxx, b, lg, lx));
}
