// solvers.cu -- row-action reconstruction on the exported system matrix.
//
// ART / Kaczmarz as the reference writes it (Iterative_algorithm/ART.m:57-75,
// commented there): for each ray j in order,
//   x <- x - lambda * a_j (a_j . x - b_j) / (a_j . a_j),
// skipping rows with a_j . a_j = 0.  Each row depends on the previous one, so
// one warp walks the rows in sequence: its lanes gather the row's entries,
// reduce the dot products in double, then scatter the update; __syncwarp
// orders the scatter before the next row's gathers.
#include "kernels.cuh"

namespace ct {

namespace {

__device__ __forceinline__ double warp_allsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(32)
kaczmarz_kernel(const long long *__restrict__ row_ptr, const int *__restrict__ col, const float *__restrict__ val,
                const float *__restrict__ b, float *x, int r0, int r1, float lambda) {
    const int lane = threadIdx.x;
    for (int row = r0; row < r1; ++row) {
        const long long e0 = row_ptr[row], e1 = row_ptr[row + 1];
        double dot = 0.0, nn = 0.0;
        for (long long e = e0 + lane; e < e1; e += 32) {
            const double v = val[e];
            dot += v * (double)x[col[e]];
            nn += v * v;
        }
        dot = warp_allsum(dot);
        nn = warp_allsum(nn);
        if (nn != 0.0) {
            const double c = (double)lambda * (dot - (double)b[row]) / nn;
            for (long long e = e0 + lane; e < e1; e += 32) {
                float *xi = x + col[e];
                *xi = (float)((double)*xi - c * (double)val[e]);
            }
        }
        __syncwarp();
    }
}

}  // namespace

}  // namespace ct

using namespace ct;

extern "C" int ct_csr_kaczmarz(const long long *d_row_ptr, const int *d_col, const float *d_val, const float *d_b,
                               float *d_x, int row_begin, int row_end, float lambda, void *stream) {
    CT_REQUIRE(d_row_ptr && d_col && d_val && d_b && d_x, "ct_csr_kaczmarz: null argument");
    CT_REQUIRE(row_begin >= 0 && row_end >= row_begin, "ct_csr_kaczmarz: bad row range");
    if (row_end == row_begin) return CT_OK;
    kaczmarz_kernel<<<1, 32, 0, as_stream(stream)>>>(d_row_ptr, d_col, d_val, d_b, d_x, row_begin, row_end, lambda);
    CT_LAUNCH_CHECK("kaczmarz_kernel");
    return CT_OK;
}
