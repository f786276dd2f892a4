// sysmat.cu -- the projectors' system matrix as CSR.
//
// The reference builds its system matrices on the CPU in MATLAB
// (GenSysMatFan.m, GenSysMatParal.m, GenSysMatCircular3D.m: a Siddon walk per
// ray, sparse(L, J, W)), and SIRT.m iterates with them (SIRT.m:79).  Here the
// rows come from the GPU tracer itself: each ray is walked with the forward
// projectors' face and voxel rules and walk (cone_setup.cuh, fan2d_dev.cuh,
// siddon.cuh), so A x equals the projector's output to float rounding, and
// rays that graze a grid plane are walked by the FP64 reference walk as the
// projector does (ref_walk.cu).  Rows are rays in sinogram order, columns
// voxel indices in the [z][s][t] layout, values segment lengths in mm;
// pieces of zero length are dropped.
//
// Two passes: count the entries of every row into row_ptr[row + 1], scan,
// then write the entries at row_ptr[row].
#include <cub/device/device_scan.cuh>

#include "cone_setup.cuh"
#include "fan2d_dev.cuh"
#include "kernels.cuh"
#include "siddon.cuh"

namespace ct {

namespace {

// Walk one ray and count (FILL false) or write (FILL true) its entries.
template <bool FILL>
__device__ __forceinline__ int csr_walk(RayWalk &w, int nmax, long long base, int *__restrict__ col,
                                        float *__restrict__ val) {
    float acur = 0.0f;
    int n = 0, prev = -1;
    for (int it = 0; it < w.nseg; ++it) {
        float len;
        int vox;
        if (it + 1 < w.nseg) {
            walk_step(w, acur, nmax, len, vox);
        } else {   // the last segment ends at the exit
            len = w.L - acur;
            vox = w.idx;
        }
        if (!(len > 0.0f)) continue;
        const float v = len * w.scale;
        if (vox == prev) {
            if (FILL) val[base + n - 1] += v;
            continue;
        }
        if (FILL) {
            col[base + n] = vox;
            val[base + n] = v;
        }
        ++n;
        prev = vox;
    }
    return n;
}

constexpr int SM_BX = 32, SM_BY = 4;

template <bool FILL>
__global__ void __launch_bounds__(SM_BX * SM_BY)
cone_sysmat_kernel(const ConeGeom g, int v0, long long *__restrict__ row_ptr, int *__restrict__ col,
                   float *__restrict__ val, const GrazeList gl) {
    const int p = blockIdx.x * SM_BX + threadIdx.x;
    const int x = blockIdx.y * SM_BY + threadIdx.y;
    const int vl = blockIdx.z;
    if (p >= g.np || x >= g.nx) return;
    const int v = v0 + vl;
    const long long row = ((long long)vl * g.nx + x) * g.np + p;
    RayWalk w;
    const bool hit = ray_setup(g, v, p, x, false, w);
    if (hit && w.grazing) {          // walked by the FP64 reference walk
        const unsigned long long r = (unsigned long long)(((long long)v * g.nx + x) * g.np + p);
        graze_push(gl, r, r);
        if (!FILL) row_ptr[row + 1] = 0;
        return;
    }
    const int n = hit ? csr_walk<FILL>(w, g.nt * g.ns * g.nz - 1, FILL ? row_ptr[row] : 0, col, val) : 0;
    if (!FILL) row_ptr[row + 1] = n;
}

template <bool FILL>
__global__ void __launch_bounds__(128)
fan_sysmat_kernel(const FanGeom g, long long *__restrict__ row_ptr, int *__restrict__ col, float *__restrict__ val,
                  const GrazeList gl) {
    const long long r = (long long)blockIdx.x * 128 + threadIdx.x;
    if (r >= (long long)g.nb * g.np) return;
    RayWalk w;
    const bool hit = fan_ray_setup(g, r, w);
    if (hit && w.grazing) {
        graze_push(gl, (unsigned long long)r, (unsigned long long)r);
        if (!FILL) row_ptr[r + 1] = 0;
        return;
    }
    const int n = hit ? csr_walk<FILL>(w, g.nt * g.ns - 1, FILL ? row_ptr[r] : 0, col, val) : 0;
    if (!FILL) row_ptr[r + 1] = n;
}

}  // namespace

int cone_sysmat_launch(const ConeGeom &g, int v0, int nv, long long *row_ptr, int *col, float *val, bool fill,
                       const GrazeList &gl, cudaStream_t st) {
    CT_REQUIRE(nv > 0 && nv <= 65535 && v0 >= 0 && v0 + nv <= g.nb, "sysmat: view range out of bounds");
    CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(*gl.count), st), "graze list reset");
    dim3 block(SM_BX, SM_BY), grid((g.np + SM_BX - 1) / SM_BX, (g.nx + SM_BY - 1) / SM_BY, nv);
    if (fill) cone_sysmat_kernel<true><<<grid, block, 0, st>>>(g, v0, row_ptr, col, val, gl);
    else cone_sysmat_kernel<false><<<grid, block, 0, st>>>(g, v0, row_ptr, col, val, gl);
    CT_LAUNCH_CHECK("cone_sysmat_kernel");
    const long long r0 = (long long)v0 * g.nx * g.np;
    return cone_sysmat_ref_launch(g, r0, row_ptr, col, val, fill, gl, st);
}

int fan_sysmat_launch(const FanGeom &g0, long long *row_ptr, int *col, float *val, bool fill, const GrazeList &gl,
                      cudaStream_t st) {
    FanGeom g = g0;
    fan_geom_derive(g);
    CT_CUDA(cudaMemsetAsync(gl.count, 0, sizeof(*gl.count), st), "graze list reset");
    const long long rays = (long long)g.nb * g.np;
    const unsigned blocks = (unsigned)((rays + 127) / 128);
    if (fill) fan_sysmat_kernel<true><<<blocks, 128, 0, st>>>(g, row_ptr, col, val, gl);
    else fan_sysmat_kernel<false><<<blocks, 128, 0, st>>>(g, row_ptr, col, val, gl);
    CT_LAUNCH_CHECK("fan_sysmat_kernel");
    return fan_sysmat_ref_launch(g, row_ptr, col, val, fill, gl, st);
}

int csr_scan(long long *row_ptr, int n, void **tmp, size_t *tmp_bytes, cudaStream_t st) {
    CT_CUDA(cudaMemsetAsync(row_ptr, 0, sizeof(long long), st), "row_ptr[0]");
    size_t need = 0;
    CT_CUDA(cub::DeviceScan::InclusiveSum(nullptr, need, row_ptr + 1, row_ptr + 1, n, st), "scan size");
    if (need > *tmp_bytes) {
        if (*tmp) cudaFree(*tmp);
        *tmp = nullptr;
        *tmp_bytes = 0;
        CT_CUDA(cudaMalloc(tmp, need), "scan scratch");
        *tmp_bytes = need;
    }
    CT_CUDA(cub::DeviceScan::InclusiveSum(*tmp, need, row_ptr + 1, row_ptr + 1, n, st), "scan");
    return CT_OK;
}

}  // namespace ct
