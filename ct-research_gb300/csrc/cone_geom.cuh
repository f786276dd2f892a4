// cone_geom.cuh -- cone-beam geometry shared by the cone kernels.
#pragma once
#include <cmath>

#include "ct_common.cuh"

namespace ct {

// Per-view source position and the D sin / D cos terms of the ray direction, FP64.
struct __align__(16) ViewSrc {
    double src_t, src_s, dsb, dcb;
};

// Geometry of one cone scan in the reference's conventions
// (ProjectionCone_3D.cpp:5-22, Backprojection3D.cu:20-27).
struct ConeGeom {
    int nt, ns, nz;          // volume size (t fastest)
    int nb, np, nx;          // views, detector columns (P), detector rows (xi)
    double size[3];          // volume extent in mm
    double res[3];           // voxel pitch Size/length
    double ires[3];          // 1 / res
    double D;                // source to rotation centre
    const double2 *trig;     // per view (sin beta, cos beta), float-overload values widened
    const ViewSrc *vsrc;     // per view source and D sin / D cos, FP64
    const float *P;          // detector column coordinates
    const float *xi;         // detector row coordinates
    // The same values in the other precision, so that hot loops convert
    // nothing (a conversion to or from double issues on the FP64 pipe, which
    // runs at a small fraction of the FP32 rate on this GPU):
    const float2 *trigf;     // trig exactly (the values are floats widened)
    const float4 *vsrcf;     // vsrc rounded to float: (src_t, src_s, D sin, D cos)
    const double *Pd, *xid;  // P and xi widened
    double ext[3];           // box extent n * res per axis
    float extf[3];           // ext rounded to float
    float iresf[3];          // ires rounded to float
    double srcz;             // source z: size[2] / 2
    float srczf;
    // detector sampling as the reference derives it (Backprojection3D.cu:304-311)
    float pint, xint, bint;  // |P1-P0|, |xi1-xi0|, |beta1-beta0|
    float minp, maxp, minx, maxx;
    float p0, x0;            // P[0], xi[0]
    float psgn, xsgn;        // +1 for ascending domains, -1 for descending
    // Row table of the backprojectors: for x < nx - 1, (x - q(xi[x]), q(xi[x+1]) - x)
    // with q(v) = |v - xi[0]| / xint the reference's row quotient (in double);
    // the bilinear row weights |xi - xi[x]| / xint and |xi[x+1] - xi| / xint of a
    // point with quotient x + f are then |f + tab.x| and |tab.y - f|.
    const float2 *xtab;
    // View order of the forward projector's launch, chunk by chunk of
    // kFpViewChunk consecutive views: in each chunk the views whose detector
    // columns run closer to t (read from the [z][s][t] volume) first, then those
    // read from the [z][t][s] copy, so that the views sharing a wave of blocks
    // read the same copy of the volume.  A chunk's views are contiguous in the
    // sinogram: a chunk can be projected and copied out on its own.
    const int *vorder;
    // Float-float (hi, lo) constants of the backprojector, set by
    // cone_bp_consts: D, res_z * xq, xi[0] * xq and 1 / PInt, where
    // xq = xsgn / XigamaInt is the row quotient per mm of xi.  Kernel
    // parameters, so the set-up reads them without holding registers.
    float2 bp_D, bp_rzxq, bp_x0xq, bp_ipint, bp_xq;
    // and its float constants: res_z, 1 / res_z, half voxel (t, s, z), size_z / 2,
    // iz at z = 0, D, 1 / D, 1 / PInt
    float bp_rz, bp_irz, bp_ht, bp_hs, bp_hz, bp_czf, bp_xbase, bp_Df, bp_iD, bp_ipintf;
};

// The scalar constants derived from the sizes and the voxel pitch (ext, extf,
// iresf, srcz, srczf); call again after changing res.
inline void cone_geom_derive(ConeGeom &g) {
    const int n[3] = {g.nt, g.ns, g.nz};
    for (int a = 0; a < 3; ++a) {
        g.ext[a] = n[a] * g.res[a];
        g.extf[a] = (float)g.ext[a];
        g.iresf[a] = (float)g.ires[a];
    }
    g.srcz = 0.5 * g.size[2];
    g.srczf = (float)g.srcz;
}

// Host float-float helpers for cone_bp_consts, with the operations of
// ffloat.cuh's ff_from and ff_mul (each rounded once), so that the constants
// equal what a kernel would compute from the same doubles.
inline float2 ff_from_host(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}
inline float2 ff_mul_host(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = std::fma(a.x, b.x, -p);
    e = std::fma(a.x, b.y, e);
    e = std::fma(a.y, b.x, e);
    const float s = p + e;
    return make_float2(s, e - (s - p));
}

// The backprojector's constants (bp_*) from D, res, size, xsgn, xint, x0 and
// pint; cone_bp_launch sets them on its copy of the geometry before each launch.
inline void cone_bp_consts(ConeGeom &g) {
    const float2 xq = ff_from_host((double)g.xsgn / (double)g.xint);
    g.bp_xq = xq;
    g.bp_D = ff_from_host(g.D);
    g.bp_rzxq = ff_mul_host(ff_from_host(g.res[2]), xq);
    g.bp_x0xq = ff_mul_host(make_float2(g.x0, 0.0f), xq);
    g.bp_ipint = ff_from_host(1.0 / (double)g.pint);
    g.bp_rz = (float)g.res[2];
    g.bp_irz = 1.0f / g.bp_rz;
    g.bp_ht = 0.5f * (float)g.res[0];
    g.bp_hs = 0.5f * (float)g.res[1];
    g.bp_hz = 0.5f * g.bp_rz;
    g.bp_czf = (float)(0.5 * g.size[2]);
    g.bp_xbase = (float)(0.5 * g.res[2] - 0.5 * g.size[2]);
    g.bp_Df = (float)g.D;
    g.bp_iD = 1.0f / g.bp_Df;
    g.bp_ipintf = 1.0f / g.pint;
}

}  // namespace ct
