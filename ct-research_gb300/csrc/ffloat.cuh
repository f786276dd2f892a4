// ffloat.cuh -- float-float (double-single) arithmetic for the backprojectors'
// detector coordinates.
//
// A value is hi + lo with |lo| <= ulp(hi) / 2: about 48 significant bits, the
// precision the reference's FP64 coordinates need (an interpolation index is
// floor(|P - P0| / PInt), discontinuous, with weights |P - P[i]| / PInt), at FP32
// instruction rates (GB300 runs FP64 at a small fraction of FP32).  Products
// use the FMA error term (Dekker / Ogita-Rump-Oishi TwoProduct), sums Knuth's
// TwoSum.  Every operation is written out, so the compiler cannot contract or
// reassociate it.
#pragma once
#include <cuda_runtime.h>

namespace ct {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_from(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ ff ff_fast2sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_2sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = ff_2sum(a.hi, b.hi);
    return ff_fast2sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_abs(ff a) { return a.hi < 0.0f ? ff_neg(a) : a; }

__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return ff_fast2sum(p, e);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_fast2sum(p, e);
}

// a / b: a first quotient, the remainder a - q b in float-float, one correction
__device__ __forceinline__ ff ff_div(ff a, ff b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const ff r = ff_sub(a, ff_mul_f(b, q1));
    return ff_fast2sum(q1, __fdiv_rn(r.hi, b.hi));
}

// a / b from an approximate reciprocal r of b.hi (a few ulp): the remainder
// a - q1 b is exact in float-float, so the first quotient's error is taken
// back and the result is within ~2^-44 of a / b (relative)
__device__ __forceinline__ ff ff_div_r(ff a, ff b, float r) {
    const float q1 = __fmul_rn(a.hi, r);
    const ff rem = ff_sub(a, ff_mul_f(b, q1));
    return ff_fast2sum(q1, __fmul_rn(rem.hi, r));
}

// floor(a) for |a| < 2^31: floor of hi, one lower when hi is an integer and lo < 0
__device__ __forceinline__ int ff_floor(ff a) {
    const float f = floorf(a.hi);
    return (int)f - ((f == a.hi && a.lo < 0.0f) ? 1 : 0);
}

// a * 2^32 as a 64-bit fixed-point value (32 fraction bits), |a| < 2^31
__device__ __forceinline__ long long ff_fixed32(ff a) {
    return __float2ll_rn(__fmul_rn(a.hi, 4294967296.0f)) + __float2ll_rn(__fmul_rn(a.lo, 4294967296.0f));
}

}  // namespace ct
