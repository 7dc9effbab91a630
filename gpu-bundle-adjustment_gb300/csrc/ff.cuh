// Float-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers (about 48 significant bits). GB300 issues FP32 FMAs at 64x its FP64
// rate, so products that need more than FP32 accuracy (the iterative-refinement
// residual of the Schur system, its right-hand side) run here instead of in FP64.
//
// Building blocks are the classical error-free transforms:
//   two_sum   s + e = a + b exactly                (Knuth, TAOCP vol. 2, 4.2.2)
//   two_prod  p + e = a * b exactly, via one FMA   (the FMA form of Dekker's product)
// and sums of products accumulate as in Dot2 (Ogita, Rump, Oishi, "Accurate sum
// and dot product", SIAM J. Sci. Comput. 26(6), 2005): the rounding errors of
// every product and every partial sum are collected in lo, giving a result as
// accurate as if computed in twice the working precision, error about
// u^2 * sum |terms| with u = 2^-24. Values are renormalised (norm) before they
// are multiplied again, so lo stays below half an ulp of hi there.
//
// The transforms use the _rn intrinsics, which the compiler never contracts
// into FMAs, so they stay exact whatever the fmad setting.
#pragma once

#include <cuda_runtime.h>

namespace gba {
namespace ffa {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

__device__ __forceinline__ ff norm(ff a) {
    const float s = __fadd_rn(a.hi, a.lo);
    return {s, __fsub_rn(a.lo, __fsub_rn(s, a.hi))};
}

__device__ __forceinline__ ff add(ff a, ff b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    return {s, __fadd_rn(e, __fadd_rn(a.lo, b.lo))};
}

// acc += a * b (FP32 a exact, float-float b)
__device__ __forceinline__ void madd(ff& acc, float a, ff b) {
    float p, e, s, r;
    two_prod(a, b.hi, p, e);
    two_sum(acc.hi, p, s, r);
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(r, __fmaf_rn(a, b.lo, e)));
}

// acc += a * b (both float-float)
__device__ __forceinline__ void madd(ff& acc, ff a, ff b) {
    float p, e, s, r;
    two_prod(a.hi, b.hi, p, e);
    two_sum(acc.hi, p, s, r);
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(r, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e))));
}

__device__ __forceinline__ ff neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff sub(ff a, ff b) { return add(a, neg(b)); }

// a * b, renormalised
__device__ __forceinline__ ff mul(ff a, ff b) {
    float p, e;
    two_prod(a.hi, b.hi, p, e);
    return norm({p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e))});
}

// a / b (b normalised, non-zero): Dekker's division, one correction of the
// FP32 quotient q1 by the exactly computed remainder a - q1 b.
__device__ __forceinline__ ff div(ff a, ff b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    float p, e;
    two_prod(q1, b.hi, p, e);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), __fmaf_rn(-q1, b.lo, a.lo));
    return norm({q1, __fdiv_rn(r, b.hi)});
}

// sqrt(a) for a > 0 (normalised): the FP32 root y corrected by (a - y^2) / 2y.
__device__ __forceinline__ ff sqrt(ff a) {
    const float y = __fsqrt_rn(a.hi);
    float p, e;
    two_prod(y, y, p, e);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), a.lo);
    return norm({y, __fdiv_rn(r, __fmul_rn(2.f, y))});
}

// Nearest float-float to an FP64 value (exact for |d| in FP32's normal range
// and 48 significant bits).
__device__ __forceinline__ ff from_double(double d) {
    const float h = __double2float_rn(d);
    return {h, __double2float_rn(d - static_cast<double>(h))};
}

__device__ __forceinline__ double to_double(ff a) { return static_cast<double>(a.hi) + static_cast<double>(a.lo); }

__device__ __forceinline__ ff shfl_up(ff a, int d) {
    return {__shfl_up_sync(0xffffffffu, a.hi, d), __shfl_up_sync(0xffffffffu, a.lo, d)};
}

__device__ __forceinline__ ff shfl_xor(ff a, int m) {
    return {__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m)};
}

}  // namespace ffa
}  // namespace gba
