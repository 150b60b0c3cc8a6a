// tc_ff.cuh -- float-float ("double-single") arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  The mixed path solves its pressure
// tridiagonals in this form: the FP64 pipe of the part is 64x slower than
// its FP32 pipes, and the low pressure modes need more than FP32's 24 bits
// (their matrices are nearly singular).
//
// The error-free transformations are the published ones: TwoSum (Knuth,
// TAOCP vol. 2, 4.2.2), Fast2Sum (Dekker 1971) and TwoProduct by a fused
// multiply-add; the addition is the accurate double-word addition of Joldes,
// Muller and Popescu (ACM TOMS 2017, "AccurateDWPlusDW"), the product
// Dekker's double-length product with the exact hi*hi product from a fused
// multiply-add and the lo*lo term dropped.  Every operation is written with
// the _rn intrinsics so that the compiler cannot contract or reassociate
// them.
#pragma once

namespace tcgb {

struct ffv {
    float hi, lo;
};

__device__ __forceinline__ ffv ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ ffv ff_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

__device__ __forceinline__ ffv ff_add(ffv a, ffv b) {
    const ffv s = ff_two_sum(a.hi, b.hi);
    const ffv t = ff_two_sum(a.lo, b.lo);
    const ffv v = ff_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return ff_fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

// double-word plus float ("DWPlusFP" of the same paper): 10 operations
// against 20 for two double words, relative error below 2 u^2
__device__ __forceinline__ ffv ff_add_f(ffv a, float b) {
    const ffv s = ff_two_sum(a.hi, b);
    return ff_fast_two_sum(s.hi, __fadd_rn(a.lo, s.lo));
}

__device__ __forceinline__ ffv ff_neg(ffv a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ ffv ff_sub(ffv a, ffv b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ffv ff_mul(ffv a, ffv b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_fast_two_sum(p, e);
}

__device__ __forceinline__ ffv ff_from(float a) { return {a, 0.0f}; }

// Nearest float of the pair.
__device__ __forceinline__ float ff_round(ffv a) { return __fadd_rn(a.hi, a.lo); }

}  // namespace tcgb
