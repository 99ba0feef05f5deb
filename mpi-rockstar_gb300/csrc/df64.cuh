// Double-float arithmetic: a value as an unevaluated sum hi + lo of two
// floats (about 48 significant bits), built from error-free transformations
// on the FP32 pipe -- Knuth's two-sum and the FMA two-product (Dekker; as in
// Hida, Li and Bailey's double-double and the "df64" of GPU literature).
// GB300's FP64 pipe runs at a small fraction of its FP32 rate, so sums that
// need FP64-grade accuracy but not the FP64 rounding of a fixed order (the
// batched form's parallel sums) run here instead.  The library is built
// without FMA contraction; every fused step below is an explicit fmaf.
#pragma once

namespace rsg {

struct DF {
    float hi, lo;
};

// s + e == a + b exactly
__device__ __forceinline__ DF df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// the same when |a| >= |b|
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add_f(DF x, float y) {
    DF s = df_two_sum(x.hi, y);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
    DF s = df_two_sum(x.hi, y.hi);
    DF t = df_two_sum(x.lo, y.lo);
    s = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ DF df_sqr(DF x) {
    const float p = __fmul_rn(x.hi, x.hi);
    float e = fmaf(x.hi, x.hi, -p);  // exact low part of hi * hi
    e = fmaf(__fadd_rn(x.hi, x.hi), x.lo, e);
    return df_fast_two_sum(p, e);
}
// f - y for a float f and a double-float y
__device__ __forceinline__ DF df_sub_from_f(float f, DF y) {
    DF s = df_two_sum(f, -y.hi);
    return df_fast_two_sum(s.hi, __fsub_rn(s.lo, y.lo));
}
__device__ __forceinline__ DF df_from_double(double v) {
    const float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}
__device__ __forceinline__ double df_to_double(DF x) { return (double)x.hi + (double)x.lo; }

}  // namespace rsg
