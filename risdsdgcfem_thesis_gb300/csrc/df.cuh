// df.cuh -- double-float numbers: the unevaluated sum hi + lo of two FP32
// values (|lo| <= ulp(hi)/2 after normalisation), about 48 significant bits.
//
// GB300 runs FP32 arithmetic about 60x faster than FP64, so products that
// need more than FP32 but less than FP64 accuracy (the mixed path's
// recomputed residual b - A y) run much faster on pairs of FP32 values.
//
// The building blocks are the classical error-free transformations: TwoSum
// (Knuth, The Art of Computer Programming vol. 2, 4.2.2), Fast2Sum (Dekker,
// "A floating-point technique for extending the available precision", 1971)
// and TwoProd through a fused multiply-add. The double-word operations are
// SloppyDWPlusDW, DWTimesFP3 and DWTimesDW1 of Joldes, Muller and Popescu,
// "Tight and rigorous error bounds for basic building blocks of double-word
// arithmetic", ACM TOMS 44(2), 2017. Addition is the sloppy form: under
// cancellation its error is bounded by about 2^-48 of the operands (not of
// the result), the same order as the operands' own representation error.
//
// Every FP32 operation is an explicit round-to-nearest intrinsic, which the
// compiler never contracts into a fused multiply-add: a contraction would
// break the error-free transformations.
#pragma once

namespace femgb {

struct DF {
    float hi, lo;
    DF() = default;
    __host__ __device__ constexpr DF(float h, float l) : hi(h), lo(l) {}
    // nearest double-float of an FP64 value (exact to 2^-48 relative)
    // (conversions to float round to nearest)
    __host__ __device__ explicit DF(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

__device__ __forceinline__ DF df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// Requires |a| >= |b| (or a == 0).
__device__ __forceinline__ DF df_fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DF df_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ DF df_from_double(double v) { return DF(v); }

__device__ __forceinline__ double df_to_double(DF a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ DF operator+(DF x, DF y)
{
    const DF s = df_two_sum(x.hi, y.hi);
    return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ DF operator-(DF x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ DF operator-(DF x, DF y) { return x + (-y); }

__device__ __forceinline__ DF operator*(DF x, float y)
{
    const DF c = df_two_prod(x.hi, y);
    return df_fast_two_sum(c.hi, __fmaf_rn(x.lo, y, c.lo));
}

__device__ __forceinline__ DF operator*(float y, DF x) { return x * y; }

__device__ __forceinline__ DF operator*(DF x, DF y)
{
    const DF c = df_two_prod(x.hi, y.hi);
    const float t = __fmul_rn(x.hi, y.lo);
    return df_fast_two_sum(c.hi, __fadd_rn(c.lo, __fmaf_rn(x.lo, y.hi, t)));
}

__device__ __forceinline__ DF& operator+=(DF& x, DF y) { return x = x + y; }
__device__ __forceinline__ DF& operator-=(DF& x, DF y) { return x = x - y; }

// Quotient (DWDivDW2 of the paper above): the FP32 quotient of the leading
// parts, corrected by the remainder x - y t_h.
__device__ __forceinline__ DF operator/(DF x, DF y)
{
    const float th = __fdiv_rn(x.hi, y.hi);
    const DF r = y * th;
    const float d = __fadd_rn(__fsub_rn(x.hi, r.hi), __fsub_rn(x.lo, r.lo));
    return df_fast_two_sum(th, __fdiv_rn(d, y.hi));
}

// Square root: the FP32 root s of the leading part, corrected by
// (x - s^2) / (2 s) (one Newton step in double-float accuracy).
__device__ __forceinline__ DF df_sqrt(DF x)
{
    if (!(x.hi > 0.f)) return DF(__fsqrt_rn(x.hi), 0.f);  // 0, or NaN below zero
    const float sr = __fsqrt_rn(x.hi);
    const DF s2 = df_two_prod(sr, sr);
    const float rem = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, s2.hi), s2.lo), x.lo);
    return df_fast_two_sum(sr, __fdiv_rn(rem, __fmul_rn(2.f, sr)));
}

__device__ __forceinline__ DF df_abs(DF x) { return x.hi < 0.f ? -x : x; }

// Order of normalised double-floats (the leading parts decide unless equal).
__device__ __forceinline__ bool operator<(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(DF a, DF b) { return b < a; }
__device__ __forceinline__ bool operator<=(DF a, DF b) { return !(b < a) && a.hi == a.hi && b.hi == b.hi; }

}  // namespace femgb
