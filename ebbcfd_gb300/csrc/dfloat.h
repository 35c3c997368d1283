// dfloat.h -- double-float arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| <= ulp(hi) / 2, about 46 significant bits.  Error bounds
// (checked on the host against exact rational arithmetic): a product, quotient or square
// root within a few units of 2^-46 of the exact result, relative; a sum or difference
// within a few units of 2^-46 of |a| + |b| -- the operands' own representation error,
// so under cancellation the result is as accurate as its operands allow.
//
// GB300 executes FP32 at 64 times its FP64 rate, so an operation that costs 8-25 FP32
// instructions still takes far less pipe time than one FP64 instruction.  The
// algorithms are the classical error-free transformations: Knuth's two-sum and
// Dekker's fast two-sum (the exact sum of two floats as a float and its rounding
// error), the FMA-based two-product, and Dekker's double-length multiplication,
// division and square root built on them (T. J. Dekker, "A floating-point technique
// for extending the available precision", Numer. Math. 18, 1971; J.-M. Muller et al.,
// Handbook of Floating-Point Arithmetic, the double-word algorithms).  They need IEEE
// rounding of every FP32 operation; multiply-add contraction only removes roundings
// where the algorithms already use fmaf.  The range is FP32's: values between ~1e-30
// and ~1e30 keep the full precision.
//
// `df` is a value type with the arithmetic operators, comparisons and the math
// functions the solver kernels use (found by argument-dependent lookup), so the
// kernels templated on their arithmetic type compile for it unchanged.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define EBB_DF_HD __host__ __device__ __forceinline__
#else
#define EBB_DF_HD inline
#endif

namespace ebbdf {

struct df {
    float hi, lo;
    df() = default;
    // exact for doubles within FP32's range (hi = RN32(x), lo = RN32(x - hi)); an
    // infinite or NaN x gives lo = 0
    EBB_DF_HD constexpr df(double x)
        : hi((float)x), lo(((float)x - (float)x) == 0.0f ? (float)(x - (double)(float)x) : 0.0f)
    {
    }
    EBB_DF_HD constexpr df(float x) : hi(x), lo(0.0f) {}
    EBB_DF_HD constexpr df(int x) : df((double)x) {}
    EBB_DF_HD constexpr df(float h, float l) : hi(h), lo(l) {}
    EBB_DF_HD explicit operator double() const { return (double)hi + (double)lo; }
    EBB_DF_HD explicit operator float() const { return hi + lo; }
};

// s + e = a + b exactly (Knuth)
EBB_DF_HD df two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return df(s, (a - (s - bb)) + (b - bb));
}
// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker)
EBB_DF_HD df fast_two_sum(float a, float b)
{
    const float s = a + b;
    return df(s, b - (s - a));
}
// p + e = a * b exactly (FMA)
EBB_DF_HD df two_prod(float a, float b)
{
    const float p = a * b;
    return df(p, fmaf(a, b, -p));
}

// Dekker's addition: the high words summed exactly, the low words added to the error
// term, one renormalisation (11 FP32 operations).  Its error is bounded by the low
// words' rounding, relative to |a| + |b|; the two-sum of the low words that would make
// it relative to |a + b| costs 9 more operations and buys nothing here, since every
// operand already carries a representation error of that size.
EBB_DF_HD df operator+(df a, df b)
{
    const df s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
EBB_DF_HD df operator-(df a) { return df(-a.hi, -a.lo); }
EBB_DF_HD df operator-(df a, df b) { return a + (-b); }
// The product: the high words' exact product and the cross terms (four FP32
// operations), left without the final renormalisation -- its low word may reach about
// 1.5 units in the last place of its high word instead of 0.5.  Every operation here
// takes such an operand: the sums and products use the low word as a correction and
// the quotient and square root only the high word as a first approximation, so the
// error bounds stay those of the renormalised form; comparisons of two values within
// a unit of 2^-46 of each other may order them either way.
EBB_DF_HD df operator*(df a, df b)
{
    df p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return p;
}
// a double-float times an FP32 number
EBB_DF_HD df mul_f(df a, float b)
{
    df p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
// a / b: a first quotient from the FP32 reciprocal, two double-word corrections
EBB_DF_HD df operator/(df a, df b)
{
    const float y = 1.0f / b.hi;
    const float q1 = a.hi * y;
    const df r = a - mul_f(b, q1);
    const float q2 = r.hi * y;
    const df r2 = r - mul_f(b, q2);
    const float q3 = r2.hi * y;
    const df q = fast_two_sum(q1, q2);
    return fast_two_sum(q.hi, q.lo + q3);
}
EBB_DF_HD df &operator+=(df &a, df b) { return a = a + b; }
EBB_DF_HD df &operator-=(df &a, df b) { return a = a - b; }
EBB_DF_HD df &operator*=(df &a, df b) { return a = a * b; }
EBB_DF_HD df &operator/=(df &a, df b) { return a = a / b; }

EBB_DF_HD bool operator<(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
EBB_DF_HD bool operator>(df a, df b) { return b < a; }
EBB_DF_HD bool operator<=(df a, df b) { return !(b < a) && a.hi == a.hi && b.hi == b.hi; }
EBB_DF_HD bool operator>=(df a, df b) { return b <= a; }
EBB_DF_HD bool operator==(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }
EBB_DF_HD bool operator!=(df a, df b) { return !(a == b); }

EBB_DF_HD bool isnan(df a) { return a.hi != a.hi || a.lo != a.lo; }
EBB_DF_HD df fabs(df a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f) ? -a : a; }
// NaN arguments: the other argument, as fmin/fmax do
EBB_DF_HD df fmin(df a, df b) { return isnan(a) ? b : (isnan(b) ? a : (b < a ? b : a)); }
EBB_DF_HD df fmax(df a, df b) { return isnan(a) ? b : (isnan(b) ? a : (a < b ? b : a)); }
// sqrt(a): the FP32 root plus one Newton correction in double-word arithmetic
EBB_DF_HD df sqrt(df a)
{
    if (!(a.hi > 0.0f)) return df(sqrtf(a.hi), 0.0f);  // zero, negative (NaN) or NaN
    const float s = sqrtf(a.hi);
    const df e = a - two_prod(s, s);
    return fast_two_sum(s, e.hi / (2.0f * s));
}

}  // namespace ebbdf
