// fdiv.h -- IEEE double division by a divisor shared by several quotients.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, and each IEEE double
// division is a sequence of several FP64 instructions.  When several quotients share
// a divisor b (e.g. u = m0/rho, v = m1/rho), one correctly rounded reciprocal
// y = RN(1/b) serves them all, and each quotient then needs one multiply and two
// fused multiply-adds: Markstein's division (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990;
// also J.-M. Muller et al., Handbook of Floating-Point Arithmetic, the FMA-based
// division and reciprocal theorems):
//   * y0 = RN32(1 / T32(b)) (an FP32 seed, relative error < 2^-22; T32 truncates b to
//     FP32 and both conversions run on bit patterns -- the integer pipe on the device,
//     where GB300 would spend FP64-unit time on conversion instructions),
//   * two Newton steps e = 1 - b y, y = y + y e (fused), which leave y faithful,
//   * one more such step, which makes y = RN(1/b) unless b's significand is all ones,
//   * per numerator: q = RN(a y), r = a - b q (exact with a fused multiply-add when q
//     is within an ulp of a/b), q' = RN(q + r y) = RN(a/b).
// The fast path covers divisors with binary exponent in [-125, 125] whose significand
// is not all ones, and numerators that are zero or have exponent in [-300, 300]
// (no intermediate overflows or underflows); anything else takes the plain division.
// Results are the IEEE quotients bit for bit, signed zeros included (a zero or exact
// quotient is returned as RN(a y), which is then exact).  Plain C++ with std::fma on
// the host and fma() on the device, so host tests check the same code.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "bitconv.h"

#if defined(__CUDACC__)
#define EBB_FDIV_HD __host__ __device__ __forceinline__
#else
#define EBB_FDIV_HD inline
#endif

namespace ebbdiv {

EBB_FDIV_HD uint64_t bits_of(double x)
{
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
}

EBB_FDIV_HD int exponent_of(double x) { return (int)((bits_of(x) >> 52) & 0x7ff) - 1023; }

struct Recip {
    double b, y;
    bool ok;  // y = RN(1/b) and the fast path applies to this divisor
};

EBB_FDIV_HD Recip recip(double b)
{
    Recip R{b, 0.0, false};
    const int e = exponent_of(b);
    if (e < -125 || e > 125 || (bits_of(b) & 0xfffffffffffffull) == 0xfffffffffffffull) return R;
    const uint64_t bb = bits_of(b);
    const uint32_t b32 = ebbbits::d2f_trunc_bits((uint32_t)(bb >> 32), (uint32_t)bb);
    float bf;
    memcpy(&bf, &b32, 4);
    const float yf = 1.0f / bf;
    uint32_t y32;
    memcpy(&y32, &yf, 4);
    const uint64_t y64 = ebbbits::f2d_bits(y32);
    double y;
    memcpy(&y, &y64, 8);
    double t = fma(-b, y, 1.0);
    y = fma(y, t, y);
    t = fma(-b, y, 1.0);
    y = fma(y, t, y);
    t = fma(-b, y, 1.0);
    R.y = fma(y, t, y);
    R.ok = true;
    return R;
}

// RN(a / R.b)
EBB_FDIV_HD double div(double a, const Recip &R)
{
    const int ea = exponent_of(a);
    if (!R.ok || (a != 0.0 && (ea < -300 || ea > 300))) return a / R.b;
    const double q = a * R.y;
    const double r = fma(-R.b, q, a);
    return r == 0.0 ? q : fma(r, R.y, q);
}

}  // namespace ebbdiv
