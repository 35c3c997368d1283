// bitconv.h -- float <-> double conversions on integer bit patterns.
//
// GB300 executes FP64 instructions, conversions between FP32 and FP64 included, at a
// small fraction of its FP32 rate, and the split path's final-stage update converts
// every FP32 increment to FP64 and every updated FP64 state back to its FP32 copy.
// These two functions do the same conversions with integer operations.  They are
// exact for every normal and special value and follow the flush-to-zero convention
// the split kernels are compiled with: an FP32 subnormal input converts to a signed
// zero, and a double of magnitude below 2^-126 (the smallest FP32 normal) converts to
// a signed zero.  Rounding of double -> float is to nearest, ties to even; overflow
// gives infinity; NaN stays NaN (quiet).  Plain C++ (no CUDA types) so that host
// tests compile the same code.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define EBB_HD __host__ __device__ __forceinline__
#else
#define EBB_HD inline
#endif

namespace ebbbits {

// IEEE binary32 pattern -> binary64 pattern
EBB_HD uint64_t f2d_bits(uint32_t f)
{
    const uint32_t e = (f >> 23) & 0xffu, m = f & 0x7fffffu;
    uint32_t hi = f & 0x80000000u, lo = 0u;
    if (e != 0u) {
        hi |= ((e == 0xffu ? 0x7ffu : e + 896u) << 20) | (m >> 3);
        lo = m << 29;
    }
    return ((uint64_t)hi << 32) | lo;
}

// IEEE binary64 pattern (high and low words) -> binary32 pattern
EBB_HD uint32_t d2f_bits(uint32_t hi, uint32_t lo)
{
    const uint32_t s = hi & 0x80000000u, mh = hi & 0xfffffu;
    const int E = (int)((hi >> 20) & 0x7ffu);
    if (E == 0x7ff) return s | 0x7f800000u | ((mh | lo) ? 0x400000u : 0u);
    const int e = E - 896;  // binary32 biased exponent
    if (e >= 255) return s | 0x7f800000u;
    if (e <= 0) return s;
    const uint32_t keep = (mh << 3) | (lo >> 29), rem = lo & 0x1fffffffu;
    const uint32_t up = (rem > 0x10000000u || (rem == 0x10000000u && (keep & 1u))) ? 1u : 0u;
    return s | (((uint32_t)e << 23) + keep + up);  // a carry out of the mantissa bumps the exponent
}

// IEEE binary64 pattern -> binary32 pattern with the mantissa truncated (not rounded)
// to 23 bits, for range filters: relative error below 2^-23 for magnitudes in
// [2^-126, 2^128); smaller magnitudes give a signed zero, larger ones (infinities and
// NaN included) a signed infinity.
EBB_HD uint32_t d2f_trunc_bits(uint32_t hi, uint32_t lo)
{
    const uint32_t mag = hi & 0x7fffffffu, sgn = hi & 0x80000000u;
    const uint32_t f = sgn | ((mag - (896u << 20)) << 3) | (lo >> 29);
    return mag < (897u << 20) ? sgn : (mag >= (1151u << 20) ? (sgn | 0x7f800000u) : f);
}

}  // namespace ebbbits
