// device_math.cuh -- per-face and per-cell arithmetic of the explicit FV update,
// templated on the arithmetic type T (double for the plain path, float for the
// split path, ebbdf::df for the double-float path).  Every expression keeps the
// evaluation order of the D reference so that, compiled without multiply-add
// contraction, the double instantiation rounds exactly like it.  Reference lines are
// cited per function.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "bitconv.h"
#include "dfloat.h"
#include "fdiv.h"

namespace ebbdev {

using ebbdf::df;
// the three arithmetic types: double (plain FP64), float (split), df (double-float)
template <typename T> constexpr bool is_fp64 = std::is_same<T, double>::value;
template <typename T> constexpr bool is_fp32 = std::is_same<T, float>::value;
template <typename T> constexpr bool is_df = std::is_same<T, df>::value;

// gamma is an immutable 1.4 (source/euler.d:89)
template <typename T> struct K;
template <> struct K<double> {
    static constexpr double g = 1.4, gm1 = 1.4 - 1, gm1d = 1.4 - 1.0;
};
template <> struct K<float> {
    static constexpr float g = 1.4f, gm1 = 1.4f - 1, gm1d = 1.4f - 1.0f;
};
template <> struct K<df> {  // the double constants, as double-floats
    static constexpr df g = df(1.4), gm1 = df(1.4 - 1), gm1d = df(1.4 - 1.0);
};

// Quotients by one divisor.  FP64: one correctly rounded reciprocal of the divisor
// serves every quotient (fdiv.h: Markstein's correction per quotient), which gives the
// IEEE quotient bit for bit at about a third of the FP64 instructions of a division
// per extra quotient; FP32: plain division, as the split path's flags compile it;
// double-float: one double-word reciprocal and a double-word product per quotient
// (relative error a few units of 2^-46, a third of a double-word division's cost).
template <typename T> struct Div {
    T b;
    __device__ __forceinline__ explicit Div(T d) : b(d) {}
    __device__ __forceinline__ T operator()(T a) const { return a / b; }
};
template <> struct Div<double> {
    ebbdiv::Recip R;
    __device__ __forceinline__ explicit Div(double d) : R(ebbdiv::recip(d)) {}
    __device__ __forceinline__ double operator()(double a) const { return ebbdiv::div(a, R); }
};
template <> struct Div<df> {
    df r;
    __device__ __forceinline__ explicit Div(df d) : r(df(1.0f) / d) {}
    __device__ __forceinline__ df operator()(df a) const { return a * r; }
};

// x / 2 = 0.5 x.  FP64: on the integer pipe -- for every x whose half is a normal
// number the product is exact and is x with its exponent field lowered by one; zeros
// are returned as they are (0.5 * +-0 = +-0).  Subnormal or tiny (biased exponent < 2),
// infinite and NaN values take the FP64 multiply, behind a warp vote so that a warp
// holding none issues no FP64 instruction.  FP32: the multiply.  Double-float: both
// words halved (exact but below FP32's normal range).
template <typename T> __device__ __forceinline__ T half(T x) { return T(0.5) * x; }
template <> __device__ __forceinline__ double half<double>(double x)
{
    const int hi = __double2hiint(x), lo = __double2loint(x);
    const unsigned e = ((unsigned)hi >> 20) & 0x7ffu;
    const bool norm = e - 2u < 2045u;
    const bool zero = ((hi & 0x7fffffff) | lo) == 0;
    double y = norm ? __hiloint2double(hi - 0x00100000, lo) : x;
    if (__any_sync(__activemask(), !(norm || zero))) {
        if (!(norm || zero)) y = x * 0.5;
    }
    return y;
}
template <> __device__ __forceinline__ df half<df>(df x) { return df(0.5f * x.hi, 0.5f * x.lo); }

// 0 + x, the start of the reference's matrix-vector sums (numd Matrix * Vector adds
// each product to a zero).  It is x except that -0 becomes +0 (NaN stays NaN).  FP64:
// that rule on the bit pattern, on the integer pipe.
template <typename T> __device__ __forceinline__ T zero_plus(T x) { return T(0.0) + x; }
template <> __device__ __forceinline__ double zero_plus<double>(double x)
{
    return __double_as_longlong(x) == (long long)0x8000000000000000ull ? 0.0 : x;
}
template <> __device__ __forceinline__ df zero_plus<df>(df x) { return x.hi == 0.0f ? df(0.0f, 0.0f) : x; }

// 0 nx + 0 ny: a signed zero, -0 when both products are -0 (nx and ny negative), and
// NaN when nx or ny is infinite or NaN.  FP64: the signs on the integer pipe for finite
// normals (a warp holding a non-finite one takes the FP64 expression).
template <typename T> __device__ __forceinline__ T zero_dot(T nx, T ny) { return T(0.0) * nx + T(0.0) * ny; }
template <> __device__ __forceinline__ double zero_dot<double>(double nx, double ny)
{
    const int hx = __double2hiint(nx), hy = __double2hiint(ny);
    const bool fin = ((hx & 0x7ff00000) != 0x7ff00000) && ((hy & 0x7ff00000) != 0x7ff00000);
    double z = (hx < 0 && hy < 0) ? -0.0 : 0.0;
    if (__any_sync(__activemask(), !fin)) {
        if (!fin) z = 0.0 * nx + 0.0 * ny;
    }
    return z;
}

template <typename T> __device__ __forceinline__ T dsqrt(T x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <typename T> __device__ __forceinline__ T dpow(T x, T y) { return pow(x, y); }
template <> __device__ __forceinline__ float dpow<float>(float x, float y) { return powf(x, y); }
// double-float: the power in FP64 (constant-pressure and inflow ghost states only)
template <> __device__ __forceinline__ df dpow<df>(df x, df y) { return df(pow((double)x, (double)y)); }

// Binary exponent of |x| (biased by 1023), read on the integer pipe; 0x7ff for inf/NaN.
__device__ __forceinline__ int bexp(double x) { return (__double2hiint(x) >> 20) & 0x7ff; }
// x finite and 2^-60 <= |x| < 2^60 (and positive when pos)
__device__ __forceinline__ bool mid_range(double x, bool pos)
{
    const int h = __double2hiint(x);
    const int e = (h >> 20) & 0x7ff;
    return e >= 1023 - 60 && e < 1023 + 60 && (!pos || h >= 0);
}
__device__ __forceinline__ bool bounded(double x) { return bexp(x) < 1023 + 60; }

// source/euler.d:91-94
template <typename T> __device__ __forceinline__ T pressure(const T q[4])
{
    T a = q[1] / q[0], b = q[2] / q[0];
    return K<T>::gm1 * (q[3] - half(q[0]) * (a * a + b * b));
}

// Sign of source/euler.d:91-94's pressure without its two divisions.  The reference
// value is gm1 * (q3 - Y) with Y = 0.5 q0 ((q1/q0)^2 + (q2/q0)^2) rounded within 7 units
// in the last place; q0 q3 - 0.5 (q1^2 + q2^2) has the same sign as q3 - Y whenever it
// exceeds 2^-44 of its terms' magnitude (>= 32x the combined rounding bound), for
// states within [2^-60, 2^60].  Anything closer to zero, or outside that range, takes
// the reference's own expression, so the decision is always the reference's.

// FP32 value of any double with its mantissa truncated to 23 bits (relative error
// below 2^-23), on the integer pipe: magnitudes below 2^-126 give a signed zero, from
// 2^128 on (infinities and NaN included) a signed infinity
__device__ __forceinline__ float trunc_sat(double x)
{
    return __uint_as_float(ebbbits::d2f_trunc_bits((unsigned)__double2hiint(x), (unsigned)__double2loint(x)));
}
// x is zero or 2^-60 <= |x| < 2^60
__device__ __forceinline__ bool f32_range(double x)
{
    const unsigned mag = (unsigned)__double2hiint(x) & 0x7fffffffu;
    const unsigned e = mag >> 20;
    return (mag | (unsigned)__double2loint(x)) == 0u || (e >= 1023u - 60u && e < 1023u + 60u);
}
__device__ __forceinline__ bool pressure_negative(const double q[4])
{
    if (mid_range(q[0], true) && mid_range(q[3], true) && bounded(q[1]) && bounded(q[2])) {
        if (f32_range(q[1]) && f32_range(q[2])) {
            // first in FP32 from the truncated values: within 2^-20 of |W| + Z of the
            // FP64 W - Z, so a sign clear of 2^-17 (|W| + Z) is that of W - Z, and with
            // it the reference's (below); closer to zero, the FP64 test
            const float r = trunc_sat(q[0]), e = trunc_sat(q[3]), m1 = trunc_sat(q[1]), m2 = trunc_sat(q[2]);
            const float Wf = __fmul_rn(e, r);
            const float Zf = __fmul_rn(0.5f, __fadd_rn(__fmul_rn(m1, m1), __fmul_rn(m2, m2)));
            const float dd = __fsub_rn(Wf, Zf);
            if (fabsf(dd) > 0x1p-17f * __fadd_rn(fabsf(Wf), Zf)) return dd < 0.0f;
        }
        double W = q[3] * q[0];
        double Z = 0.5 * (q[1] * q[1] + q[2] * q[2]);
        double d = W - Z;
        if (fabs(d) > 0x1p-44 * (W + Z)) return d < 0;
    }
    return pressure(q) < 0;
}
__device__ __forceinline__ bool pressure_negative(const float q[4]) { return pressure(q) < 0; }
// Double-float: the sign of q0 q3 - 0.5 (q1^2 + q2^2) from the high words in FP32 first
// (for q0 > 0 it is the pressure's sign).  That value is within 2^-20 of |W| + Z of
// the double-float one (low words at most 2^-22 of the high ones, three roundings), so
// a sign clear of 2^-17 (|W| + Z) + 2^-100 is the double-float expression's; anything
// closer to zero, a non-positive density, NaN or overflow takes that expression.
__device__ __forceinline__ bool pressure_negative(const df q[4])
{
    const float r = q[0].hi;
    if (r > 0.0f) {
        const float W = q[3].hi * r, Z = 0.5f * (q[1].hi * q[1].hi + q[2].hi * q[2].hi);
        const float d = W - Z;
        if (fabsf(d) > 0x1p-17f * (fabsf(W) + Z) + 0x1p-100f) return d < 0.0f;
    }
    return pressure(q) < df(0.0f);
}

// source/flux.d:19-24.  Single precision rounds every operation on its own (no
// multiply-add contraction): the flux kernel's value for two equal face states and the
// update kernel's freestream correction (k_update) then agree bit for bit wherever
// they are evaluated.
template <typename T>
__device__ __forceinline__ void convective_flux(T p, T u, T v, T rho, T e, T nx, T ny, T out[4])
{
    if constexpr (is_fp32<T>) {
        const float ru = __fmul_rn(rho, u), rv = __fmul_rn(rho, v), ruv = __fmul_rn(ru, v), pe = __fadd_rn(p, e);
        const float f1 = __fadd_rn(p, __fmul_rn(rho, __fmul_rn(u, u))), h2 = __fadd_rn(p, __fmul_rn(rho, __fmul_rn(v, v)));
        const float f3 = __fmul_rn(u, pe), h3 = __fmul_rn(v, pe);
        out[0] = __fadd_rn(__fmul_rn(ru, nx), __fmul_rn(rv, ny));
        out[1] = __fadd_rn(__fmul_rn(f1, nx), __fmul_rn(ruv, ny));
        out[2] = __fadd_rn(__fmul_rn(ruv, nx), __fmul_rn(h2, ny));
        out[3] = __fadd_rn(__fmul_rn(f3, nx), __fmul_rn(h3, ny));
    } else {
        T f0 = rho * u, f1 = p + rho * (u * u), f2 = rho * u * v, f3 = u * (p + e);
        T h0 = rho * v, h1 = rho * u * v, h2 = p + rho * (v * v), h3 = v * (p + e);
        out[0] = f0 * nx + h0 * ny;
        out[1] = f1 * nx + h1 * ny;
        out[2] = f2 * nx + h2 * ny;
        out[3] = f3 * nx + h3 * ny;
    }
}

// gm1 (e - 0.5 rho (u^2 + v^2)), the pressure of source/flux.d's flux functions;
// single precision without contraction, as convective_flux
template <typename T> __device__ __forceinline__ T pressure_of(T rho, T u, T v, T e)
{
    if constexpr (is_fp32<T>)
        return __fmul_rn(K<float>::gm1,
                         __fsub_rn(e, __fmul_rn(__fmul_rn(0.5f, rho), __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)))));
    else
        return K<T>::gm1 * (e - half(rho) * (u * u + v * v));
}

template <typename T> __device__ __forceinline__ T entropy_fix(T lam, T eps)
{
    if (lam < eps) lam = (eps * eps + lam * lam) / (T(2.0) * eps);
    return lam;
}

template <typename T> __device__ __forceinline__ T max4(T a, T b, T c, T d)
{
    T m = a;
    if (b > m) m = b;
    if (c > m) m = c;
    if (d > m) m = d;
    return m;
}

// source/flux.d:224-303
template <typename T>
__device__ __forceinline__ void roe_flux(const T qL[4], const T qR[4], T nx, T ny, T out[4], T &sMax)
{
    const T gm1 = K<T>::gm1;
    T rhoL = qL[0];
    const Div<T> byL(rhoL);  // four quotients by rhoL, three by rhoR
    T uL = byL(qL[1]), vL = byL(qL[2]);
    T rvL0 = rhoL * uL, rvL1 = rhoL * vL;
    T pL = pressure_of(rhoL, uL, vL, qL[3]);
    T hL = byL(qL[3] + pL);
    T rhoR = qR[0];
    const Div<T> byR(rhoR);
    T uR = byR(qR[1]), vR = byR(qR[2]);
    T rvR0 = rhoR * uR, rvR1 = rhoR * vR;
    T pR = pressure_of(rhoR, uR, vR, qR[3]);
    T hR = byR(qR[3] + pR);

    T di = dsqrt(byL(rhoR));
    T d1 = T(1.0) / (T(1.0) + di);
    T vel0 = (di * uR + uL) * d1;
    T vel1 = (di * vR + vL) * d1;
    T u = vel0 * nx + vel1 * ny;
    T h = (di * hR + hL) * d1;
    T a = dsqrt(K<T>::gm1d * (h - half(vel0 * vel0 + vel1 * vel1)));

    T dRV0 = rvR0 - rvL0, dRV1 = rvR1 - rvL1;
    T dRho = rhoR - rhoL;
    T dRhoE = qR[3] - qL[3];

    T lam1 = fabs(u + a), lam2 = fabs(u - a), lam3 = fabs(u);
    T eps = T(0.01) * a;
    lam1 = entropy_fix(lam1, eps);
    lam2 = entropy_fix(lam2, eps);
    lam3 = entropy_fix(lam3, eps);
    sMax = max4(fabs(lam1), fabs(lam2), fabs(lam3), fabs(lam3));

    T s1 = half(lam1 + lam2);
    T s2 = half(lam1 - lam2);
    T qq = dsqrt(vel0 * vel0 + vel1 * vel1);
    T G1 = gm1 * (half(qq * qq) * dRho - (vel0 * dRV0 + vel1 * dRV1) + dRhoE);
    T G2 = -u * dRho + (dRV0 * nx + dRV1 * ny);
    const Div<T> byA(a);
    T C1 = (G1 / (a * a)) * (s1 - lam3) + byA(G2) * s2;
    T C2 = byA(G1) * s2 + (s1 - lam3) * G2;

    T fL[4], fR[4];
    convective_flux(pL, uL, vL, rhoL, qL[3], nx, ny, fL);
    convective_flux(pR, uR, vR, rhoR, qR[3], nx, ny, fR);
    T D0 = lam3 * dRho + C1;
    T D1 = lam3 * dRV0 + C1 * vel0 + C2 * nx;
    T D2 = lam3 * dRV1 + C1 * vel1 + C2 * ny;
    T D3 = lam3 * dRhoE + C1 * h + C2 * u;
    out[0] = half(fL[0] + fR[0]) - half(D0);
    out[1] = half(fL[1] + fR[1]) - half(D1);
    out[2] = half(fL[2] + fR[2]) - half(D2);
    out[3] = half(fL[3] + fR[3]) - half(D3);
}

// source/flux.d:66-141 (Roe-type averaged speed; every wave set to sMax)
template <typename T>
__device__ __forceinline__ void rusanov_flux_full(const T qL[4], const T qR[4], T nx, T ny, T out[4], T &sMax);

// With every wave speed equal to sMax the reference's s1 - sMax and s2 are exact
// zeros, so its C1 and C2 terms are signed zeros whenever G1/a^2, G2/a and G1/a are
// finite, and the flux reduces to 0.5 (fL + fR) - 0.5 sMax (qR - qL) bit for bit (up
// to the sign of exact zeros).  That holds for densities, states and sound speeds in
// the ranges checked below (integer-pipe exponent tests); outside them the full
// expression runs.  Single precision computes the reduced form directly.
template <typename T>
__device__ __forceinline__ void rusanov_flux(const T qL[4], const T qR[4], T nx, T ny, T out[4], T &sMax)
{
    if constexpr (is_fp64<T>) {
        const double *a = reinterpret_cast<const double *>(qL), *b = reinterpret_cast<const double *>(qR);
        bool ok = mid_range(a[0], true) && mid_range(b[0], true) && bounded(a[1]) && bounded(a[2]) &&
                  bounded(a[3]) && bounded(b[1]) && bounded(b[2]) && bounded(b[3]);
        if (!ok) {
            rusanov_flux_full(qL, qR, nx, ny, out, sMax);
            return;
        }
    }
    T rhoL = qL[0];
    const Div<T> byL(rhoL);
    T uL = byL(qL[1]), vL = byL(qL[2]);
    T pL = pressure_of(rhoL, uL, vL, qL[3]);
    T rhoR = qR[0];
    const Div<T> byR(rhoR);
    T uR = byR(qR[1]), vR = byR(qR[2]);
    T pR = pressure_of(rhoR, uR, vR, qR[3]);
    T rho = dsqrt(rhoL * rhoR);
    T sL = dsqrt(rhoL), sR = dsqrt(rhoR);
    const Div<T> byS(sL + sR);
    T vel0 = byS(sL * uL + sR * uR);
    T vel1 = byS(sL * vL + sR * vR);
    T u = vel0 * nx + vel1 * ny;
    T p = byS(sL * pL + sR * pR);
    T a = dsqrt(K<T>::g * (p / rho));
    if constexpr (is_fp64<T>) {
        const int e = bexp((double)a);
        if (!(e >= 1023 - 200 && e < 1023 + 100)) {
            rusanov_flux_full(qL, qR, nx, ny, out, sMax);
            return;
        }
    }
    T lam1 = fabs(u + a), lam2 = fabs(u - a), lam3 = fabs(u);
    T eps = T(0.01) * a;
    lam1 = entropy_fix(lam1, eps);
    lam2 = entropy_fix(lam2, eps);
    lam3 = entropy_fix(lam3, eps);
    T sm = max4(fabs(lam1), fabs(lam2), fabs(lam3), fabs(lam3));
    sMax = sm;
    T fL[4], fR[4];
    convective_flux(pL, uL, vL, rhoL, qL[3], nx, ny, fL);
    convective_flux(pR, uR, vR, rhoR, qR[3], nx, ny, fR);
    T dRho = rhoR - rhoL;
    T dRV0 = rhoR * uR - rhoL * uL, dRV1 = rhoR * vR - rhoL * vL;
    T dRhoE = qR[3] - qL[3];
    out[0] = half(fL[0] + fR[0]) - half(sm * dRho);
    out[1] = half(fL[1] + fR[1]) - half(sm * dRV0);
    out[2] = half(fL[2] + fR[2]) - half(sm * dRV1);
    out[3] = half(fL[3] + fR[3]) - half(sm * dRhoE);
}

template <typename T>
__device__ __forceinline__ void rusanov_flux_full(const T qL[4], const T qR[4], T nx, T ny, T out[4], T &sMax)
{
    const T gm1 = K<T>::gm1;
    T rhoL = qL[0], uL = qL[1] / rhoL, vL = qL[2] / rhoL;
    T rvL0 = rhoL * uL, rvL1 = rhoL * vL;
    T pL = pressure_of(rhoL, uL, vL, qL[3]);
    T hL = (qL[3] + pL) / rhoL;
    T rhoR = qR[0], uR = qR[1] / rhoR, vR = qR[2] / rhoR;
    T rvR0 = rhoR * uR, rvR1 = rhoR * vR;
    T pR = pressure_of(rhoR, uR, vR, qR[3]);
    T hR = (qR[3] + pR) / rhoR;

    T rho = dsqrt(rhoL * rhoR);
    T sL = dsqrt(rhoL), sR = dsqrt(rhoR);
    T vel0 = (sL * uL + sR * uR) / (sL + sR);
    T vel1 = (sL * vL + sR * vR) / (sL + sR);
    T u = vel0 * nx + vel1 * ny;
    T p = (sL * pL + sR * pR) / (sL + sR);
    T h = (sL * hL + sR * hR) / (sL + sR);
    T a = dsqrt(K<T>::g * (p / rho));

    T dRV0 = rvR0 - rvL0, dRV1 = rvR1 - rvL1;
    T dRho = rhoR - rhoL;
    T dRhoE = qR[3] - qL[3];

    T lam1 = fabs(u + a), lam2 = fabs(u - a), lam3 = fabs(u);
    T eps = T(0.01) * a;
    lam1 = entropy_fix(lam1, eps);
    lam2 = entropy_fix(lam2, eps);
    lam3 = entropy_fix(lam3, eps);
    T sm = max4(fabs(lam1), fabs(lam2), fabs(lam3), fabs(lam3));
    sMax = sm;

    T s1 = T(0.5) * (sm + sm);
    T s2 = T(0.5) * (sm - sm);
    T qq = dsqrt(vel0 * vel0 + vel1 * vel1);
    T G1 = gm1 * (((qq * qq) / T(2)) * dRho - (vel0 * dRV0 + vel1 * dRV1) + dRhoE);
    T G2 = -u * dRho + (dRV0 * nx + dRV1 * ny);
    T C1 = (G1 / (a * a)) * (s1 - sm) + G2 / a * s2;
    T C2 = (G1 / a) * s2 + (s1 - sm) * G2;

    T fL[4], fR[4];
    convective_flux(pL, uL, vL, rhoL, qL[3], nx, ny, fL);
    convective_flux(pR, uR, vR, rhoR, qR[3], nx, ny, fR);
    T D0 = sm * dRho + C1;
    T D1 = sm * dRV0 + C1 * vel0 + C2 * nx;
    T D2 = sm * dRV1 + C1 * vel1 + C2 * ny;
    T D3 = sm * dRhoE + C1 * h + C2 * u;
    out[0] = T(0.5) * (fL[0] + fR[0]) - T(0.5) * D0;
    out[1] = T(0.5) * (fL[1] + fR[1]) - T(0.5) * D1;
    out[2] = T(0.5) * (fL[2] + fR[2]) - T(0.5) * D2;
    out[3] = T(0.5) * (fL[3] + fR[3]) - T(0.5) * D3;
}

template <typename T>
__device__ __forceinline__ void inviscid_flux(int kind, const T qL[4], const T qR[4], T nx, T ny, T out[4], T &sMax)
{
    if (kind == 1)
        roe_flux(qL, qR, nx, ny, out, sMax);
    else
        rusanov_flux(qL, qR, nx, ny, out, sMax);
}

// source/flux.d:28-64.  dq[k][r] is d(q_k)/d(x_r).  The four 4x4 matrices are
// scaled by mu/rho and applied row by row; structurally zero entries are skipped
// (their products are signed zeros, which leave every non-zero sum unchanged).
// The terms of flux.d:28-64 that depend on the Prandtl number only: gamma / Pr and its
// sums with the matrix constants.  FP64: rounded once on the host (the same IEEE
// operations as here); FP32: formed per face from the FP32 Prandtl number.
template <typename T> struct ViscConst {
    T gP, c43gP, m1gP, p43mgP, omgP;  // g/Pr, -4/3 + g/Pr, -1 + g/Pr, 4/3 - g/Pr, 1 - g/Pr
};
template <typename T> __device__ __forceinline__ ViscConst<T> visc_const_of(T Pr)
{
    const T gP = K<T>::g / Pr;
    return {gP, T(-4.0 / 3.0) + gP, T(-1.0) + gP, T(4.0 / 3.0) - gP, T(1.0) - gP};
}

template <typename T>
__device__ __forceinline__ void diffusive_flux(const ViscConst<T> &vc, T mu, const T q[4], const T dq[4][2], T nx, T ny,
                                               T out[4])
{
    T rho = q[0];
    const Div<T> byRho(q[0]);
    T u = byRho(q[1]);
    T v = byRho(q[2]);
    T E = byRho(q[3]);
    const T gP = vc.gP;
    T s = byRho(mu);
    const T c43 = T(-4.0 / 3.0), p43 = T(4.0 / 3.0), p23 = T(2.0 / 3.0), m23 = T(-2.0 / 3.0), c231 = T(2.0 / 3.0 - 1.0);
    T tmp0 = vc.c43gP * (u * u) + vc.m1gP * (v * v) - gP * E;
    T tmp1 = vc.m1gP * (u * u) + vc.c43gP * (v * v) - gP * E;
    // A00 rows (row 0 is zero)
    T a10 = s * (c43 * u), a11 = s * p43;
    T a20 = s * (-v), a22 = s * T(1);
    T a30 = s * tmp0, a31 = s * (vc.p43mgP * u), a32 = s * (vc.omgP * v), a33 = s * gP;
    // A01
    T b10 = s * (p23 * v), b12 = s * m23;
    T b20 = s * (-u), b21 = s * T(1);
    T b30 = s * (c231 * u * v), b31 = s * v, b32 = s * (m23 * u);
    // A10
    T c10 = s * (-v), c12 = s * T(1);
    T c20 = s * (p23 * u), c22 = s * m23;
    T c30 = s * (c231 * u * v), c31 = s * (m23 * v), c32 = s * u;
    // A11
    T d10 = s * (-u), d11 = s * T(1);
    T d20 = s * (c43 * v), d22 = s * p43;
    T d30 = s * tmp1, d31 = s * (vc.omgP * u), d32 = s * (vc.p43mgP * v), d33 = s * gP;
    const T x0 = dq[0][0], x1 = dq[1][0], x2 = dq[2][0], x3 = dq[3][0];
    const T y0 = dq[0][1], y1 = dq[1][1], y2 = dq[2][1], y3 = dq[3][1];
    // matrix-vector products accumulate left to right from 0 (numd Matrix * Vector)
    T G0_1 = (zero_plus(a10 * x0) + a11 * x1) + (zero_plus(b10 * y0) + b12 * y2);
    T G0_2 = (zero_plus(a20 * x0) + a22 * x2) + (zero_plus(b20 * y0) + b21 * y1);
    T G0_3 = (zero_plus(a30 * x0) + a31 * x1 + a32 * x2 + a33 * x3) + (zero_plus(b30 * y0) + b31 * y1 + b32 * y2);
    T G1_1 = (zero_plus(c10 * x0) + c12 * x2) + (zero_plus(d10 * y0) + d11 * y1);
    T G1_2 = (zero_plus(c20 * x0) + c22 * x2) + (zero_plus(d20 * y0) + d22 * y2);
    T G1_3 = (zero_plus(c30 * x0) + c31 * x1 + c32 * x2) + (zero_plus(d30 * y0) + d31 * y1 + d32 * y2 + d33 * y3);
    out[0] = zero_dot(nx, ny);
    out[1] = G0_1 * nx + G1_1 * ny;
    out[2] = G0_2 * nx + G1_2 * ny;
    out[3] = G0_3 * nx + G1_3 * ny;
}

}  // namespace ebbdev
