// kernels.cuh -- the explicit unstructured FV update as three kernels per stage,
// templated on the arithmetic type T:
//   T = double  plain FP64 path (k_fp64.cu, compiled without multiply-add contraction:
//               the reference's operation order, bitwise its results);
//   T = float   split path (k_split.cu): FP32 face, flux, gradient and limiter
//               arithmetic on FP32 copies of the FP64 geometry; the solution, the
//               u += dt R updates and the norm/force reductions stay FP64.
//   T = df      double-float path (k_df.cu): the same arithmetic on pairs of FP32
//               numbers (dfloat.h, ~46 bits) on double-float copies of the geometry,
//               stage states in double-float; the solution's update in the last
//               stage and the norm/force reductions stay FP64.
//
//   k_cell    one thread per interior cell: ghost states of its boundary faces
//             (solve.d:521-689), least-squares gradient and neighbour min/max
//             (solve.d:329-358), scalar and LP limiters (solve.d:360-497), and the
//             reconstructed state of each of its faces with the negative-pressure
//             fallback (solve.d:283-319,980-1011), written to that face's slot.
//   k_flux    one thread per edge: interior Roe/Rusanov (+viscous) flux from the two
//             face slots (solve.d:970-1033), boundary fluxes per BC (solve.d:769-968);
//             stores len*F and len*sMax once per edge.
//   k_update  one thread per interior cell: gathers its edges' len*F with the
//             +-1 multipliers in the cell's own edge order (the reference's summation
//             order), CFL time step, Rmax, -1/area scaling (solve.d:1080-1121), the
//             manufactured source, and the integrator stage combination
//             (integrators.d), with min/max/sum reductions in fixed-order trees;
//             split path: the freestream correction (uniform flow stays uniform).
// Accumulation is atomic-free (gather, not scatter); the only atomics are the
// order-independent min/max of dt and Rmax and the first-error key.  All three and
// the step epilogue use programmatic dependent launch (grid_dep_wait below).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "bitconv.h"
#include "device_math.cuh"
#include "layout.h"

namespace ebbdev {

constexpr int BC_FULLSTATE = 0, BC_CONSTP = 1, BC_INVWALL = 2, BC_VISCWALL = 3, BC_SYMMETRY = 4, BC_TPINFLOW = 5,
              BC_DIRICHLET = 6;
constexpr int BC_VERTICAL = 0x100;  // flag: reflection across a vertical edge (x1 == x2)
constexpr int ERR_NAN_EDGE = 8, ERR_NAN_CELL = 9, ERR_BC = 11;
// Threads per block and minimum resident blocks per SM requested through
// __launch_bounds__ (a register cap per thread: more warps in flight, possibly some
// spilling).  The FP32 (split) kernels are memory-latency bound and gain from it; the
// FP64 kernels are FP64-pipe bound.  Values picked by ebbcfd_gb300/autotune.py
// (per-kernel event timing on GB300; 1 = the compiler's own register choice).
#include "tuned.h"
constexpr int UPD_THREADS = EBB_UPD_TB;
static_assert(EBB_UPD_TB == 256 || EBB_UPD_TB == 512, "k_update's block reductions take 256 or 512 threads");
// Launch shapes per arithmetic type and profile: _F split (float) on viscous meshes
// (tuned on the Navier-Stokes plate), _FI split on inviscid meshes (tuned on the Euler
// wedge: no stored gradients, fewer live values), _D plain FP64, _W double-float.  The
// profile PR (0 viscous or other forms, 1 split inviscid) is a template parameter of the
// stage kernels because the register cap is a compile-time launch bound.
#ifndef EBB_CELL_TB_FI
#define EBB_CELL_TB_FI 128
#endif
#ifndef EBB_CELL_MINB_FI
#define EBB_CELL_MINB_FI 8
#endif
#ifndef EBB_FLUX_TB_FI
#define EBB_FLUX_TB_FI 128
#endif
#ifndef EBB_FLUX_MINB_FI
#define EBB_FLUX_MINB_FI 12
#endif
#ifndef EBB_UPD_MINB_FI
#define EBB_UPD_MINB_FI 8
#endif
#ifndef EBB_CELL_TB_W
#define EBB_CELL_TB_W 128
#endif
#ifndef EBB_FLUX_TB_W
#define EBB_FLUX_TB_W 128
#endif
#ifndef EBB_CELL_MINB_W
#define EBB_CELL_MINB_W 2
#endif
#ifndef EBB_FLUX_MINB_W
#define EBB_FLUX_MINB_W 2
#endif
#ifndef EBB_UPD_MINB_W
#define EBB_UPD_MINB_W 3
#endif
template <typename T, int PR> constexpr int pick(int f, int fi, int d, int w)
{
    return std::is_same<T, float>::value ? (PR ? fi : f) : (std::is_same<T, double>::value ? d : w);
}
template <typename T, int PR> constexpr int cell_threads()
{
    return pick<T, PR>(EBB_CELL_TB_F, EBB_CELL_TB_FI, EBB_CELL_TB_D, EBB_CELL_TB_W);
}
template <typename T, int PR> constexpr int flux_threads()
{
    return pick<T, PR>(EBB_FLUX_TB_F, EBB_FLUX_TB_FI, EBB_FLUX_TB_D, EBB_FLUX_TB_W);
}
template <typename T, int PR> constexpr int cell_minb()
{
    return pick<T, PR>(EBB_CELL_MINB_F, EBB_CELL_MINB_FI, EBB_CELL_MINB_D, EBB_CELL_MINB_W);
}
template <typename T, int PR> constexpr int flux_minb()
{
    return pick<T, PR>(EBB_FLUX_MINB_F, EBB_FLUX_MINB_FI, EBB_FLUX_MINB_D, EBB_FLUX_MINB_W);
}
template <typename T, int PR> constexpr int upd_minb()
{
    return pick<T, PR>(EBB_UPD_MINB_F, EBB_UPD_MINB_FI, EBB_UPD_MINB_D, EBB_UPD_MINB_W);
}
// an SM holds at most 2048 threads: every (threads, minimum blocks) pair must fit
static_assert(EBB_CELL_TB_F * EBB_CELL_MINB_F <= 2048 && EBB_CELL_TB_D * EBB_CELL_MINB_D <= 2048 &&
                  EBB_CELL_TB_FI * EBB_CELL_MINB_FI <= 2048,
              "k_cell bounds");
static_assert(EBB_FLUX_TB_F * EBB_FLUX_MINB_F <= 2048 && EBB_FLUX_TB_D * EBB_FLUX_MINB_D <= 2048 &&
                  EBB_FLUX_TB_FI * EBB_FLUX_MINB_FI <= 2048,
              "k_flux bounds");
static_assert(EBB_UPD_TB * EBB_UPD_MINB_F <= 2048 && EBB_UPD_TB * EBB_UPD_MINB_D <= 2048 &&
                  EBB_UPD_TB * EBB_UPD_MINB_FI <= 2048,
              "k_update bounds");
static_assert(EBB_CELL_TB_W * EBB_CELL_MINB_W <= 2048 && EBB_FLUX_TB_W * EBB_FLUX_MINB_W <= 2048 &&
                  EBB_UPD_TB * EBB_UPD_MINB_W <= 2048,
              "double-float bounds");


// Viscosity, Prandtl and CFL numbers in the arithmetic type: the split kernels read
// FP32 copies rounded once on the host or in the step epilogue (a per-thread FP64
// conversion occupies the FP64 pipe as long as an FP64 add)
template <typename T> __device__ __forceinline__ T visc_mu(const DMesh &M, const DPhys &P, int inst);
template <> __device__ __forceinline__ double visc_mu<double>(const DMesh &M, const DPhys &P, int inst)
{
    return M.inst_mu ? M.inst_mu[inst] : P.mu;
}
template <> __device__ __forceinline__ float visc_mu<float>(const DMesh &M, const DPhys &P, int inst)
{
    return M.inst_muf ? M.inst_muf[inst] : P.muf;
}
template <> __device__ __forceinline__ df visc_mu<df>(const DMesh &M, const DPhys &P, int inst)
{
    return M.inst_mu ? df(M.inst_mu[inst]) : P.muw;
}
template <typename T> __device__ __forceinline__ ViscConst<T> visc_const(const DPhys &P);
template <> __device__ __forceinline__ ViscConst<double> visc_const<double>(const DPhys &P)
{
    return {P.gP, P.c43gP, P.m1gP, P.p43mgP, P.omgP};
}
template <> __device__ __forceinline__ ViscConst<float> visc_const<float>(const DPhys &P)
{
    return visc_const_of<float>(P.prf);
}
template <> __device__ __forceinline__ ViscConst<df> visc_const<df>(const DPhys &P)
{
    return {P.gPw, P.c43gPw, P.m1gPw, P.p43mgPw, P.omgPw};
}
template <typename T> __device__ __forceinline__ T cfl_of(const DState *st)
{
    if constexpr (is_fp32<T>)
        return st->cflf;
    else
        return T(st->cfl);
}

__device__ __forceinline__ bool halted(const DState *st) { return st->done || st->err_key != EBB_NOERR; }

__device__ __forceinline__ void flag_error(DState *st, unsigned phase, unsigned code, unsigned idx)
{
    unsigned long long key = ((unsigned long long)phase << 48) | ((unsigned long long)code << 40) | idx;
    atomicMin(&st->err_key, key);
}

// Programmatic dependent launch.  The stage kernels and the step epilogue are
// launched with programmatic stream serialisation: a kernel's blocks may start while
// the previous kernel's last blocks still run, load the read-only mesh arrays (slot
// indices, geometry), and then wait at grid_dep_wait() until the previous kernel has
// completed and its writes are visible.  Every thread passes the wait before its
// first access to data another kernel writes and before it exits, so completion of a
// kernel implies completion of all kernels before it.  grid_dep_release() lets the
// next kernel start launching once every block of this one has issued it; it orders
// nothing.  In a launch without the attribute the wait returns at once.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KP, typename... AP>
inline cudaError_t launch_dep(void (*kernel)(KP...), dim3 grid, dim3 block, cudaStream_t s, AP... args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t c = {};
    c.gridDim = grid;
    c.blockDim = block;
    c.dynamicSmemBytes = 0;
    c.stream = s;
    c.attrs = at;
    c.numAttrs = 1;
    return cudaLaunchKernelEx(&c, kernel, args...);
}

// FP32 <-> FP64 conversions on the integer pipe (bitconv.h), for the split path
__device__ __forceinline__ double f2d_int(float x)
{
    const uint64_t b = ebbbits::f2d_bits(__float_as_uint(x));
    return __hiloint2double((int)(uint32_t)(b >> 32), (int)(uint32_t)b);
}
__device__ __forceinline__ float d2f_int(double x)
{
    return __uint_as_float(ebbbits::d2f_bits((uint32_t)__double2hiint(x), (uint32_t)__double2loint(x)));
}

// The FP64 value of a stage-kernel value and back.  Double-float: the word conversions
// on the integer pipe (exact), so each direction costs one FP64 add or subtract instead
// of two or three FP64-pipe conversions and an add; below FP32's normal range the
// words flush to zero, and an infinite or NaN value keeps a zero low word.
template <typename T> __device__ __forceinline__ double to_f64(T x) { return (double)x; }
template <> __device__ __forceinline__ double to_f64<df>(df x) { return f2d_int(x.hi) + f2d_int(x.lo); }
template <typename T> __device__ __forceinline__ T from_f64(double x) { return (T)x; }
template <> __device__ __forceinline__ df from_f64<df>(double x)
{
    const float h = d2f_int(x);
    const float l = d2f_int(x - f2d_int(h));
    return df(h, isfinite(h) ? l : 0.0f);
}

// 4-vector loads/stores: two 16-byte accesses for double, one for float
__device__ __forceinline__ void ld4(const double *p, double v[4])
{
    const double2 *q = reinterpret_cast<const double2 *>(p);
    double2 a = q[0], b = q[1];
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}
__device__ __forceinline__ void st4(double *p, const double v[4])
{
    double2 *q = reinterpret_cast<double2 *>(p);
    q[0] = make_double2(v[0], v[1]);
    q[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ void ld4(const float *p, float v[4])
{
    float4 a = *reinterpret_cast<const float4 *>(p);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = a.z;
    v[3] = a.w;
}
__device__ __forceinline__ void st4(float *p, const float v[4])
{
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
// double-floats: (hi, lo) pairs, two 16-byte accesses per 4-vector as for double
__device__ __forceinline__ void ld4(const df *p, df v[4])
{
    const float4 *q = reinterpret_cast<const float4 *>(p);
    const float4 a = q[0], b = q[1];
    v[0] = df(a.x, a.y);
    v[1] = df(a.z, a.w);
    v[2] = df(b.x, b.y);
    v[3] = df(b.z, b.w);
}
__device__ __forceinline__ void st4(df *p, const df v[4])
{
    float4 *q = reinterpret_cast<float4 *>(p);
    q[0] = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
    q[1] = make_float4(v[2].hi, v[2].lo, v[3].hi, v[3].lo);
}
struct __align__(16) df2 {
    df x, y;
};
template <typename T> struct V2;
template <> struct V2<df> {
    using t = df2;
};
template <> struct V2<double> {
    using t = double2;
};
template <> struct V2<float> {
    using t = float2;
};
template <typename T> __device__ __forceinline__ typename V2<T>::t ld2(const void *base, size_t i)
{
    return reinterpret_cast<const typename V2<T>::t *>(base)[i];
}
template <typename T> __device__ __forceinline__ T ld1(const void *base, size_t i)
{
    return reinterpret_cast<const T *>(base)[i];
}
template <typename T> __device__ __forceinline__ const T *ptr(const void *base) { return reinterpret_cast<const T *>(base); }

template <typename T>
__device__ __forceinline__ void reflect(int type, const T *refl, T v0, T v1, T &o0, T &o1)
{
    if (type & BC_VERTICAL) {
        o0 = -v0;
        o1 = v1;
    } else {
        o0 = refl[0] * v0 + refl[1] * v1;
        o1 = refl[2] * v0 + refl[3] * v1;
    }
}

// ghost state of boundary edge b from the owner's state qi (solve.d:521-689)
template <typename T>
__device__ void ghost_state(const DMesh &M, const DPhys &P, DState *st, int b, const T qi[4], T qn[4])
{
    const int type = M.b_type[b];
    const T G = K<T>::g;
    switch (type & 0xff) {
    case BC_DIRICHLET:
        ld4(ptr<T>(M.g.b_dq) + 4 * (size_t)b, qn);
        break;
    case BC_FULLSTATE:
        for (int k = 0; k < 4; k++) qn[k] = qi[k];
        break;
    case BC_INVWALL:
    case BC_SYMMETRY: {
        T v0 = qi[1] / qi[0], v1 = qi[2] / qi[0], n0, n1;
        reflect(type, ptr<T>(M.g.b_refl) + 4 * (size_t)b, v0, v1, n0, n1);
        qn[0] = qi[0];
        qn[1] = qi[0] * n0;
        qn[2] = qi[0] * n1;
        qn[3] = qi[3];
        break;
    }
    case BC_VISCWALL:
        qn[0] = qi[0];
        qn[1] = -qi[1];
        qn[2] = -qi[2];
        qn[3] = qi[3];
        break;
    case BC_CONSTP: {
        T rhop = qi[0], up = qi[1] / qi[0], vp = qi[2] / qi[0];
        T pp = pressure(qi);
        T ap = dsqrt(G * (pp / rhop));
        T Jp = up + (T(2.0) * ap) / (G - 1);
        T Sp = pp / dpow(rhop, G);
        T pb = ptr<T>(M.g.b_data)[4 * (size_t)b];
        T rhob = dpow(pb / Sp, T(1.0 / 1.4));
        T ab = dsqrt(G * (pb / rhob));
        T ub = Jp - (T(2.0) * ab) / (G - 1);
        T vb = vp;
        T mag = dsqrt(ub * ub + vb * vb);
        T rEb = pb / (G - 1) + T(0.5) * rhob * (mag * mag);
        const typename V2<T>::t n = ld2<T>(M.g.b_n, b);
        T vpn = up * n.x + vp * n.y;
        T vbn = ub * n.x + vb * n.y;
        T g0 = up - vpn * n.x + vbn * n.x;
        T g1 = vp - vpn * n.y + vbn * n.y;
        qn[0] = rhob;
        qn[1] = rhob * g0;
        qn[2] = rhob * g1;
        qn[3] = rEb;
        break;
    }
    case BC_TPINFLOW: {
        const T *bd = ptr<T>(M.g.b_data) + 4 * (size_t)b;
        T Tt = bd[0], Pt = bd[1], nin0 = bd[2], nin1 = bd[3];
        T rhop = qi[0], up = qi[1] / qi[0];
        T pp = pressure(qi);
        T ap = dsqrt(G * (pp / rhop));
        T Jp = up + (T(2.0) * ap) / (G - 1);
        const typename V2<T>::t n = ld2<T>(M.g.b_n, b);
        T d = nin0 * n.x + nin1 * n.y;
        T Rg = (T)P.r_gas;
        T aa = G * Rg * Tt * (d * d) - T(0.5) * (G - 1) * (Jp * Jp);
        T bb = (T(4.0) * G * Rg * Tt * d) / (G - 1);
        T cc = (T(4.0) * G * Rg * Tt) / ((G - 1) * (G - 1)) - Jp * Jp;
        T M1 = (-bb + dsqrt(bb * bb - 4 * aa * cc)) / (T(2.0) * aa);
        T M2 = (-bb - dsqrt(bb * bb - 4 * aa * cc)) / (T(2.0) * aa);
        T Mb = 0;
        if (M1 >= 0 && M2 >= 0)
            Mb = fmin(M1, M2);
        else if (M1 >= 0 && M2 < 0)
            Mb = M1;
        else if (M1 < 0 && M2 >= 0)
            Mb = M2;
        else
            flag_error(st, 0, ERR_BC, (unsigned)M.b_ref[b]);
        T Tb = Tt / (1 + T(0.5) * (G - 1) * (Mb * Mb));
        T pb = Pt * dpow(Tb / Tt, G / (G - 1));
        T rhob = pb / (Rg * Tb);
        T ab = dsqrt(G * (pb / rhob));
        T vb0 = Mb * ab * nin0, vb1 = Mb * ab * nin1;
        T mag = dsqrt(vb0 * vb0 + vb1 * vb1);
        T rEb = pb / (G - 1) + T(0.5) * rhob * (mag * mag);
        // solve.d:678-681 writes every value into component 0; the other
        // components of the ghost slot are never written and stay zero
        qn[0] = rEb;
        qn[1] = 0;
        qn[2] = 0;
        qn[3] = 0;
        break;
    }
    default:
        for (int k = 0; k < 4; k++) qn[k] = qi[k];
    }
}

// LP!m (solve.d:37-173) on the m = 4 + 2*nNb constraints of solve.d:404-497
template <typename T>
__device__ __forceinline__ void lp_limit(const DMesh &M, int i, int ne, const T qi[4], const T mn[4], const T mx[4],
                                         const T g[4][2], T lim0[4], T lim1[4], T thresh)
{
#pragma unroll 1
    for (int k = 0; k < 4; k++) {
        if (!(lim0[k] < thresh) || !(ne == 3 || ne == 4)) continue;
        T A[12][2], b[12];
        int mr = 4 + 2 * ne;
        A[0][0] = 1;
        A[0][1] = 0;
        A[1][0] = 0;
        A[1][1] = 1;
        A[2][0] = -1;
        A[2][1] = 0;
        A[3][0] = 0;
        A[3][1] = -1;
        b[0] = 0;
        b[1] = 0;
        b[2] = -1;
        b[3] = -1;
        for (int j = 0; j < ne; j++) {
            const typename V2<T>::t nd = ld2<T>(M.g.s_nd, (size_t)j * M.Cs + i);
            A[2 * j + 4][0] = nd.x * g[k][0];
            A[2 * j + 4][1] = nd.y * g[k][1];
            b[2 * j + 4] = mn[k] - qi[k];
            A[2 * j + 5][0] = -nd.x * g[k][0];
            A[2 * j + 5][1] = -nd.y * g[k][1];
            b[2 * j + 5] = qi[k] - mx[k];
        }
        T c0 = -fabs(g[k][0]), c1 = -fabs(g[k][1]);
        T xk0 = 0, xk1 = 0;
        int W0 = 0, W1 = 1;
        T Ak[4] = {A[0][0], A[0][1], A[1][0], A[1][1]};
        for (int it = 0;;) {
            T det = Ak[0] * Ak[3] - Ak[1] * Ak[2];
            T id = T(1.0) / det;
            T l0 = (Ak[3] * id) * c0 + (-Ak[2] * id) * c1;
            T l1 = (-Ak[1] * id) * c0 + (Ak[0] * id) * c1;
            if ((l0 >= T(-10e-9)) && (l1 >= T(-10e-9))) break;
            int qi_ = (l0 < l1) ? W0 : W1;
            T e0 = (l0 < l1) ? 1 : 0, e1 = (l0 < l1) ? 0 : 1;
            T pk0 = (Ak[3] * id) * e0 + (-Ak[1] * id) * e1;
            T pk1 = (-Ak[2] * id) * e0 + (Ak[0] * id) * e1;
            T alpha = INFINITY;
            int t = 0;
            T gam[12];
            int D[12], Dlen = 0;
            for (int r = 0; r < mr; r++)
                if (r != W0 && r != W1)
                    if (A[r][0] * pk0 + A[r][1] * pk1 < T(-1e-11)) D[Dlen++] = r;
            for (int r = 0; r < Dlen; r++) {
                T aixk = A[D[r]][0] * xk0 + A[D[r]][1] * xk1;
                T aipk = A[D[r]][0] * pk0 + A[D[r]][1] * pk1;
                gam[r] = (aixk - b[D[r]]) / (-aipk);
                alpha = fmin(alpha, gam[r]);
            }
            for (int r = 0; r < Dlen; r++)
                if (gam[r] == alpha) {
                    t = D[r];
                    break;
                }
            if (qi_ == W0)
                W0 = t;
            else if (qi_ == W1)
                W1 = t;
            Ak[0] = A[W0][0];
            Ak[1] = A[W0][1];
            Ak[2] = A[W1][0];
            Ak[3] = A[W1][1];
            xk0 += alpha * pk0;
            xk1 += alpha * pk1;
            if (++it > 15) break;
        }
        lim0[k] = xk0;
        lim1[k] = xk1;
    }
}

template <typename T, int MJ, bool LP, bool UNI, int PR>
__global__ void __launch_bounds__(cell_threads<T, PR>(), cell_minb<T, PR>()) k_cell(DMesh M, DPhys P, DArrays A, const T *__restrict__ qin, int limit)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < M.C;
    const int Cs = M.Cs;
    // read-only mesh data first, before the wait for the previous kernel.  Split path:
    // the neighbour rows are loaded whatever the cell's edge count (rows past it hold
    // 0), and the limiter's and the reconstruction's geometry (neighbour and face
    // midpoint offsets) is loaded here, not behind the gathers
    int ne = 0, inst = 0;
    int nbv[MJ];
    typename V2<T>::t gmv[MJ], ndv[MJ], fdv[MJ];
    if (act) {
        ne = UNI ? MJ : M.nedge[i];  // UNI: every cell has MJ edges (all triangles, all quads)
        if (M.cell_inst) inst = M.cell_inst[i];
        if constexpr (sizeof(T) == 4) {
#pragma unroll
            for (int j = 0; j < MJ; j++) nbv[j] = M.s_nbr[(size_t)j * Cs + i];
#pragma unroll
            for (int j = 0; j < MJ; j++) {
                gmv[j] = ld2<T>(M.g.s_gm, (size_t)j * Cs + i);
                ndv[j] = ld2<T>(M.g.s_nd, (size_t)j * Cs + i);
                fdv[j] = ld2<T>(M.g.s_fd, (size_t)j * Cs + i);
            }
        }
    }
    grid_dep_release();
    grid_dep_wait();
    if (!act) return;
    DState *st = A.st + inst;
    if (halted(st)) return;
    T *qghost = const_cast<T *>(qin);  // ghost slots [C, C+G) are written by their owner only
    T qi[4];
    ld4(qin + 4 * (size_t)i, qi);
    T mn[4], mx[4], g[4][2];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        mn[k] = qi[k];
        mx[k] = qi[k];
        g[k][0] = T(0.0);
        g[k][1] = T(0.0);
    }
    const bool second = P.order > 1;
    if constexpr (sizeof(T) == 4) {
        // all neighbour-state gathers in flight before any dependent math
        T qv[MJ][4];
#pragma unroll
        for (int j = 0; j < MJ; j++) nbv[j] = (j < ne) ? nbv[j] : i;
#pragma unroll
        for (int j = 0; j < MJ; j++) ld4(qin + 4 * (size_t)(nbv[j] < M.C ? nbv[j] : i), qv[j]);
#pragma unroll
        for (int j = 0; j < MJ; j++) {
            if (j < ne) {
                if (nbv[j] >= M.C) {
                    ghost_state<T>(M, P, st, nbv[j] - M.C, qi, qv[j]);
                    st4(qghost + 4 * (size_t)nbv[j], qv[j]);
                }
                if (second) {
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        mn[k] = fmin(mn[k], qv[j][k]);
                        mx[k] = fmax(mx[k], qv[j][k]);
                        T du = qv[j][k] - qi[k];
                        g[k][0] = g[k][0] + gmv[j].x * du;
                        g[k][1] = g[k][1] + gmv[j].y * du;
                    }
                }
            }
        }
    } else if constexpr (is_df<T>) {
        // double-float: the neighbour-state gathers in flight before the arithmetic,
        // which keeps the FP64 path's order (long dependent FP32 sequences leave the
        // warps waiting on one gather at a time otherwise)
        int nb[MJ];
        T qv[MJ][4];
#pragma unroll
        for (int j = 0; j < MJ; j++) nb[j] = (j < ne) ? M.s_nbr[(size_t)j * Cs + i] : i;
#pragma unroll
        for (int j = 0; j < MJ; j++) ld4(qin + 4 * (size_t)(nb[j] < M.C ? nb[j] : i), qv[j]);
#pragma unroll
        for (int j = 0; j < MJ; j++) {
            if (j < ne) {
                if (nb[j] >= M.C) {
                    ghost_state<T>(M, P, st, nb[j] - M.C, qi, qv[j]);
                    st4(qghost + 4 * (size_t)nb[j], qv[j]);
                }
                if (second) {
                    const typename V2<T>::t gm = ld2<T>(M.g.s_gm, (size_t)j * Cs + i);
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        mn[k] = fmin(mn[k], qv[j][k]);
                        mx[k] = fmax(mx[k], qv[j][k]);
                        T du = qv[j][k] - qi[k];
                        g[k][0] = g[k][0] + gm.x * du;
                        g[k][1] = g[k][1] + gm.y * du;
                    }
                }
            }
        }
    } else {
#pragma unroll
    for (int j = 0; j < MJ; j++) {
        if (j < ne) {
            const size_t s = (size_t)j * Cs + i;
            const int nb = M.s_nbr[s];
            T qn[4];
            if (nb < M.C) {
                ld4(qin + 4 * (size_t)nb, qn);
            } else {
                ghost_state<T>(M, P, st, nb - M.C, qi, qn);
                st4(qghost + 4 * (size_t)nb, qn);
            }
            if (second) {
                const typename V2<T>::t gm = ld2<T>(M.g.s_gm, s);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    mn[k] = fmin(mn[k], qn[k]);
                    mx[k] = fmax(mx[k], qn[k]);
                    T du = qn[k] - qi[k];
                    g[k][0] = g[k][0] + gm.x * du;
                    g[k][1] = g[k][1] + gm.y * du;
                }
            }
        }
    }
    }
    T lim0[4] = {T(1.0), T(1.0), T(1.0), T(1.0)}, lim1[4] = {T(1.0), T(1.0), T(1.0), T(1.0)};
    if (second && P.limited && limit && sizeof(T) == 8) {
        // FP64: the out-of-bounds tests first, then only the needed divisions in a
        // compact loop.  Branching on each (neighbour, component) pair makes a warp run
        // a division whenever any of its lanes needs it, and an FP64 division costs
        // about ten FP64-unit instructions per warp; the compact loop runs as many as
        // the busiest lane needs.  Each component's limiter still takes the minimum in
        // neighbour order (pairs in bounds give s = 1, which leaves it unchanged).
        unsigned need = 0, above = 0;
        // FP64: each test is first taken in FP32 from the values truncated on the
        // integer pipe (trunc_sat: within 2^-23, tiny values to zero, huge ones to
        // infinity).  The FP32 qE is within 2^-20 of S = |q| + |g0 nx| + |g1 ny| of the
        // FP64 one, so a side clear of 2^-18 S + 2^-100 (and 2^-20 of each bound) is
        // the FP64 expression's; pairs closer to a bound (in uniform regions every
        // pair), and NaN or overflowing ones, take the FP64 expression.
        float qf[4], g0f[4], g1f[4], lof[4], hif[4];
        if constexpr (is_fp64<T>) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                qf[k] = trunc_sat(qi[k]);
                g0f[k] = trunc_sat(g[k][0]);
                g1f[k] = trunc_sat(g[k][1]);
                lof[k] = trunc_sat(mn[k]);
                hif[k] = trunc_sat(mx[k]);
            }
        }
#pragma unroll
        for (int j = 0; j < MJ; j++) {
            if (j < ne) {
                const typename V2<T>::t nd = ld2<T>(M.g.s_nd, (size_t)j * Cs + i);
                float nxf = 0.0f, nyf = 0.0f;
                if constexpr (is_fp64<T>) {
                    nxf = trunc_sat(nd.x);
                    nyf = trunc_sat(nd.y);
                }
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const unsigned bit = 1u << (4 * j + k);
                    int side = -1;
                    if constexpr (is_fp64<T>) {
                        const float a = __fmul_rn(g0f[k], nxf), b = __fmul_rn(g1f[k], nyf);
                        const float e = __fadd_rn(qf[k], __fadd_rn(a, b));
                        const float B = __fadd_rn(0x1p-18f * __fadd_rn(__fadd_rn(fabsf(qf[k]), fabsf(a)), fabsf(b)), 0x1p-100f);
                        const float bl = __fadd_rn(0x1p-20f * fabsf(lof[k]), 0x1p-100f);
                        const float bh = __fadd_rn(0x1p-20f * fabsf(hif[k]), 0x1p-100f);
                        if (__fsub_rn(e, B) > __fadd_rn(lof[k], bl) && __fadd_rn(e, B) < __fsub_rn(hif[k], bh))
                            side = 0;
                        else if (__fadd_rn(e, B) < __fsub_rn(lof[k], bl))
                            side = 1;
                        else if (__fsub_rn(e, B) > __fadd_rn(hif[k], bh))
                            side = 2;
                    }
                    if (side < 0) {
                        const T qE = qi[k] + (g[k][0] * nd.x + g[k][1] * nd.y);
                        side = qE < mn[k] ? 1 : (qE > mx[k] ? 2 : 0);
                    }
                    if (side) need |= bit;
                    if (side == 2) above |= bit;
                }
            }
        }
        while (need) {
            const int t = __ffs(need) - 1;
            const unsigned bit = 1u << t;
            need &= need - 1;
            const int j = t >> 2, k = t & 3;
            const typename V2<T>::t nd = ld2<T>(M.g.s_nd, (size_t)j * Cs + i);
            T g0 = g[0][0], g1 = g[0][1], q = qi[0], lo = mn[0], hi = mx[0], l = lim0[0];
#pragma unroll
            for (int kk = 1; kk < 4; kk++)
                if (k == kk) {
                    g0 = g[kk][0];
                    g1 = g[kk][1];
                    q = qi[kk];
                    lo = mn[kk];
                    hi = mx[kk];
                    l = lim0[kk];
                }
            const T s = ((above & bit) ? hi - q : lo - q) / (g0 * nd.x + g1 * nd.y);
            l = fmin(l, s);
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                if (k == kk) lim0[kk] = l;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) lim1[k] = lim0[k];
        if (LP) lp_limit<T>(M, i, ne, qi, mn, mx, g, lim0, lim1, (T)P.lp_thresh);
    } else if (second && P.limited && limit) {
#pragma unroll
        for (int j = 0; j < MJ; j++) {
            if (j < ne) {
                typename V2<T>::t nd;
                if constexpr (sizeof(T) == 4)
                    nd = ndv[j];
                else
                    nd = ld2<T>(M.g.s_nd, (size_t)j * Cs + i);
                // every pair's quotient is formed and selected (no divergent branch; the
                // FP32 division is a reciprocal and a multiply): pairs in bounds leave the
                // limiter unchanged, as s = 1 does in solve.d:360-402
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const T dd = g[k][0] * nd.x + g[k][1] * nd.y;
                    const T qE = qi[k] + dd;
                    const bool lo = qE < mn[k], hi = qE > mx[k];
                    const T s = ((lo ? mn[k] : mx[k]) - qi[k]) / dd;
                    lim0[k] = (lo || hi) ? fmin(lim0[k], s) : lim0[k];
                    lim1[k] = lim0[k];
                }
            }
        }
        if (LP) lp_limit<T>(M, i, ne, qi, mn, mx, g, lim0, lim1, (T)P.lp_thresh);
    }
    if (P.need_grad) {
        T *gp = reinterpret_cast<T *>(A.grad) + 8 * (size_t)i;
        if (second) {
            T a[4] = {g[0][0], g[0][1], g[1][0], g[1][1]}, b[4] = {g[2][0], g[2][1], g[3][0], g[3][1]};
            st4(gp, a);
            st4(gp + 4, b);
        } else {  // order 1: interior gradients are never computed (NaN-initialised in the reference)
            T nanv[4] = {T(NAN), T(NAN), T(NAN), T(NAN)};
            st4(gp, nanv);
            st4(gp + 4, nanv);
        }
    }
    if (A.lim) {  // limiter values, exported for ebb-reconstruct
        T *lp = reinterpret_cast<T *>(A.lim) + 8 * (size_t)i;
        T a[4] = {lim0[0], lim1[0], lim0[1], lim1[1]}, b[4] = {lim0[2], lim1[2], lim0[3], lim1[3]};
        st4(lp, a);
        st4(lp + 4, b);
    }
    T lg0[4], lg1[4];
    T l0 = T(1.0), l1 = T(1.0);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        lg0[k] = lim0[k] * g[k][0];
        lg1[k] = lim1[k] * g[k][1];
        l0 = fmin(l0, lim0[k]);
        l1 = fmin(l1, lim1[k]);
    }
    T *face = reinterpret_cast<T *>(A.face);
#pragma unroll
    for (int j = 0; j < MJ; j++) {
        if (j < ne) {
            const size_t s = (size_t)j * Cs + i;
            T f[4];
            if (!second) {
#pragma unroll
                for (int k = 0; k < 4; k++) f[k] = qi[k];
            } else {
                typename V2<T>::t fd;
                if constexpr (sizeof(T) == 4)
                    fd = fdv[j];
                else
                    fd = ld2<T>(M.g.s_fd, s);
#pragma unroll
                for (int k = 0; k < 4; k++) f[k] = qi[k] + lg0[k] * fd.x + lg1[k] * fd.y;
                if (pressure_negative(f)) {
                    const int ev = M.s_edge[s] & 0x7fffffff;
                    const T ll1 = (ev >= M.Eint) ? l0 : l1;  // updateBoundaryEdge uses lim[0] twice
#pragma unroll
                    for (int k = 0; k < 4; k++) f[k] = qi[k] + l0 * g[k][0] * fd.x + ll1 * g[k][1] * fd.y;
                }
            }
            st4(face + 4 * s, f);
        }
    }
}

template <typename T> __device__ __forceinline__ void load_grad(const void *grad, int c, T g[4][2])
{
    T a[4], b[4];
    const T *p = reinterpret_cast<const T *>(grad) + 8 * (size_t)c;
    ld4(p, a);
    ld4(p + 4, b);
    g[0][0] = a[0];
    g[0][1] = a[1];
    g[1][0] = a[2];
    g[1][1] = a[3];
    g[2][0] = b[0];
    g[2][1] = b[1];
    g[3][0] = b[2];
    g[3][1] = b[3];
}

template <typename T> __device__ __forceinline__ bool has_nan(const T F[4])
{
    return isnan(F[0]) || isnan(F[1]) || isnan(F[2]) || isnan(F[3]);
}

template <typename T>
__device__ void boundary_flux(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, int b)
{
    const T G = K<T>::g;
    const int type = M.b_type[b];
    const size_t fsl = (size_t)M.b_slot[b];
    T qL[4];
    ld4(reinterpret_cast<const T *>(A.face) + 4 * fsl, qL);
    const typename V2<T>::t n = ld2<T>(M.g.b_n, b);
    const T nx = n.x, ny = n.y;
    T F[4], sMax = 0;
    const int owner = M.b_cell[b];
    const int ghost = M.C + b;
    const int inst = M.cell_inst ? M.cell_inst[owner] : 0;
    DState *st = A.st + inst;
    if (halted(st)) return;
    const ViscConst<T> pr = visc_const<T>(P);
    const T mu = visc_mu<T>(M, P, inst);
    switch (type & 0xff) {
    case BC_DIRICHLET:
    case BC_FULLSTATE: {
        T qR[4];
        ld4(ptr<T>((type & 0xff) == BC_DIRICHLET ? M.g.b_dmid : M.g.b_data) + 4 * (size_t)b, qR);
        inviscid_flux(P.flux, qL, qR, nx, ny, F, sMax);
        if (P.viscous) {
            T g1[4][2], g2[4][2], dq[4][2], qa[4], Fv[4];
            load_grad<T>(A.grad, owner, g1);
            load_grad<T>(A.grad, ghost, g2);
            for (int k = 0; k < 4; k++) {
                qa[k] = half(qL[k] + qR[k]);
                dq[k][0] = half(g1[k][0] + g2[k][0]);
                dq[k][1] = half(g1[k][1] + g2[k][1]);
            }
            diffusive_flux(pr, mu, qa, dq, nx, ny, Fv);
            for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
        }
        break;
    }
    case BC_INVWALL: {
        T inv = 1 / qL[0];
        T vp0 = inv * qL[1], vp1 = inv * qL[2];
        T vn = vp0 * nx + vp1 * ny;
        T t0 = vp0 - vn * nx, t1 = vp1 - vn * ny;
        T vel = dsqrt(t0 * t0 + t1 * t1);
        T p = (G - 1) * (qL[3] - T(0.5) * qL[0] * (vel * vel));
        T a = dsqrt(G * (p / qL[0]));
        if (p < 0) p = T(1.0e-12);
        F[0] = 0;
        F[1] = p * nx;
        F[2] = p * ny;
        F[3] = 0;
        sMax = fabs(a);
        break;
    }
    case BC_VISCWALL: {
        T vel = 0.0;
        T p = (G - 1) * (qL[3] - T(0.5) * qL[0] * (vel * vel));
        T a = dsqrt(G * (p / qL[0]));
        if (p < 0) p = T(1.0e-12);
        T qR[4] = {qL[0], qL[1] * -1, qL[2] * -1, qL[3]};
        T qa[4], dq[4][2], Fv[4];
        for (int k = 0; k < 4; k++) qa[k] = half(qL[k] + qR[k]);
        qa[1] = 0.0;
        qa[2] = 0.0;
        load_grad<T>(A.grad, owner, dq);
        dq[3][0] = (qa[3] / qa[0]) * dq[0][0];
        dq[3][1] = (qa[3] / qa[0]) * dq[0][1];
        diffusive_flux(pr, mu, qa, dq, nx, ny, Fv);
        F[0] = 0 - Fv[0];
        F[1] = p * nx - Fv[1];
        F[2] = p * ny - Fv[2];
        F[3] = 0 - Fv[3];
        sMax = fabs(a);
        break;
    }
    case BC_CONSTP: {
        T qg[4];
        ld4(qin + 4 * (size_t)ghost, qg);
        T p = pressure(qg);
        T u = qg[1] / qg[0], v = qg[2] / qg[0];
        T a = dsqrt(G * (p / qg[0]));
        convective_flux(p, u, v, qg[0], qg[3], nx, ny, F);
        sMax = fabs(a);
        break;
    }
    case BC_SYMMETRY: {
        T v0 = qL[1] / qL[0], v1 = qL[2] / qL[0], n0, n1;
        reflect(type, ptr<T>(M.g.b_refl) + 4 * (size_t)b, v0, v1, n0, n1);
        T qR[4] = {qL[0], qL[0] * n0, qL[0] * n1, qL[3]};
        inviscid_flux(P.flux, qL, qR, nx, ny, F, sMax);
        if (P.viscous) {
            T gp[4][2], qa[4], Fv[4];
            load_grad<T>(A.grad, owner, gp);
            for (int k = 0; k < 4; k++) qa[k] = half(qL[k] + qR[k]);
            // bGrad = gradp*nOuter + (A*gradp)*(I - 2 nOuter), solve.d:913-925
            T nO[2][2] = {{nx * nx, nx * ny}, {ny * nx, ny * ny}};
            T Am[4][4] = {{1, 0, 0, 0}, {0, 1 - nO[0][0], 0 - nO[0][1], 0}, {0, 0 - nO[1][0], 1 - nO[1][1], 0},
                          {0, 0, 0, 1}};
            T t2[2][2] = {{1 - 2 * nO[0][0], 0 - 2 * nO[0][1]}, {0 - 2 * nO[1][0], 1 - 2 * nO[1][1]}};
            T t1[4][2], bG[4][2];
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 2; c++) {
                    T acc = 0.0;
                    for (int k = 0; k < 4; k++) acc += Am[r][k] * gp[k][c];
                    t1[r][c] = acc;
                }
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 2; c++) {
                    T a3 = 0.0;
                    for (int k = 0; k < 2; k++) a3 += t1[r][k] * t2[k][c];
                    T a1 = 0.0;
                    for (int k = 0; k < 2; k++) a1 += gp[r][k] * nO[k][c];
                    bG[r][c] = a1 + a3;
                }
            diffusive_flux(pr, mu, qa, bG, nx, ny, Fv);
            for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
        }
        break;
    }
    case BC_TPINFLOW: {
        T qR[4];
        ld4(qin + 4 * (size_t)ghost, qR);
        inviscid_flux(P.flux, qL, qR, nx, ny, F, sMax);
        if (P.viscous) {
            T gp[4][2], qa[4], Fv[4];
            load_grad<T>(A.grad, owner, gp);
            for (int k = 0; k < 4; k++) qa[k] = half(qL[k] + qR[k]);
            diffusive_flux(pr, mu, qa, gp, nx, ny, Fv);
            for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
        }
        break;
    }
    default:
        F[0] = F[1] = F[2] = F[3] = T(NAN);
    }
    if (has_nan(F)) flag_error(st, 1, ERR_NAN_EDGE, (unsigned)M.b_ref[b]);
    const T len = ld1<T>(M.g.b_len, b);
    const size_t e = (size_t)M.Eint + b;
    T lf[4] = {len * F[0], len * F[1], len * F[2], len * F[3]};
    st4(reinterpret_cast<T *>(A.fl) + 4 * e, lf);
    reinterpret_cast<T *>(A.fs)[e] = len * sMax;
}

template <typename T, int PR>
__global__ void __launch_bounds__(flux_threads<T, PR>(), flux_minb<T, PR>()) k_flux(DMesh M, DPhys P, DArrays A, const T *__restrict__ qin, int nbi)
{
    if ((int)blockIdx.x >= nbi) {
        grid_dep_release();
        grid_dep_wait();
        const int b = (blockIdx.x - nbi) * blockDim.x + threadIdx.x;
        if (b < M.G) boundary_flux<T>(M, P, A, qin, b);
        return;
    }
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = e < M.Eint;
    // read-only mesh data before the wait for the previous kernel
    int inst = 0;
    int2 sl = make_int2(0, 0);
    typename V2<T>::t n = {};
    T len = T(0.0);
    if (act) {
        if (M.cell_inst) inst = M.cell_inst[reinterpret_cast<const int2 *>(M.e_cell)[e].x];
        sl = reinterpret_cast<const int2 *>(M.e_slot)[e];
        n = ld2<T>(M.g.e_n, e);
        len = ld1<T>(M.g.e_len, e);
    }
    grid_dep_release();
    grid_dep_wait();
    if (!act) return;
    DState *st = A.st + inst;
    if (halted(st)) return;
    const T *face = reinterpret_cast<const T *>(A.face);
    T qL[4], qR[4], F[4], sMax;
    ld4(face + 4 * (size_t)sl.x, qL);
    ld4(face + 4 * (size_t)sl.y, qR);
    inviscid_flux(P.flux, qL, qR, n.x, n.y, F, sMax);
    if (P.viscous) {
        const int2 c = reinterpret_cast<const int2 *>(M.e_cell)[e];
        T g1[4][2], g2[4][2], dq[4][2], qa[4], Fv[4];
        load_grad<T>(A.grad, c.x, g1);
        load_grad<T>(A.grad, c.y, g2);
        for (int k = 0; k < 4; k++) {
            qa[k] = half(qL[k] + qR[k]);
            dq[k][0] = half(g1[k][0] + g2[k][0]);
            dq[k][1] = half(g1[k][1] + g2[k][1]);
        }
        diffusive_flux(visc_const<T>(P), visc_mu<T>(M, P, inst), qa, dq, n.x, n.y, Fv);
        for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
    }
    if (has_nan(F)) flag_error(st, 2, ERR_NAN_EDGE, (unsigned)M.e_ref[e]);
    T lf[4] = {len * F[0], len * F[1], len * F[2], len * F[3]};
    st4(reinterpret_cast<T *>(A.fl) + 4 * (size_t)e, lf);
    reinterpret_cast<T *>(A.fs)[e] = len * sMax;
}

// ---- fixed-order block reductions -------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = v + __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_sumf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = v + __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_minf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_maxf(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Residual of one interior cell and the stage combination.  The solution's update runs
// in FP64 for every precision form.  FP64 path: qin/qout are double stage states as in
// integrators.d.  Split path: qin is the FP32 stage input, q64 is updated in FP64 and
// the next stage input (qout) is its FP32 rounding.  Double-float path: stages before
// the last form their stage state in double-float from the solution's double-float
// copy; the last updates q64 in FP64 and refreshes that copy.
template <typename T, int ST, int MJ, bool UNI, int PR>
__global__ void __launch_bounds__(UPD_THREADS, upd_minb<T, PR>()) k_update(DMesh M, DPhys P, DArrays A, const T *__restrict__ qin, T *qout,
                                                       int dt_update, int need_dt, int final_stage)
{
    constexpr bool SPLIT = sizeof(T) == 4;
    int i, iend, inst = 0;
    if (M.blk_first) {  // batched arena: each block lies inside one instance's cell range
        i = M.blk_first[blockIdx.x] + threadIdx.x;
        iend = M.blk_end[blockIdx.x];
        inst = M.blk_inst[blockIdx.x];
    } else {
        i = blockIdx.x * blockDim.x + threadIdx.x;
        iend = M.C;
    }
    const bool act = i < iend;
    const int Cs = M.Cs;
    // read-only mesh data before the wait for the previous kernel: every edge row is
    // loaded whatever the cell's edge count (rows past it hold 0)
    int ev[MJ], ne = 0;
    typename V2<T>::t sn[MJ];  // split path: the slots' edge normals and lengths
    T sl[MJ];
    if (act) {
#pragma unroll
        for (int j = 0; j < MJ; j++) ev[j] = M.s_edge[(size_t)j * Cs + i];
        ne = UNI ? MJ : M.nedge[i];
        if constexpr (SPLIT) {
#pragma unroll
            for (int j = 0; j < MJ; j++) {
                sn[j] = ld2<T>(M.g.s_en, (size_t)j * Cs + i);
                sl[j] = ld1<T>(M.g.s_elen, (size_t)j * Cs + i);
            }
        }
    }
    grid_dep_release();
    grid_dep_wait();
    DState *st = A.st + inst;
    if (halted(st)) return;
    double dtc = INFINITY, rm = 0.0;
    double ss[4] = {0, 0, 0, 0}, vs[4] = {0, 0, 0, 0};
    float fss[4] = {0, 0, 0, 0}, fvs[4] = {0, 0, 0, 0};  // split path: FP32 lane values
    float fdtc = INFINITY, frm = 0.0f;
    bool bad = false;
    if (act) {
        // all flux gathers are issued before the sums, which add in edge order
        const T *fl = reinterpret_cast<const T *>(A.fl);
        const T *fs = reinterpret_cast<const T *>(A.fs);
        T f[MJ][4], fe[MJ];
#pragma unroll
        for (int j = 0; j < MJ; j++) {
            if (j < ne) {
                const size_t e = (size_t)(ev[j] & 0x7fffffff);
                ld4(fl + 4 * e, f[j]);
                fe[j] = fs[e];
            }
        }
        T r[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
        T sAve = 0;
#pragma unroll
        for (int j = 0; j < MJ; j++) {
            if (j < ne) {
                if (ev[j] < 0) {
#pragma unroll
                    for (int k = 0; k < 4; k++) r[k] = r[k] + (-f[j][k]);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) r[k] = r[k] + f[j][k];
                }
                sAve += fe[j];
            }
        }
        if constexpr (SPLIT) {
            // Freestream preservation.  Subtract the same edge sum of the cell's own
            // physical flux, sum_j m_j len_j F(q_i).n_j = F(q_i) . sum_j m_j len_j n_j,
            // which is zero but for the rounding of the FP32 edge terms.  Where the
            // cell and its neighbours hold one state (face states equal to it, the flux
            // of two equal states equal to the physical flux, computed without
            // contraction in both kernels) both sums are the same bits and the residual
            // is exactly zero, as in FP64; otherwise the correction is of the size of
            // the FP32 rounding.  Without it a uniform region takes FP32-rounding-size
            // increments every step, which seed the locally unstable modes the scheme
            // has on some meshes (a plain FP64 run with 1e-7 noise added each step
            // fails at the same edge as the split run).  It runs on every cell: limited
            // to cells whose neighbours hold bitwise their state, 13 of 512 batch
            // instances failed instead of 6 (nearly uniform cells then take the full
            // edge-term rounding); limited to neighbours within 1e-3, the failures and
            // the accuracy were those of the ungated form, at a higher cost.
            T qc[4];
            ld4(qin + 4 * (size_t)i, qc);
            const T uc = qc[1] / qc[0], vc = qc[2] / qc[0];
            const T pc = pressure_of(qc[0], uc, vc, qc[3]);
            T c[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
#pragma unroll
            for (int j = 0; j < MJ; j++) {
                if (j < ne) {
                    const T len = sl[j];
                    T F[4];
                    convective_flux(pc, uc, vc, qc[0], qc[3], sn[j].x, sn[j].y, F);
                    // len F rounded on its own, as k_flux stores it (no contraction)
                    if (ev[j] < 0) {
#pragma unroll
                        for (int k = 0; k < 4; k++) c[k] = __fadd_rn(c[k], -__fmul_rn(len, F[k]));
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; k++) c[k] = __fadd_rn(c[k], __fmul_rn(len, F[k]));
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] = r[k] - c[k];
        }
        T *cdt = reinterpret_cast<T *>(A.cdt);
        if (need_dt || (P.local_ts && dt_update)) {
            sAve /= ld1<T>(M.g.perim, i);
            T c = (cfl_of<T>(st) * ld1<T>(M.g.dlen, i)) / sAve;
            if (need_dt) {
                if (SPLIT)
                    fdtc = (float)c;
                else
                    dtc = to_f64(c);
            }
            if (P.local_ts && dt_update) cdt[i] = isnan(c) ? T(0.0) : c;
        }
        if (SPLIT) {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if ((float)fabs(r[k]) > frm) frm = (float)fabs(r[k]);
        } else if constexpr (is_df<T>) {  // the largest |r| found in double-float, one conversion
            T m = T(0.0f);
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (fabs(r[k]) > m) m = fabs(r[k]);
            rm = to_f64(m);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if ((double)fabs(r[k]) > rm) rm = (double)fabs(r[k]);
        }
        const T s = ld1<T>(M.g.neg_inv_area, i);
        T R[4];
#pragma unroll
        for (int k = 0; k < 4; k++) R[k] = r[k] * s;
        if (P.mms) {
            T S[4];
            ld4(ptr<T>(M.g.src) + 4 * (size_t)i, S);
#pragma unroll
            for (int k = 0; k < 4; k++) R[k] = R[k] + S[k];
        }
        if (ST == ST_RESID) {
            st4(reinterpret_cast<T *>(A.R) + 4 * (size_t)i, R);
        } else if constexpr (SPLIT) {
            // increments at the precision of R.  Intermediate stage inputs are FP32
            // (the FP32 shadow of the solution plus the increment); the final stage
            // accumulates the solution u += inc in FP64 and refreshes the shadow.
            T *aux = reinterpret_cast<T *>(A.aux);
            const float dtf = st->dtf, hf = P.local_ts ? (float)cdt[i] : dtf;
            float inc[4];
            if (ST == ST_EULER || ST == ST_TVD_1) {
                if (ST == ST_TVD_1) st4(aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) inc[k] = hf * R[k];
            } else if (ST == ST_RK2_1) {
                st4(aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) inc[k] = dtf * R[k];
            } else if (ST == ST_RK2_2) {
                T k1[4];
                ld4(aux + 4 * (size_t)i, k1);
                const float hh = P.local_ts ? hf * 0.5f : st->dt_half_f;
#pragma unroll
                for (int k = 0; k < 4; k++) inc[k] = hh * (k1[k] + R[k]);
            } else if (ST == ST_TVD_2) {  // 0.5 (q + (q + h R1) + h R2) = q + 0.5 h (R1 + R2)
                T r1[4];
                ld4(aux + 4 * (size_t)i, r1);
#pragma unroll
                for (int k = 0; k < 4; k++) inc[k] = (0.5f * hf) * (r1[k] + R[k]);
            } else if (ST == ST_RK4_1) {
                st4(aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) inc[k] = st->dt_half_f * R[k];
            } else if (ST == ST_RK4_2 || ST == ST_RK4_3) {
                T acc[4];
                ld4(aux + 4 * (size_t)i, acc);
#pragma unroll
                for (int k = 0; k < 4; k++) acc[k] = acc[k] + 2.0f * R[k];
                st4(aux + 4 * (size_t)i, acc);
                const float h2 = ST == ST_RK4_2 ? st->dt_half_f : dtf;
#pragma unroll
                for (int k = 0; k < 4; k++) inc[k] = h2 * R[k];
            } else {  // ST_RK4_4
                T acc[4];
                ld4(aux + 4 * (size_t)i, acc);
                const float hh = P.local_ts ? hf / 6.0f : st->dt_sixth_f;
#pragma unroll
                for (int k = 0; k < 4; k++) inc[k] = hh * (acc[k] + R[k]);
            }
            T o[4];
            if (final_stage) {
                // u += inc in FP64; the conversions run on the integer pipe (an FP64
                // conversion costs about as much FP64-pipe time as the add)
                double q0[4], out[4];
                ld4(A.q64 + 4 * (size_t)i, q0);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    out[k] = q0[k] + f2d_int(inc[k]);
                    o[k] = d2f_int(out[k]);
                }
                st4(A.q64 + 4 * (size_t)i, out);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    fss[k] = inc[k] * inc[k];
                    fvs[k] = o[k];
                }
                bad = isnan(o[0]) || isnan(o[1]) || isnan(o[2]) || isnan(o[3]);
            } else {
                T q32[4];
                ld4(reinterpret_cast<const T *>(A.qs1) + 4 * (size_t)i, q32);
#pragma unroll
                for (int k = 0; k < 4; k++) o[k] = q32[k] + inc[k];
            }
            st4(qout + 4 * (size_t)i, o);
        } else if (is_df<T> && !final_stage) {
            // double-float, a stage before the last: the stage state is the solution's
            // double-float copy plus the stage increment, all in double-float (it is
            // stored as one anyway); the FP64 solution is updated by the last stage
            if constexpr (is_df<T> && (ST == ST_RK2_1 || ST == ST_TVD_1 || ST == ST_RK4_1 || ST == ST_RK4_2 ||
                                       ST == ST_RK4_3)) {
                T *aux = reinterpret_cast<T *>(A.aux);
                T qs[4];
                ld4(reinterpret_cast<const T *>(A.qs1) + 4 * (size_t)i, qs);
                T h = st->dtw;
                if (ST == ST_TVD_1) {
                    if (P.local_ts) h = cdt[i];
                } else if (ST == ST_RK2_1 || ST == ST_RK4_1) {
                    st4(aux + 4 * (size_t)i, R);
                    if (ST == ST_RK4_1) h = st->dt_half_w;
                } else {
                    T acc[4];
                    ld4(aux + 4 * (size_t)i, acc);
#pragma unroll
                    for (int k = 0; k < 4; k++) acc[k] = acc[k] + T(2.0f) * R[k];
                    st4(aux + 4 * (size_t)i, acc);
                    if (ST == ST_RK4_2) h = st->dt_half_w;
                }
                T o[4];
#pragma unroll
                for (int k = 0; k < 4; k++) o[k] = qs[k] + h * R[k];
                st4(qout + 4 * (size_t)i, o);
            }
        } else {
            T *aux = reinterpret_cast<T *>(A.aux);
            double q0[4], Rd[4], out[4];
            ld4(A.q64 + 4 * (size_t)i, q0);
#pragma unroll
            for (int k = 0; k < 4; k++) Rd[k] = to_f64(R[k]);
            const double dt = st->dt;
            const double h = P.local_ts ? to_f64(cdt[i]) : dt;
            if (ST == ST_EULER) {
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + h * Rd[k];
            } else if (ST == ST_RK2_1) {
                st4(aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + (dt * Rd[k]);
            } else if (ST == ST_RK2_2) {
                T k1[4];
                ld4(aux + 4 * (size_t)i, k1);
                const double hh = P.local_ts ? h / 2.0 : st->dt_half;
                if (SPLIT) {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + hh * ((double)k1[k] + Rd[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + hh * to_f64(k1[k] + R[k]);
                }
            } else if (ST == ST_TVD_1) {
                if (SPLIT) st4(aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + h * Rd[k];
            } else if (ST == ST_TVD_2) {
                double qfe[4];
                if (SPLIT) {  // recompute qFE = q + h R1 in FP64 from the FP32 R1
                    T r1[4];
                    ld4(aux + 4 * (size_t)i, r1);
#pragma unroll
                    for (int k = 0; k < 4; k++) qfe[k] = q0[k] + h * (double)r1[k];
                } else {
                    T qf[4];
                    ld4(qin + 4 * (size_t)i, qf);
#pragma unroll
                    for (int k = 0; k < 4; k++) qfe[k] = to_f64(qf[k]);
                }
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = 0.5 * (q0[k] + qfe[k] + h * Rd[k]);
            } else if (ST == ST_RK4_1) {
                st4(aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + (st->dt_half * Rd[k]);
            } else if (ST == ST_RK4_2 || ST == ST_RK4_3) {
                T acc[4];
                ld4(aux + 4 * (size_t)i, acc);
#pragma unroll
                for (int k = 0; k < 4; k++) acc[k] = acc[k] + T(2.0) * R[k];
                st4(aux + 4 * (size_t)i, acc);
                if (ST == ST_RK4_2) {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + (st->dt_half * Rd[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + (dt * Rd[k]);
                }
            } else {  // ST_RK4_4
                T acc[4];
                ld4(aux + 4 * (size_t)i, acc);
                const double hh = P.local_ts ? h / 6.0 : st->dt_sixth;
                if (SPLIT) {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + hh * ((double)acc[k] + Rd[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + hh * to_f64(acc[k] + R[k]);
                }
            }
            if (final_stage) {
                st4(A.q64 + 4 * (size_t)i, out);
                if (!is_fp64<T>) {  // the double-float shadow of the solution
                    T o[4] = {from_f64<T>(out[0]), from_f64<T>(out[1]), from_f64<T>(out[2]), from_f64<T>(out[3])};
                    st4(qout + 4 * (size_t)i, o);
                }
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    double d = out[k] - q0[k];
                    ss[k] = d * d;
                    vs[k] = out[k];
                }
                bad = isnan(out[0]) || isnan(out[1]) || isnan(out[2]) || isnan(out[3]);
            } else {
                T o[4] = {from_f64<T>(out[0]), from_f64<T>(out[1]), from_f64<T>(out[2]), from_f64<T>(out[3])};
                st4(qout + 4 * (size_t)i, o);
            }
        }
    }
    if (bad) flag_error(st, 3, ERR_NAN_CELL, (unsigned)M.cell_ref[i]);
    // block reductions: dt (min), Rmax (max), RMS partials (sum) in a fixed tree
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (SPLIT) {
        // The whole block in FP32 (an FP64 instruction costs a warp the same with one
        // lane active as with 32), one conversion per block value; the grid-wide
        // accumulation of the block partials is FP64.  Every thread's values go to
        // shared memory and one warp reduces each column (lane l takes rows l, l+32,
        // ..., then a shuffle tree): 10 values cost a warp ~60 instructions instead of
        // ten 5-level shuffle trees.  Column 1 holds -Rmax so that columns 0 and 1 are
        // both minima.  Fixed order.
        constexpr int WF = 11;  // row stride in floats: conflict-free column reads
        __shared__ float shf[UPD_THREADS * WF];
        __shared__ float partf[10];
        const int t = threadIdx.x;
        const int ncol = final_stage ? 10 : 2;
        shf[t * WF + 0] = fdtc;
        shf[t * WF + 1] = -frm;
        if (final_stage) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                shf[t * WF + 2 + k] = fss[k];
                shf[t * WF + 6 + k] = fvs[k];
            }
        }
        __syncthreads();
        for (int c = w; c < ncol; c += UPD_THREADS / 32) {
            float a = shf[lane * WF + c];
            if (c < 2) {
#pragma unroll
                for (int r = 1; r < UPD_THREADS / 32; r++) a = fminf(a, shf[(lane + 32 * r) * WF + c]);
                a = warp_minf(a);
            } else {
#pragma unroll
                for (int r = 1; r < UPD_THREADS / 32; r++) a = a + shf[(lane + 32 * r) * WF + c];
                a = warp_sumf(a);
            }
            if (lane == 0) partf[c] = a;
        }
        __syncthreads();
        if (t == 0) {
            const float a = partf[0], b = -partf[1];
            if (need_dt && a == a) {
                const double ad = (double)a;
                atomicMin(&st->newdt_bits, (unsigned long long)__double_as_longlong(ad));
            }
            if (b > 0) {
                const double bd = (double)b;
                atomicMax(&st->rmax_bits, (unsigned long long)__double_as_longlong(bd));
            }
            if (final_stage)
                for (int k = 0; k < 8; k++) A.red[8 * (size_t)blockIdx.x + k] = (double)partf[2 + k];
        }
        return;
    } else if constexpr (!SPLIT) {
        // FP64: every thread's values go to shared memory, and whole warps reduce
        // columns, one lane per (column, group of 16 rows): an FP64 warp instruction
        // costs the same with 1 or 32 lanes active, so a shuffle tree per value (5
        // levels x 10 values per warp) would spend most of the kernel's FP64 time here.
        // Column 1 holds -Rmax so that every column of warp 0 is a min.  Fixed order.
        constexpr int W = 11;  // row stride in doubles: conflict-free strided reads
        __shared__ double shr[UPD_THREADS * W];
        __shared__ double part[10][16];
        const int t = threadIdx.x;
        const int ncol = final_stage ? 10 : 2;
        shr[t * W + 0] = dtc;
        shr[t * W + 1] = -rm;
        if (final_stage) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                shr[t * W + 2 + k] = ss[k];
                shr[t * W + 6 + k] = vs[k];
            }
        }
        __syncthreads();
        if (t < 16 * ncol) {  // group g of column c: rows g, g+16, ..., g+240
            const int c = t >> 4, g = t & 15;
            double a = shr[g * W + c];
            if (c < 2) {
                for (int r = 1; r < UPD_THREADS / 16; r++) a = fmin(a, shr[(g + 16 * r) * W + c]);
            } else {
                for (int r = 1; r < UPD_THREADS / 16; r++) a = a + shr[(g + 16 * r) * W + c];
            }
            part[c][g] = a;
        }
        __syncthreads();
        if (t < ncol) {
            double a = part[t][0];
            if (t < 2) {
                for (int g = 1; g < 16; g++) a = fmin(a, part[t][g]);
            } else {
                for (int g = 1; g < 16; g++) a = a + part[t][g];
            }
            if (t == 0) {
                if (need_dt && a == a) atomicMin(&st->newdt_bits, (unsigned long long)__double_as_longlong(a));
            } else if (t == 1) {
                const double b = -a;
                if (b > 0) atomicMax(&st->rmax_bits, (unsigned long long)__double_as_longlong(b));
            } else {
                A.red[8 * (size_t)blockIdx.x + (t - 2)] = a;
            }
        }
    }
}

inline int ret(cudaError_t e) { return e == cudaSuccess ? 0 : (int)e; }

template <typename T, int PR>
int launch_cell_pr(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, int limit, void *stream)
{
    const int TB = cell_threads<T, PR>();
    dim3 grid((M.C + TB - 1) / TB);
    if (grid.x == 0) return 0;
    cudaStream_t s = (cudaStream_t)stream;
    const bool lp = P.lp && P.limited;
    cudaError_t e;
#define EBB_CELL_U(MJ, U)                                                                 \
    if (lp)                                                                               \
        e = launch_dep(k_cell<T, MJ, true, U, PR>, grid, dim3(TB), s, M, P, A, qin, limit); \
    else                                                                                  \
        e = launch_dep(k_cell<T, MJ, false, U, PR>, grid, dim3(TB), s, M, P, A, qin, limit);
#define EBB_CELL(MJ)           \
    if (M.uniform) {           \
        EBB_CELL_U(MJ, true)   \
    } else {                   \
        EBB_CELL_U(MJ, false)  \
    }
    if (M.maxJ <= 3) {
        EBB_CELL(3)
    } else if (M.maxJ == 4) {
        EBB_CELL(4)
    } else {  // meshes of hexagons only are not specialised
        EBB_CELL_U(6, false)
    }
#undef EBB_CELL
#undef EBB_CELL_U
    return ret(e);
}

template <typename T, int PR>
int launch_flux_pr(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, void *stream)
{
    const int TB = flux_threads<T, PR>();
    int nbi = (M.Eint + TB - 1) / TB, nbb = (M.G + TB - 1) / TB;
    if (nbi + nbb == 0) return 0;
    return ret(launch_dep(k_flux<T, PR>, dim3(nbi + nbb), dim3(TB), (cudaStream_t)stream, M, P, A, qin, nbi));
}

template <typename T, int PR>
int launch_update_pr(const DMesh &M, const DPhys &P, const DArrays &A, int stage, const T *qin, T *qout,
                     int dt_update, int need_dt, int final_stage, void *stream)
{
    dim3 grid(M.n_upd_blocks);
    if (grid.x == 0) return 0;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
#define EBB_UPD_MJ(S, MJ)                                                                                         \
    e = M.uniform ? launch_dep(k_update<T, S, MJ, true, PR>, grid, dim3(UPD_THREADS), s, M, P, A, qin, qout,       \
                               dt_update, need_dt, final_stage)                                                      \
                  : launch_dep(k_update<T, S, MJ, false, PR>, grid, dim3(UPD_THREADS), s, M, P, A, qin, qout,      \
                               dt_update, need_dt, final_stage)
#define EBB_UPD(S)                                                                                                 \
    case S:                                                                                                        \
        if (M.maxJ <= 3)                                                                                           \
            EBB_UPD_MJ(S, 3);                                                                                      \
        else if (M.maxJ == 4)                                                                                      \
            EBB_UPD_MJ(S, 4);                                                                                      \
        else                                                                                                       \
            e = launch_dep(k_update<T, S, 6, false, PR>, grid, dim3(UPD_THREADS), s, M, P, A, qin, qout, dt_update,\
                           need_dt, final_stage);                                                                  \
        break;
    switch (stage) {
        EBB_UPD(ST_RESID)
        EBB_UPD(ST_EULER)
        EBB_UPD(ST_RK2_1)
        EBB_UPD(ST_RK2_2)
        EBB_UPD(ST_TVD_1)
        EBB_UPD(ST_TVD_2)
        EBB_UPD(ST_RK4_1)
        EBB_UPD(ST_RK4_2)
        EBB_UPD(ST_RK4_3)
        EBB_UPD(ST_RK4_4)
    default:
        return -1;
    }
#undef EBB_UPD
#undef EBB_UPD_MJ
    return ret(e);
}

// the launch-shape profile: split solves of inviscid meshes take their own shapes
template <typename T> int shape_profile(const DPhys &P) { return (is_fp32<T> && !P.viscous) ? 1 : 0; }

template <typename T>
int launch_cell_impl(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, int limit, void *stream)
{
    if constexpr (is_fp32<T>)
        if (shape_profile<T>(P)) return launch_cell_pr<T, 1>(M, P, A, qin, limit, stream);
    return launch_cell_pr<T, 0>(M, P, A, qin, limit, stream);
}
template <typename T> int launch_flux_impl(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, void *stream)
{
    if constexpr (is_fp32<T>)
        if (shape_profile<T>(P)) return launch_flux_pr<T, 1>(M, P, A, qin, stream);
    return launch_flux_pr<T, 0>(M, P, A, qin, stream);
}
template <typename T>
int launch_update_impl(const DMesh &M, const DPhys &P, const DArrays &A, int stage, const T *qin, T *qout,
                       int dt_update, int need_dt, int final_stage, void *stream)
{
    if constexpr (is_fp32<T>)
        if (shape_profile<T>(P))
            return launch_update_pr<T, 1>(M, P, A, stage, qin, qout, dt_update, need_dt, final_stage, stream);
    return launch_update_pr<T, 0>(M, P, A, stage, qin, qout, dt_update, need_dt, final_stage, stream);
}

// ---- ebb-reconstruct (app/reconstruct.d:239-424) --------------------------------
// Edge values 0.5 (q[0] + q[1]) of every edge, at its reference edge id.  q[1] of a
// boundary edge is what the boundary flux code of solve.d:769-968 leaves there:
// the exact state at the midpoint (Dirichlet), the freestream (fullState), the ghost
// state (inviscid wall, constant pressure, TP inflow), the face state with negated
// momentum (viscous wall) or with reflected velocity (symmetry).
template <typename T>
__global__ void k_recon_edges(DMesh M, DArrays A, const T *__restrict__ qs, double *out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M.Eint + M.G) return;
    const T *face = reinterpret_cast<const T *>(A.face);
    T q0[4], q1[4];
    int ref;
    if (e < M.Eint) {
        const int2 sl = reinterpret_cast<const int2 *>(M.e_slot)[e];
        ld4(face + 4 * (size_t)sl.x, q0);
        ld4(face + 4 * (size_t)sl.y, q1);
        ref = M.e_ref[e];
    } else {
        const int b = e - M.Eint;
        ld4(face + 4 * (size_t)M.b_slot[b], q0);
        ref = M.b_ref[b];
        const int type = M.b_type[b];
        switch (type & 0xff) {
        case BC_DIRICHLET:
            ld4(ptr<T>(M.g.b_dmid) + 4 * (size_t)b, q1);
            break;
        case BC_FULLSTATE:
            ld4(ptr<T>(M.g.b_data) + 4 * (size_t)b, q1);
            break;
        case BC_VISCWALL:
            q1[0] = q0[0];
            q1[1] = -q0[1];
            q1[2] = -q0[2];
            q1[3] = q0[3];
            break;
        case BC_SYMMETRY: {
            T v0 = q0[1] / q0[0], v1 = q0[2] / q0[0], n0, n1;
            reflect(type, ptr<T>(M.g.b_refl) + 4 * (size_t)b, v0, v1, n0, n1);
            q1[0] = q0[0];
            q1[1] = q0[0] * n0;
            q1[2] = q0[0] * n1;
            q1[3] = q0[3];
            break;
        }
        default:  // inviscid wall, constant pressure, TP inflow: the ghost state
            ld4(qs + 4 * ((size_t)M.C + b), q1);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) out[4 * (size_t)ref + k] = 0.5 * ((double)q0[k] + (double)q1[k]);
}

// Node values of the nodes the elements use.  Interior node: the average over the
// node's cells (reference element order) of q + lim0 g0 dx + lim1 g1 dy at the node
// (reconstruct.d:303-324); boundary node: the average of the edge values of the
// boundary edges its cells share with it (reconstruct.d:326-346).  A NaN value records
// the lowest node index in *err (reconstruct.d enforces no NaN).
template <typename T>
__global__ void k_recon_nodes(DMesh M, DArrays A, int n, const int32_t *__restrict__ off,
                              const int32_t *__restrict__ items, const uint8_t *__restrict__ is_b,
                              const double *__restrict__ nxy, const double *__restrict__ cxy,
                              const double *__restrict__ edge_vals, double *out, unsigned long long *err)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    const int a0 = off[v], a1 = off[v + 1];
    if (!is_b[v]) {
        const T *g = reinterpret_cast<const T *>(A.grad);
        const T *l = reinterpret_cast<const T *>(A.lim);
        for (int a = a0; a < a1; a++) {
            const int c = items[a];  // device cell
            const double dx = nxy[2 * (size_t)v] - cxy[2 * (size_t)c];
            const double dy = nxy[2 * (size_t)v + 1] - cxy[2 * (size_t)c + 1];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const double q = A.q64[4 * (size_t)c + k];
                const double g0 = (double)g[8 * (size_t)c + 2 * k], g1 = (double)g[8 * (size_t)c + 2 * k + 1];
                const double l0 = (double)l[8 * (size_t)c + 2 * k], l1 = (double)l[8 * (size_t)c + 2 * k + 1];
                s[k] += q + l0 * g0 * dx + l1 * g1 * dy;
            }
        }
    } else {
        for (int a = a0; a < a1; a++) {
            const int e = items[a];  // reference edge id
#pragma unroll
            for (int k = 0; k < 4; k++) s[k] += edge_vals[4 * (size_t)e + k];
        }
    }
    const double r = 1.0 / (double)(a1 - a0);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        s[k] *= r;
        out[4 * (size_t)v + k] = s[k];
    }
    if (isnan(s[0]) || isnan(s[1]) || isnan(s[2]) || isnan(s[3])) atomicMin(err, (unsigned long long)v);
}

template <typename T>
int launch_recon_impl(const DMesh &M, const DArrays &A, const T *qs, double *edge_out, int n_nodes,
                      const int32_t *off, const int32_t *items, const uint8_t *is_b, const double *nxy,
                      const double *cxy, double *node_out, unsigned long long *err, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    const int ne = M.Eint + M.G;
    if (ne > 0) k_recon_edges<T><<<(ne + 255) / 256, 256, 0, st>>>(M, A, qs, edge_out);
    if (n_nodes > 0)
        k_recon_nodes<T><<<(n_nodes + 255) / 256, 256, 0, st>>>(M, A, n_nodes, off, items, is_b, nxy, cxy, edge_out,
                                                                node_out, err);
    return ret(cudaGetLastError());
}

}  // namespace ebbdev

#define EBB_INSTANTIATE(T)                                                                                        \
    template <>                                                                                                   \
    int launch_cell<T>(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, int limit, void *stream)  \
    {                                                                                                             \
        return ebbdev::launch_cell_impl<T>(M, P, A, qin, limit, stream);                                          \
    }                                                                                                             \
    template <>                                                                                                   \
    int launch_flux<T>(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, void *stream)              \
    {                                                                                                             \
        return ebbdev::launch_flux_impl<T>(M, P, A, qin, stream);                                                 \
    }                                                                                                             \
    template <>                                                                                                   \
    int launch_update<T>(const DMesh &M, const DPhys &P, const DArrays &A, int stage, const T *qin, T *qout,      \
                         int dt_update, int need_dt, int final_stage, void *stream)                               \
    {                                                                                                             \
        return ebbdev::launch_update_impl<T>(M, P, A, stage, qin, qout, dt_update, need_dt, final_stage, stream); \
    }                                                                                                             \
    template <>                                                                                                   \
    int launch_recon<T>(const DMesh &M, const DArrays &A, const T *qs, double *edge_out, int n_nodes,            \
                        const int32_t *off, const int32_t *items, const uint8_t *is_b, const double *nxy,         \
                        const double *cxy, double *node_out, unsigned long long *err, void *stream)               \
    {                                                                                                             \
        return ebbdev::launch_recon_impl<T>(M, A, qs, edge_out, n_nodes, off, items, is_b, nxy, cxy, node_out,   \
                                            err, stream);                                                         \
    }
