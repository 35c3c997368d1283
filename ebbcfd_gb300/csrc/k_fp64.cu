// k_fp64.cu -- plain FP64 kernels of the explicit unstructured FV update (sm_103a).
//
// Compiled with -fmad=false: every multiply and add rounds separately, in the
// reference's left-to-right order, so results are bitwise those of the FP64 CPU
// path (up to the sign of exact zeros) except where CUDA's pow() is used
// (constant-pressure ghost states).
//
// Per stage three launches, all atomic-free on the state:
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
//             (integrators.d), with min/max/sum reductions in fixed-order trees.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "device_math.cuh"
#include "layout.h"

using namespace ebbdev;

namespace {

constexpr int BC_FULLSTATE = 0, BC_CONSTP = 1, BC_INVWALL = 2, BC_VISCWALL = 3, BC_SYMMETRY = 4, BC_TPINFLOW = 5,
              BC_DIRICHLET = 6;
constexpr int BC_VERTICAL = 0x100;  // flag: reflection across a vertical edge (x1 == x2)
constexpr int ERR_NAN_EDGE = 8, ERR_NAN_CELL = 9, ERR_BC = 11;

__device__ __forceinline__ bool halted(const DState *st) { return st->done || st->err_key != EBB_NOERR; }

__device__ __forceinline__ void flag_error(DState *st, unsigned phase, unsigned code, unsigned idx)
{
    unsigned long long key = ((unsigned long long)phase << 48) | ((unsigned long long)code << 40) | idx;
    atomicMin(&st->err_key, key);
}

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

__device__ __forceinline__ void reflect(int type, const double *refl, double v0, double v1, double &o0, double &o1)
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
__device__ void ghost_state(const DMesh &M, const DPhys &P, DState *st, int b, const double qi[4], double qn[4])
{
    const int type = M.b_type[b];
    const double G = 1.4;
    switch (type & 0xff) {
    case BC_DIRICHLET:
        ld4(M.b_dq + 4 * (size_t)b, qn);
        break;
    case BC_FULLSTATE:
        qn[0] = qi[0];
        qn[1] = qi[1];
        qn[2] = qi[2];
        qn[3] = qi[3];
        break;
    case BC_INVWALL:
    case BC_SYMMETRY: {
        double v0 = qi[1] / qi[0], v1 = qi[2] / qi[0], n0, n1;
        reflect(type, M.b_refl + 4 * (size_t)b, v0, v1, n0, n1);
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
        double rhop = qi[0], up = qi[1] / qi[0], vp = qi[2] / qi[0];
        double pp = pressure(qi);
        double ap = sqrt(G * (pp / rhop));
        double Jp = up + (2.0 * ap) / (G - 1);
        double Sp = pp / pow(rhop, G);
        double pb = M.b_data[4 * (size_t)b];
        double rhob = pow(pb / Sp, 1.0 / G);
        double ab = sqrt(G * (pb / rhob));
        double ub = Jp - (2.0 * ab) / (G - 1);
        double vb = vp;
        double mag = sqrt(ub * ub + vb * vb);
        double rEb = pb / (G - 1) + 0.5 * rhob * (mag * mag);
        double nx = M.b_n[2 * (size_t)b], ny = M.b_n[2 * (size_t)b + 1];
        double vpn = up * nx + vp * ny;
        double vbn = ub * nx + vb * ny;
        double g0 = up - vpn * nx + vbn * nx;
        double g1 = vp - vpn * ny + vbn * ny;
        qn[0] = rhob;
        qn[1] = rhob * g0;
        qn[2] = rhob * g1;
        qn[3] = rEb;
        break;
    }
    case BC_TPINFLOW: {
        const double *bd = M.b_data + 4 * (size_t)b;
        double Tt = bd[0], Pt = bd[1], nin0 = bd[2], nin1 = bd[3];
        double rhop = qi[0], up = qi[1] / qi[0];
        double pp = pressure(qi);
        double ap = sqrt(G * (pp / rhop));
        double Jp = up + (2.0 * ap) / (G - 1);
        double nx = M.b_n[2 * (size_t)b], ny = M.b_n[2 * (size_t)b + 1];
        double d = nin0 * nx + nin1 * ny;
        double Rg = P.r_gas;
        double aa = G * Rg * Tt * (d * d) - 0.5 * (G - 1) * (Jp * Jp);
        double bb = (4.0 * G * Rg * Tt * d) / (G - 1);
        double cc = (4.0 * G * Rg * Tt) / ((G - 1) * (G - 1)) - Jp * Jp;
        double M1 = (-bb + sqrt(bb * bb - 4 * aa * cc)) / (2.0 * aa);
        double M2 = (-bb - sqrt(bb * bb - 4 * aa * cc)) / (2.0 * aa);
        double Mb = 0;
        if (M1 >= 0 && M2 >= 0)
            Mb = fmin(M1, M2);
        else if (M1 >= 0 && M2 < 0)
            Mb = M1;
        else if (M1 < 0 && M2 >= 0)
            Mb = M2;
        else
            flag_error(st, 0, ERR_BC, (unsigned)M.b_ref[b]);
        double Tb = Tt / (1 + 0.5 * (G - 1) * (Mb * Mb));
        double pb = Pt * pow(Tb / Tt, G / (G - 1));
        double rhob = pb / (Rg * Tb);
        double ab = sqrt(G * (pb / rhob));
        double vb0 = Mb * ab * nin0, vb1 = Mb * ab * nin1;
        double mag = sqrt(vb0 * vb0 + vb1 * vb1);
        double rEb = pb / (G - 1) + 0.5 * rhob * (mag * mag);
        // solve.d:678-681 writes every value into component 0; the other
        // components of the ghost slot are never written and stay zero
        qn[0] = rEb;
        qn[1] = 0;
        qn[2] = 0;
        qn[3] = 0;
        break;
    }
    default:
        qn[0] = qi[0];
        qn[1] = qi[1];
        qn[2] = qi[2];
        qn[3] = qi[3];
    }
}

// LP!m (solve.d:37-173) on the m = 4 + 2*nNb constraints of solve.d:404-497
__device__ __noinline__ void lp_limit(const DMesh &M, int i, int ne, const double qi[4], const double mn[4],
                                      const double mx[4], const double g[4][2], double lim0[4], double lim1[4],
                                      double thresh)
{
    for (int k = 0; k < 4; k++) {
        if (!(lim0[k] < thresh) || !(ne == 3 || ne == 4)) continue;
        double A[12][2], b[12];
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
            const double *nd = M.s_nd + 2 * ((size_t)j * M.Cs + i);
            A[2 * j + 4][0] = nd[0] * g[k][0];
            A[2 * j + 4][1] = nd[1] * g[k][1];
            b[2 * j + 4] = mn[k] - qi[k];
            A[2 * j + 5][0] = -nd[0] * g[k][0];
            A[2 * j + 5][1] = -nd[1] * g[k][1];
            b[2 * j + 5] = qi[k] - mx[k];
        }
        double c0 = -fabs(g[k][0]), c1 = -fabs(g[k][1]);
        double xk0 = 0, xk1 = 0;
        int W0 = 0, W1 = 1;
        double Ak[4] = {A[0][0], A[0][1], A[1][0], A[1][1]};
        for (int it = 0;;) {
            double det = Ak[0] * Ak[3] - Ak[1] * Ak[2];
            double id = 1.0 / det;
            double l0 = (Ak[3] * id) * c0 + (-Ak[2] * id) * c1;
            double l1 = (-Ak[1] * id) * c0 + (Ak[0] * id) * c1;
            if ((l0 >= -10e-9) && (l1 >= -10e-9)) break;
            int qi_ = (l0 < l1) ? W0 : W1;
            double e0 = (l0 < l1) ? 1 : 0, e1 = (l0 < l1) ? 0 : 1;
            double pk0 = (Ak[3] * id) * e0 + (-Ak[1] * id) * e1;
            double pk1 = (-Ak[2] * id) * e0 + (Ak[0] * id) * e1;
            double alpha = INFINITY;
            int t = 0;
            double gam[12];
            int D[12], Dlen = 0;
            for (int r = 0; r < mr; r++)
                if (r != W0 && r != W1)
                    if (A[r][0] * pk0 + A[r][1] * pk1 < -1e-11) D[Dlen++] = r;
            for (int r = 0; r < Dlen; r++) {
                double aixk = A[D[r]][0] * xk0 + A[D[r]][1] * xk1;
                double aipk = A[D[r]][0] * pk0 + A[D[r]][1] * pk1;
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

template <int MJ>
__global__ void __launch_bounds__(128) k_cell(DMesh M, DPhys P, DArrays A, const double *__restrict__ qin,
                                             double *qghost, int limit)
{
    if (halted(A.st)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.C) return;
    const int Cs = M.Cs;
    double qi[4];
    ld4(qin + 4 * (size_t)i, qi);
    const int ne = M.nedge[i];
    double mn[4], mx[4], g[4][2];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        mn[k] = qi[k];
        mx[k] = qi[k];
        g[k][0] = 0.0;
        g[k][1] = 0.0;
    }
    const bool second = P.order > 1;
#pragma unroll
    for (int j = 0; j < MJ; j++) {
        if (j < ne) {
            const size_t s = (size_t)j * Cs + i;
            const int nb = M.s_nbr[s];
            double qn[4];
            if (nb < M.C) {
                ld4(qin + 4 * (size_t)nb, qn);
            } else {
                ghost_state(M, P, A.st, nb - M.C, qi, qn);
                st4(qghost + 4 * (size_t)nb, qn);
            }
            if (second) {
                const double2 gm = reinterpret_cast<const double2 *>(M.s_gm)[s];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    mn[k] = fmin(mn[k], qn[k]);
                    mx[k] = fmax(mx[k], qn[k]);
                    double du = qn[k] - qi[k];
                    g[k][0] = g[k][0] + gm.x * du;
                    g[k][1] = g[k][1] + gm.y * du;
                }
            }
        }
    }
    double lim0[4] = {1.0, 1.0, 1.0, 1.0}, lim1[4] = {1.0, 1.0, 1.0, 1.0};
    if (second && P.limited && limit) {
#pragma unroll
        for (int j = 0; j < MJ; j++) {
            if (j < ne) {
                const double2 nd = reinterpret_cast<const double2 *>(M.s_nd)[(size_t)j * Cs + i];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    double s = 1.0;
                    double qE = qi[k] + (g[k][0] * nd.x + g[k][1] * nd.y);
                    if (qE < mn[k])
                        s = (mn[k] - qi[k]) / (g[k][0] * nd.x + g[k][1] * nd.y);
                    else if (qE > mx[k])
                        s = (mx[k] - qi[k]) / (g[k][0] * nd.x + g[k][1] * nd.y);
                    lim0[k] = fmin(lim0[k], s);
                    lim1[k] = lim0[k];
                }
            }
        }
        if (P.lp) lp_limit(M, i, ne, qi, mn, mx, g, lim0, lim1, P.lp_thresh);
    }
    if (P.need_grad) {
        double *gp = A.grad + 8 * (size_t)i;
        if (second) {
            double a[4] = {g[0][0], g[0][1], g[1][0], g[1][1]}, b[4] = {g[2][0], g[2][1], g[3][0], g[3][1]};
            st4(gp, a);
            st4(gp + 4, b);
        } else {  // order 1: interior gradients are never computed (NaN-initialised in the reference)
            double nanv[4] = {NAN, NAN, NAN, NAN};
            st4(gp, nanv);
            st4(gp + 4, nanv);
        }
    }
    double lg0[4], lg1[4];
    double l0 = 1.0, l1 = 1.0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        lg0[k] = lim0[k] * g[k][0];
        lg1[k] = lim1[k] * g[k][1];
        l0 = fmin(l0, lim0[k]);
        l1 = fmin(l1, lim1[k]);
    }
#pragma unroll
    for (int j = 0; j < MJ; j++) {
        if (j < ne) {
            const size_t s = (size_t)j * Cs + i;
            double f[4];
            if (!second) {
#pragma unroll
                for (int k = 0; k < 4; k++) f[k] = qi[k];
            } else {
                const double2 fd = reinterpret_cast<const double2 *>(M.s_fd)[s];
#pragma unroll
                for (int k = 0; k < 4; k++) f[k] = qi[k] + lg0[k] * fd.x + lg1[k] * fd.y;
                if (pressure(f) < 0) {
                    const int ev = M.s_edge[s] & 0x7fffffff;
                    const double ll1 = (ev >= M.Eint) ? l0 : l1;  // updateBoundaryEdge uses lim[0] twice
#pragma unroll
                    for (int k = 0; k < 4; k++) f[k] = qi[k] + l0 * g[k][0] * fd.x + ll1 * g[k][1] * fd.y;
                }
            }
            st4(A.face + 4 * s, f);
        }
    }
}

__device__ __forceinline__ void load_grad(const double *grad, int c, double g[4][2])
{
    double a[4], b[4];
    ld4(grad + 8 * (size_t)c, a);
    ld4(grad + 8 * (size_t)c + 4, b);
    g[0][0] = a[0];
    g[0][1] = a[1];
    g[1][0] = a[2];
    g[1][1] = a[3];
    g[2][0] = b[0];
    g[2][1] = b[1];
    g[3][0] = b[2];
    g[3][1] = b[3];
}

__device__ __forceinline__ bool has_nan(const double F[4])
{
    return isnan(F[0]) || isnan(F[1]) || isnan(F[2]) || isnan(F[3]);
}

__device__ void boundary_flux(const DMesh &M, const DPhys &P, const DArrays &A, const double *qin, int b)
{
    const double G = 1.4;
    const int type = M.b_type[b];
    const size_t fs = (size_t)M.b_slot[b];
    double qL[4];
    ld4(A.face + 4 * fs, qL);
    const double nx = M.b_n[2 * (size_t)b], ny = M.b_n[2 * (size_t)b + 1];
    double F[4], sMax = 0;
    const int owner = M.b_cell[b];
    const int ghost = M.C + b;
    switch (type & 0xff) {
    case BC_DIRICHLET:
    case BC_FULLSTATE: {
        double qR[4];
        ld4(((type & 0xff) == BC_DIRICHLET ? M.b_dmid : M.b_data) + 4 * (size_t)b, qR);
        inviscid_flux(P.flux, qL, qR, nx, ny, F, sMax);
        if (P.viscous) {
            double g1[4][2], g2[4][2], dq[4][2], qa[4], Fv[4];
            load_grad(A.grad, owner, g1);
            load_grad(A.grad, ghost, g2);
            for (int k = 0; k < 4; k++) {
                qa[k] = 0.5 * (qL[k] + qR[k]);
                dq[k][0] = 0.5 * (g1[k][0] + g2[k][0]);
                dq[k][1] = 0.5 * (g1[k][1] + g2[k][1]);
            }
            diffusive_flux(P.pr, P.mu, qa, dq, nx, ny, Fv);
            for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
        }
        break;
    }
    case BC_INVWALL: {
        double inv = 1 / qL[0];
        double vp0 = inv * qL[1], vp1 = inv * qL[2];
        double vn = vp0 * nx + vp1 * ny;
        double t0 = vp0 - vn * nx, t1 = vp1 - vn * ny;
        double vel = sqrt(t0 * t0 + t1 * t1);
        double p = (G - 1) * (qL[3] - 0.5 * qL[0] * (vel * vel));
        double a = sqrt(G * (p / qL[0]));
        if (p < 0) p = 1.0e-12;
        F[0] = 0;
        F[1] = p * nx;
        F[2] = p * ny;
        F[3] = 0;
        sMax = fabs(a);
        break;
    }
    case BC_VISCWALL: {
        double vel = 0.0;
        double p = (G - 1) * (qL[3] - 0.5 * qL[0] * (vel * vel));
        double a = sqrt(G * (p / qL[0]));
        if (p < 0) p = 1.0e-12;
        double qR[4] = {qL[0], qL[1] * -1, qL[2] * -1, qL[3]};
        double qa[4], dq[4][2], Fv[4];
        for (int k = 0; k < 4; k++) qa[k] = 0.5 * (qL[k] + qR[k]);
        qa[1] = 0.0;
        qa[2] = 0.0;
        load_grad(A.grad, owner, dq);
        dq[3][0] = (qa[3] / qa[0]) * dq[0][0];
        dq[3][1] = (qa[3] / qa[0]) * dq[0][1];
        diffusive_flux(P.pr, P.mu, qa, dq, nx, ny, Fv);
        F[0] = 0 - Fv[0];
        F[1] = p * nx - Fv[1];
        F[2] = p * ny - Fv[2];
        F[3] = 0 - Fv[3];
        sMax = fabs(a);
        break;
    }
    case BC_CONSTP: {
        double qg[4];
        ld4(qin + 4 * (size_t)ghost, qg);
        double p = pressure(qg);
        double u = qg[1] / qg[0], v = qg[2] / qg[0];
        double a = sqrt(G * (p / qg[0]));
        convective_flux(p, u, v, qg[0], qg[3], nx, ny, F);
        sMax = fabs(a);
        break;
    }
    case BC_SYMMETRY: {
        double v0 = qL[1] / qL[0], v1 = qL[2] / qL[0], n0, n1;
        reflect(type, M.b_refl + 4 * (size_t)b, v0, v1, n0, n1);
        double qR[4] = {qL[0], qL[0] * n0, qL[0] * n1, qL[3]};
        inviscid_flux(P.flux, qL, qR, nx, ny, F, sMax);
        if (P.viscous) {
            double gp[4][2], qa[4], Fv[4];
            load_grad(A.grad, owner, gp);
            for (int k = 0; k < 4; k++) qa[k] = 0.5 * (qL[k] + qR[k]);
            // bGrad = gradp*nOuter + (A*gradp)*(I - 2 nOuter), solve.d:913-925
            double nO[2][2] = {{nx * nx, nx * ny}, {ny * nx, ny * ny}};
            double Am[4][4] = {{1, 0, 0, 0}, {0, 1 - nO[0][0], 0 - nO[0][1], 0}, {0, 0 - nO[1][0], 1 - nO[1][1], 0},
                               {0, 0, 0, 1}};
            double t2[2][2] = {{1 - 2 * nO[0][0], 0 - 2 * nO[0][1]}, {0 - 2 * nO[1][0], 1 - 2 * nO[1][1]}};
            double t1[4][2], bG[4][2];
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 2; c++) {
                    double acc = 0.0;
                    for (int k = 0; k < 4; k++) acc += Am[r][k] * gp[k][c];
                    t1[r][c] = acc;
                }
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 2; c++) {
                    double a3 = 0.0;
                    for (int k = 0; k < 2; k++) a3 += t1[r][k] * t2[k][c];
                    double a1 = 0.0;
                    for (int k = 0; k < 2; k++) a1 += gp[r][k] * nO[k][c];
                    bG[r][c] = a1 + a3;
                }
            diffusive_flux(P.pr, P.mu, qa, bG, nx, ny, Fv);
            for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
        }
        break;
    }
    case BC_TPINFLOW: {
        double qR[4];
        ld4(qin + 4 * (size_t)ghost, qR);
        inviscid_flux(P.flux, qL, qR, nx, ny, F, sMax);
        if (P.viscous) {
            double gp[4][2], qa[4], Fv[4];
            load_grad(A.grad, owner, gp);
            for (int k = 0; k < 4; k++) qa[k] = 0.5 * (qL[k] + qR[k]);
            diffusive_flux(P.pr, P.mu, qa, gp, nx, ny, Fv);
            for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
        }
        break;
    }
    default:
        F[0] = F[1] = F[2] = F[3] = NAN;
    }
    if (has_nan(F)) flag_error(A.st, 1, ERR_NAN_EDGE, (unsigned)M.b_ref[b]);
    const double len = M.b_len[b];
    const size_t e = (size_t)M.Eint + b;
    double lf[4] = {len * F[0], len * F[1], len * F[2], len * F[3]};
    st4(A.fl + 4 * e, lf);
    A.fs[e] = len * sMax;
}

__global__ void __launch_bounds__(128) k_flux(DMesh M, DPhys P, DArrays A, const double *__restrict__ qin, int nbi)
{
    if (halted(A.st)) return;
    if ((int)blockIdx.x >= nbi) {
        const int b = (blockIdx.x - nbi) * blockDim.x + threadIdx.x;
        if (b < M.G) boundary_flux(M, P, A, qin, b);
        return;
    }
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M.Eint) return;
    const int2 sl = reinterpret_cast<const int2 *>(M.e_slot)[e];
    double qL[4], qR[4], F[4], sMax;
    ld4(A.face + 4 * (size_t)sl.x, qL);
    ld4(A.face + 4 * (size_t)sl.y, qR);
    const double2 n = reinterpret_cast<const double2 *>(M.e_n)[e];
    inviscid_flux(P.flux, qL, qR, n.x, n.y, F, sMax);
    if (P.viscous) {
        const int2 c = reinterpret_cast<const int2 *>(M.e_cell)[e];
        double g1[4][2], g2[4][2], dq[4][2], qa[4], Fv[4];
        load_grad(A.grad, c.x, g1);
        load_grad(A.grad, c.y, g2);
        for (int k = 0; k < 4; k++) {
            qa[k] = 0.5 * (qL[k] + qR[k]);
            dq[k][0] = 0.5 * (g1[k][0] + g2[k][0]);
            dq[k][1] = 0.5 * (g1[k][1] + g2[k][1]);
        }
        diffusive_flux(P.pr, P.mu, qa, dq, n.x, n.y, Fv);
        for (int k = 0; k < 4; k++) F[k] = F[k] - Fv[k];
    }
    if (has_nan(F)) flag_error(A.st, 2, ERR_NAN_EDGE, (unsigned)M.e_ref[e]);
    const double len = M.e_len[e];
    double lf[4] = {len * F[0], len * F[1], len * F[2], len * F[3]};
    st4(A.fl + 4 * (size_t)e, lf);
    A.fs[e] = len * sMax;
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

constexpr int UPD_THREADS = 256;

template <int ST>
__global__ void __launch_bounds__(UPD_THREADS) k_update(DMesh M, DPhys P, DArrays A, const double *__restrict__ qin,
                                                       double *qout, int dt_update, int need_dt, int final_stage)
{
    DState *st = A.st;
    if (halted(st)) return;
    __shared__ double sh[UPD_THREADS / 32][10];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < M.C;
    double dtc = INFINITY, rm = 0.0;
    double ss[4] = {0, 0, 0, 0}, vs[4] = {0, 0, 0, 0};
    bool bad = false;
    if (act) {
        const int Cs = M.Cs;
        const int ne = M.nedge[i];
        double r[4] = {0.0, 0.0, 0.0, 0.0};
        double sAve = 0;
        for (int j = 0; j < ne; j++) {
            const int ev = M.s_edge[(size_t)j * Cs + i];
            const size_t e = (size_t)(ev & 0x7fffffff);
            double f[4];
            ld4(A.fl + 4 * e, f);
            if (ev < 0) {
#pragma unroll
                for (int k = 0; k < 4; k++) r[k] = r[k] + (-f[k]);
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++) r[k] = r[k] + f[k];
            }
            sAve += A.fs[e];
        }
        if (need_dt || (P.local_ts && dt_update)) {
            sAve /= M.perim[i];
            double c = (st->cfl * M.dlen[i]) / sAve;
            if (need_dt) dtc = c;
            if (P.local_ts && dt_update) A.cdt[i] = isnan(c) ? 0.0 : c;
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (fabs(r[k]) > rm) rm = fabs(r[k]);
        const double s = M.neg_inv_area[i];
        double R[4];
#pragma unroll
        for (int k = 0; k < 4; k++) R[k] = r[k] * s;
        if (P.mms) {
            double S[4];
            ld4(M.src + 4 * (size_t)i, S);
#pragma unroll
            for (int k = 0; k < 4; k++) R[k] = R[k] + S[k];
        }
        if (ST == ST_RESID) {
            st4(A.R + 4 * (size_t)i, R);
        } else {
            double q0[4];
            ld4(A.q + 4 * (size_t)i, q0);
            const double dt = st->dt;
            const double h = P.local_ts ? A.cdt[i] : dt;
            double out[4];
            if (ST == ST_EULER) {
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + h * R[k];
            } else if (ST == ST_RK2_1) {
                st4(A.aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + (dt * R[k]);
            } else if (ST == ST_RK2_2) {
                double k1[4];
                ld4(A.aux + 4 * (size_t)i, k1);
                const double hh = P.local_ts ? h / 2.0 : st->dt_half;
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + hh * (k1[k] + R[k]);
            } else if (ST == ST_TVD_1) {
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + h * R[k];
            } else if (ST == ST_TVD_2) {
                double qfe[4];
                ld4(qin + 4 * (size_t)i, qfe);
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = 0.5 * (q0[k] + qfe[k] + h * R[k]);
            } else if (ST == ST_RK4_1) {
                st4(A.aux + 4 * (size_t)i, R);
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + (st->dt_half * R[k]);
            } else if (ST == ST_RK4_2 || ST == ST_RK4_3) {
                double acc[4];
                ld4(A.aux + 4 * (size_t)i, acc);
#pragma unroll
                for (int k = 0; k < 4; k++) acc[k] = acc[k] + 2.0 * R[k];
                st4(A.aux + 4 * (size_t)i, acc);
                if (ST == ST_RK4_2) {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + (st->dt_half * R[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) out[k] = q0[k] + (dt * R[k]);
                }
            } else {  // ST_RK4_4
                double acc[4];
                ld4(A.aux + 4 * (size_t)i, acc);
                const double hh = P.local_ts ? h / 6.0 : st->dt_sixth;
#pragma unroll
                for (int k = 0; k < 4; k++) out[k] = q0[k] + hh * (acc[k] + R[k]);
            }
            st4(qout + 4 * (size_t)i, out);
            if (final_stage) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    double d = out[k] - q0[k];
                    ss[k] = d * d;
                    vs[k] = out[k];
                }
                bad = isnan(out[0]) || isnan(out[1]) || isnan(out[2]) || isnan(out[3]);
            }
        }
    }
    if (bad) flag_error(st, 3, ERR_NAN_CELL, (unsigned)M.cell_ref[i]);
    // block reductions: dt (min), Rmax (max), RMS partials (sum) in a fixed tree
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    dtc = warp_min(dtc);
    rm = warp_max(rm);
    if (final_stage) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            ss[k] = warp_sum(ss[k]);
            vs[k] = warp_sum(vs[k]);
        }
    }
    if (lane == 0) {
        sh[w][0] = dtc;
        sh[w][1] = rm;
        for (int k = 0; k < 4; k++) {
            sh[w][2 + k] = ss[k];
            sh[w][6 + k] = vs[k];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = sh[0][0], b = sh[0][1];
        double s8[8];
        for (int k = 0; k < 8; k++) s8[k] = sh[0][2 + k];
        for (int ww = 1; ww < UPD_THREADS / 32; ww++) {
            a = fmin(a, sh[ww][0]);
            b = fmax(b, sh[ww][1]);
            for (int k = 0; k < 8; k++) s8[k] = s8[k] + sh[ww][2 + k];
        }
        if (need_dt && a == a) atomicMin(&st->newdt_bits, (unsigned long long)__double_as_longlong(a));
        if (b > 0) atomicMax(&st->rmax_bits, (unsigned long long)__double_as_longlong(b));
        if (final_stage)
            for (int k = 0; k < 8; k++) A.red[8 * (size_t)blockIdx.x + k] = s8[k];
    }
}

// end of one runIntegrator iteration (app/solver.d:126-249), one block
__global__ void __launch_bounds__(EBB_RED_THREADS) k_step_end(DMesh M, DArrays A, int nblk)
{
    DState *st = A.st;
    if (st->done) return;
    if (st->err_key != EBB_NOERR) {
        if (threadIdx.x == 0) st->done = 1;
        return;
    }
    __shared__ double sh[EBB_RED_THREADS][10];
    double s[10];
    for (int k = 0; k < 10; k++) s[k] = 0.0;
    for (int b = threadIdx.x; b < nblk; b += EBB_RED_THREADS)
        for (int k = 0; k < 8; k++) s[k] = s[k] + A.red[8 * (size_t)b + k];
    for (int f = threadIdx.x; f < M.n_force; f += EBB_RED_THREADS) {
        const size_t e = (size_t)M.Eint + M.force_b[f];
        s[8] = s[8] + A.fl[4 * e + 1];
        s[9] = s[9] + A.fl[4 * e + 2];
    }
    for (int k = 0; k < 10; k++) sh[threadIdx.x][k] = s[k];
    __syncthreads();
    for (int o = EBB_RED_THREADS / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int k = 0; k < 10; k++) sh[threadIdx.x][k] = sh[threadIdx.x][k] + sh[threadIdx.x + o][k];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double newdt = __longlong_as_double((long long)st->newdt_bits);
    const double rmax = __longlong_as_double((long long)st->rmax_bits);
    if (st->dynamic_dt) st->dt = newdt;
    double resid[4];
    for (int k = 0; k < 4; k++) resid[k] = sqrt((double)M.C * sh[0][k]) / sh[0][4 + k];
    const double f0 = sh[0][8], f1 = sh[0][9];
    const double drag = st->rot[0] * f0 + st->rot[1] * f1;
    const double lift = st->rot[2] * f0 + st->rot[3] * f1;
    double residMax = fmax(fmax(resid[0], resid[1]), fmax(resid[2], resid[3]));
    if (st->cfl_adjust) {
        if (st->resid_last < residMax)
            st->resid_inc++;
        else if (st->resid_inc >= 1)
            st->resid_inc--;
        if (st->resid_inc >= 2000) {
            st->cfl *= 0.99;
            st->resid_inc = 0;
        }
    }
    st->resid_last = residMax;
    if (st->rec_enabled) {
        DRecord &r = A.rec[st->n_rec % EBB_REC_CAP];
        r.t = st->t;
        r.drag = drag;
        r.lift = lift;
        for (int k = 0; k < 4; k++) r.resid[k] = resid[k];
        r.rmax = rmax;
        r.dt = st->dt;
        r.cfl = st->cfl;
        st->n_rec++;
    }
    st->t += st->dt;
    st->iter++;
    st->done = !(st->t < st->t_end);
    st->dt_half = st->dt / 2.0;
    st->dt_sixth = st->dt / 6.0;
    st->newdt_bits = 0x7FF0000000000000ull;  // +inf
    st->rmax_bits = 0ull;
}

__global__ void k_flux_batch(int kind, int64_t n, const double *qL, const double *qR, const double *nrm, double *F,
                             double *s)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a[4], b[4], f[4], sm;
    ld4(qL + 4 * i, a);
    ld4(qR + 4 * i, b);
    inviscid_flux(kind, a, b, nrm[2 * i], nrm[2 * i + 1], f, sm);
    st4(F + 4 * i, f);
    s[i] = sm;
}

inline int ret(cudaError_t e) { return e == cudaSuccess ? 0 : (int)e; }

}  // namespace

int update_blocks(int C) { return (C + UPD_THREADS - 1) / UPD_THREADS; }

int launch_cell_fp64(const DMesh &M, const DPhys &P, const DArrays &A, const double *qin, double *qghost, int limit,
                     void *stream)
{
    const int T = 128;
    dim3 grid((M.C + T - 1) / T);
    cudaStream_t s = (cudaStream_t)stream;
    if (M.maxJ <= 3)
        k_cell<3><<<grid, T, 0, s>>>(M, P, A, qin, qghost, limit);
    else if (M.maxJ == 4)
        k_cell<4><<<grid, T, 0, s>>>(M, P, A, qin, qghost, limit);
    else
        k_cell<6><<<grid, T, 0, s>>>(M, P, A, qin, qghost, limit);
    return ret(cudaGetLastError());
}

int launch_flux_fp64(const DMesh &M, const DPhys &P, const DArrays &A, const double *qin, void *stream)
{
    const int T = 128;
    int nbi = (M.Eint + T - 1) / T, nbb = (M.G + T - 1) / T;
    if (nbi + nbb == 0) return 0;
    k_flux<<<nbi + nbb, T, 0, (cudaStream_t)stream>>>(M, P, A, qin, nbi);
    return ret(cudaGetLastError());
}

int launch_update_fp64(const DMesh &M, const DPhys &P, const DArrays &A, int stage, const double *qin, double *qout,
                       int dt_update, int need_dt, int final_stage, void *stream)
{
    dim3 grid(update_blocks(M.C));
    cudaStream_t s = (cudaStream_t)stream;
#define EBB_UPD(S)                                                                                 \
    case S:                                                                                        \
        k_update<S><<<grid, UPD_THREADS, 0, s>>>(M, P, A, qin, qout, dt_update, need_dt, final_stage); \
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
    return ret(cudaGetLastError());
}

int launch_step_end(const DMesh &M, const DArrays &A, int nred_blocks, void *stream)
{
    k_step_end<<<1, EBB_RED_THREADS, 0, (cudaStream_t)stream>>>(M, A, nred_blocks);
    return ret(cudaGetLastError());
}

int launch_flux_batch(int kind, int64_t n, const double *qL, const double *qR, const double *nrm, double *F, double *s,
                      void *stream)
{
    if (n <= 0) return 0;
    const int T = 128;
    k_flux_batch<<<(unsigned)((n + T - 1) / T), T, 0, (cudaStream_t)stream>>>(kind, n, qL, qR, nrm, F, s);
    return ret(cudaGetLastError());
}

namespace {
// gather: dst[i] = src[idx[i]]; scatter: dst[idx[i]] = src[i]  (4 doubles per item)
__global__ void k_permute4(const double *__restrict__ src, double *__restrict__ dst, const int32_t *__restrict__ idx,
                           int64_t n, int gather)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    if (gather) {
        ld4(src + 4 * (size_t)idx[i], v);
        st4(dst + 4 * (size_t)i, v);
    } else {
        ld4(src + 4 * (size_t)i, v);
        st4(dst + 4 * (size_t)idx[i], v);
    }
}
}  // namespace

int launch_permute4(const double *src, double *dst, const int32_t *idx, int64_t n, int gather, void *stream)
{
    if (n <= 0) return 0;
    const int T = 256;
    k_permute4<<<(unsigned)((n + T - 1) / T), T, 0, (cudaStream_t)stream>>>(src, dst, idx, n, gather);
    return ret(cudaGetLastError());
}
