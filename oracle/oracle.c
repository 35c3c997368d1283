/*
 * oracle.c -- CPU FP64 restatement of EbbCFD's explicit second-order unstructured
 * finite-volume update.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: it is compiled and
 * loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg,
 * and never by the product library (ebbcfd_gb300/).  It restates, operation by
 * operation and in the same evaluation order, the D reference:
 *
 *   source/mesh.d:217-381,481-642   UMesh2.buildMesh (topology, geometry, ghosts, gradMat)
 *   source/solve.d:37-173           LP (all-inequality simplex on 2 variables)
 *   source/solve.d:175-279          ufvmSetup (IC, BC binding)
 *   source/solve.d:283-319          updateBoundaryEdge (incl. its fallback quirk)
 *   source/solve.d:322-1122         ufvmSolver (ghosts, gradients, limiters, fluxes, residual)
 *   source/flux.d:19-303            convectiveFlux, diffusiveFlux, rusanovFlux, roeFlux
 *   source/integrators.d:1-270      Euler, RK4, RK2_TVD, RK2
 *   app/solver.d:38-277             runIntegrator (dt/t protocol, NaN check, RMS, forces, CFL adjust)
 *   source/manufacturedsolution.d   manufactured fields, gradient and source term
 *   app/ms.d:131-188                addSourceTerm, computeL2
 *
 * D's `x^^2.0` / `x^^2` are compiled as x*x (integral exponent), `x^^y` with a
 * non-integral y as pow(x, y).  Left-associative evaluation order is kept
 * everywhere; the file must be compiled with -ffp-contract=off so that no
 * multiply-add is fused.
 *
 * The third-party `numd` library (Vector.normalize, Matrix!(2,2).inverse) is not in
 * the reference tree; its arithmetic is restated as v/|v| and adj(M)*(1/det M).
 * Parity against the running reference is therefore unpinned at the ULP level for
 * interior edge normals and the least-squares matrices (numd ~>0.1.0).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAX_EDGES 6
#define GAMMA 1.4

enum { BC_FULLSTATE = 0, BC_CONSTP, BC_INVWALL, BC_VISCWALL, BC_SYMMETRY, BC_TPINFLOW, BC_DIRICHLET };
enum { FLUX_RUSANOV = 0, FLUX_ROE = 1 };
enum { INT_EULER = 0, INT_RK2 = 1, INT_RK2_TVD = 2, INT_RK4 = 3 };
enum { O_OK = 0, O_ERR_NAN_EDGE = 8, O_ERR_NAN_CELL = 9, O_ERR_BC = 11, O_ERR_MESH = 4 };

#define MAX_BC 32

/* Flat restatement of struct Config (source/config.d:72-94). */
typedef struct {
    double dt;
    int dynamicDt;
    double tEnd;
    int flux;
    int integrator;
    int limited;
    double lpThresh;
    int order;
    double CFL;
    double ic[4];
    int localTimestep, multistageLimiting, cflAdjust, viscosity;
    double Pr, R, mu, Re, L;
    int mms; /* 0 none, 1 reference manufactured fields, 2 sinusoidal fields */
    int nbc;
    int bcType[MAX_BC];
    int bcNData[MAX_BC];
    double bcData[MAX_BC][4];
    int nForceGroups;
    int forceGroups[MAX_BC];
} ocfg;

typedef struct {
    uint32_t nodeIdx[2];
    double len, sMax;
    double normal[2], mid[2];
    uint32_t cellIdx[2];
    double q[2][4];
    double flux[4];
    int isBoundary, bGroup, bIdx, type;
    double bData[4];
} OEdge;

typedef struct {
    uint32_t edges[MAX_EDGES];
    double fluxMultiplier[MAX_EDGES];
    uint32_t nb[MAX_EDGES];
    double gradMat[2][MAX_EDGES];
    double grad[4][2];
    double lim[4][2];
    double minQ[4], maxQ[4];
    uint32_t nNb, nEdges;
    double area, d, perim;
    double centroid[2];
    double dt;
} OCell;

typedef struct {
    int nNodes;
    double (*nodes)[2];
    int nElem;
    int *elemOff;   /* nElem+1 */
    int *elemNodes; /* 1-based node numbers, CCW */
    int nB;
    int (*bNodes)[2]; /* 0-based */
    int nGroups;
    int *bGroupStart;
    int *groupBc; /* config boundary index per group (findBcIndex) */

    int nInterior, nCells;
    OCell *cells;
    double (*q)[4];
    int nEdges, capEdges;
    OEdge *edges;
    int nInt, nBnd;
    int *interiorEdges, *boundaryEdges;
    int *groupEdgeOff, *groupEdges; /* bGroups: edge ids per boundary group */

    ocfg cfg;
    double (*R)[4], (*tmp)[4], (*k1)[4], (*k2)[4], (*k3)[4], (*k4)[4], (*qFE)[4];
    double *last[4];
    double residRhoLast;
    unsigned residIncIters;
    double t, dt;
    long iterations;
    long errIndex;
    double mmsSrcScale;
    long nFallback[2]; /* faces whose reconstruction took the negative-pressure fallback in
                          the last residual evaluation: [0] interior, [1] boundary */
} OMesh;

/* ------------------------------------------------------------------------- */
/* euler.d:91-94 */
static double getPressure(const double q[4])
{
    double a = q[1] / q[0], b = q[2] / q[0];
    return (GAMMA - 1) * (q[3] - 0.5 * q[0] * (a * a + b * b));
}

/* flux.d:19-24 */
static void convectiveFlux(double p, double u, double v, double rho, double e, const double n[2], double out[4])
{
    double f[4] = {rho * u, p + rho * (u * u), rho * u * v, u * (p + e)};
    double h[4] = {rho * v, rho * u * v, p + rho * (v * v), v * (p + e)};
    for (int c = 0; c < 4; c++) out[c] = f[c] * n[0] + h[c] * n[1];
}

static void matvec4(const double A[4][4], const double x[4], double y[4])
{
    for (int i = 0; i < 4; i++) {
        double acc = 0.0;
        for (int k = 0; k < 4; k++) acc += A[i][k] * x[k];
        y[i] = acc;
    }
}

/* flux.d:28-64 */
static void diffusiveFlux(double Pr, double mu, const double q[4], const double dq[4][2], const double n[2], double out[4])
{
    double rho = q[0];
    double u = q[1] / q[0];
    double v = q[2] / q[0];
    double E = q[3] / q[0];
    double dqdx[4] = {dq[0][0], dq[1][0], dq[2][0], dq[3][0]};
    double dqdy[4] = {dq[0][1], dq[1][1], dq[2][1], dq[3][1]};
    double gP = GAMMA / Pr;
    double s = mu / rho;
    double tmp = (-4.0 / 3.0 + gP) * (u * u) + (-1.0 + gP) * (v * v) - gP * E;
    double B00[4][4] = {{0, 0, 0, 0}, {-4.0 / 3.0 * u, 4.0 / 3.0, 0, 0}, {-v, 0, 1, 0},
                        {tmp, (4.0 / 3.0 - gP) * u, (1.0 - gP) * v, gP}};
    double B01[4][4] = {{0, 0, 0, 0}, {2.0 / 3.0 * v, 0, -2.0 / 3.0, 0}, {-u, 1, 0, 0},
                        {(2.0 / 3.0 - 1.0) * u * v, v, -2.0 / 3.0 * u, 0}};
    double B10[4][4] = {{0, 0, 0, 0}, {-v, 0, 1, 0}, {2.0 / 3.0 * u, 0, -2.0 / 3.0, 0},
                        {(2.0 / 3.0 - 1.0) * u * v, -2.0 / 3.0 * v, u, 0}};
    tmp = (-1.0 + gP) * (u * u) + (-4.0 / 3.0 + gP) * (v * v) - gP * E;
    double B11[4][4] = {{0, 0, 0, 0}, {-u, 1, 0, 0}, {-4.0 / 3.0 * v, 0, 4.0 / 3.0, 0},
                        {tmp, (1.0 - gP) * u, (4.0 / 3.0 - gP) * v, gP}};
    double A00[4][4], A01[4][4], A10[4][4], A11[4][4];
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 4; k++) {
            A00[i][k] = s * B00[i][k];
            A01[i][k] = s * B01[i][k];
            A10[i][k] = s * B10[i][k];
            A11[i][k] = s * B11[i][k];
        }
    double a[4], b[4], G0[4], G1[4];
    matvec4(A00, dqdx, a);
    matvec4(A01, dqdy, b);
    for (int c = 0; c < 4; c++) G0[c] = a[c] + b[c];
    matvec4(A10, dqdx, a);
    matvec4(A11, dqdy, b);
    for (int c = 0; c < 4; c++) G1[c] = a[c] + b[c];
    for (int c = 0; c < 4; c++) out[c] = G0[c] * n[0] + G1[c] * n[1];
}

static double dmax4(double a, double b, double c, double d)
{
    /* std.algorithm.max over finite non-negative values; NaN propagates as in a
       chain of (a > b ? a : b) comparisons */
    double m = a;
    if (b > m) m = b;
    if (c > m) m = c;
    if (d > m) m = d;
    return m;
}

static double entropyFix(double lam, double eps)
{
    if (lam < eps) lam = (eps * eps + lam * lam) / (2.0 * eps);
    return lam;
}

/* flux.d:66-141 */
void o_rusanovFlux(const double qL[4], const double qR[4], const double n[2], double out[4], double *sMax)
{
    double rhoL = qL[0];
    double uL = qL[1] / rhoL;
    double vL = qL[2] / rhoL;
    double rhoVelL[2] = {rhoL * uL, rhoL * vL};
    double pL = (GAMMA - 1) * (qL[3] - 0.5 * rhoL * (uL * uL + vL * vL));
    double hL = (qL[3] + pL) / rhoL;

    double rhoR = qR[0];
    double uR = qR[1] / rhoR;
    double vR = qR[2] / rhoR;
    double rhoVelR[2] = {rhoR * uR, rhoR * vR};
    double pR = (GAMMA - 1) * (qR[3] - 0.5 * rhoR * (uR * uR + vR * vR));
    double hR = (qR[3] + pR) / rhoR;

    double rho = sqrt(rhoL * rhoR);
    double sL = sqrt(rhoL), sR = sqrt(rhoR);
    double vel[2];
    vel[0] = (sL * uL + sR * uR) / (sL + sR);
    vel[1] = (sL * vL + sR * vR) / (sL + sR);
    double u = vel[0] * n[0] + vel[1] * n[1];
    double p = (sL * pL + sR * pR) / (sL + sR);
    double h = (sL * hL + sR * hR) / (sL + sR);
    double a = sqrt(GAMMA * (p / rho));

    double dRhoV[2] = {rhoVelR[0] - rhoVelL[0], rhoVelR[1] - rhoVelL[1]};
    double dRho = rhoR - rhoL;
    double dRhoE = qR[3] - qL[3];

    double lam1 = fabs(u + a), lam2 = fabs(u - a), lam3 = fabs(u), lam4 = fabs(u);
    double eps = 0.01 * a;
    lam1 = entropyFix(lam1, eps);
    lam2 = entropyFix(lam2, eps);
    lam3 = entropyFix(lam3, eps);
    lam4 = entropyFix(lam4, eps);
    double sm = dmax4(fabs(lam1), fabs(lam2), fabs(lam3), fabs(lam4));
    *sMax = sm;

    double s1 = 0.5 * (sm + sm);
    double s2 = 0.5 * (sm - sm);
    double qq = sqrt(vel[0] * vel[0] + vel[1] * vel[1]);
    double G1 = (GAMMA - 1) * (((qq * qq) / 2) * dRho - (vel[0] * dRhoV[0] + vel[1] * dRhoV[1]) + dRhoE);
    double G2 = -u * dRho + (dRhoV[0] * n[0] + dRhoV[1] * n[1]);
    double C1 = (G1 / (a * a)) * (s1 - sm) + G2 / a * s2;
    double C2 = (G1 / a) * s2 + (s1 - sm) * G2;

    double fL[4], fR[4];
    convectiveFlux(pL, uL, vL, rhoL, qL[3], n, fL);
    convectiveFlux(pR, uR, vR, rhoR, qR[3], n, fR);
    double D[4] = {sm * dRho + C1, sm * dRhoV[0] + C1 * vel[0] + C2 * n[0], sm * dRhoV[1] + C1 * vel[1] + C2 * n[1],
                   sm * dRhoE + C1 * h + C2 * u};
    for (int c = 0; c < 4; c++) out[c] = 0.5 * (fL[c] + fR[c]) - 0.5 * D[c];
}

/* flux.d:224-303 */
void o_roeFlux(const double qL[4], const double qR[4], const double n[2], double out[4], double *sMax)
{
    double rhoL = qL[0];
    double uL = qL[1] / rhoL;
    double vL = qL[2] / rhoL;
    double rhoVelL[2] = {rhoL * uL, rhoL * vL};
    double pL = (GAMMA - 1) * (qL[3] - 0.5 * rhoL * (uL * uL + vL * vL));
    double hL = (qL[3] + pL) / rhoL;

    double rhoR = qR[0];
    double uR = qR[1] / rhoR;
    double vR = qR[2] / rhoR;
    double rhoVelR[2] = {rhoR * uR, rhoR * vR};
    double pR = (GAMMA - 1) * (qR[3] - 0.5 * rhoR * (uR * uR + vR * vR));
    double hR = (qR[3] + pR) / rhoR;

    double di = sqrt(rhoR / rhoL);
    double d1 = 1.0 / (1.0 + di);
    double vel[2];
    vel[0] = (di * uR + uL) * d1;
    vel[1] = (di * vR + vL) * d1;
    double u = vel[0] * n[0] + vel[1] * n[1];
    double h = (di * hR + hL) * d1;
    double a = sqrt((GAMMA - 1.0) * (h - 0.5 * (vel[0] * vel[0] + vel[1] * vel[1])));

    double dRhoV[2] = {rhoVelR[0] - rhoVelL[0], rhoVelR[1] - rhoVelL[1]};
    double dRho = rhoR - rhoL;
    double dRhoE = qR[3] - qL[3];

    double lam1 = fabs(u + a), lam2 = fabs(u - a), lam3 = fabs(u), lam4 = fabs(u);
    double eps = 0.01 * a;
    lam1 = entropyFix(lam1, eps);
    lam2 = entropyFix(lam2, eps);
    lam3 = entropyFix(lam3, eps);
    lam4 = entropyFix(lam4, eps);
    *sMax = dmax4(fabs(lam1), fabs(lam2), fabs(lam3), fabs(lam4));

    double s1 = 0.5 * (lam1 + lam2);
    double s2 = 0.5 * (lam1 - lam2);
    double qq = sqrt(vel[0] * vel[0] + vel[1] * vel[1]);
    double G1 = (GAMMA - 1) * (((qq * qq) / 2.0) * dRho - (vel[0] * dRhoV[0] + vel[1] * dRhoV[1]) + dRhoE);
    double G2 = -u * dRho + (dRhoV[0] * n[0] + dRhoV[1] * n[1]);
    double C1 = (G1 / (a * a)) * (s1 - lam3) + G2 / a * s2;
    double C2 = (G1 / a) * s2 + (s1 - lam3) * G2;

    double fL[4], fR[4];
    convectiveFlux(pL, uL, vL, rhoL, qL[3], n, fL);
    convectiveFlux(pR, uR, vR, rhoR, qR[3], n, fR);
    double D[4] = {lam3 * dRho + C1, lam3 * dRhoV[0] + C1 * vel[0] + C2 * n[0],
                   lam3 * dRhoV[1] + C1 * vel[1] + C2 * n[1], lam3 * dRhoE + C1 * h + C2 * u};
    for (int c = 0; c < 4; c++) out[c] = 0.5 * (fL[c] + fR[c]) - 0.5 * D[c];
}

static void invFlux(int kind, const double qL[4], const double qR[4], const double n[2], double out[4], double *sMax)
{
    if (kind == FLUX_ROE)
        o_roeFlux(qL, qR, n, out, sMax);
    else
        o_rusanovFlux(qL, qR, n, out, sMax);
}

/* Batched flux evaluation for the known-answer tests (flux.d:143-219). */
void o_flux_batch(int kind, int count, const double *qL, const double *qR, const double *n, double *F, double *sMax)
{
    for (int i = 0; i < count; i++) invFlux(kind, qL + 4 * i, qR + 4 * i, n + 2 * i, F + 4 * i, sMax + i);
}

void o_diffusive_flux(double Pr, double mu, const double *q, const double *dq, const double *n, double *out)
{
    double g[4][2];
    for (int i = 0; i < 4; i++) {
        g[i][0] = dq[2 * i];
        g[i][1] = dq[2 * i + 1];
    }
    diffusiveFlux(Pr, mu, q, g, n, out);
}

/* ------------------------------------------------------------------------- */
/* Manufactured solutions.
 * kind 1: the reference's fields (manufacturedsolution.d:27-282).
 * kind 2: rho=1+0.1 sin(2 pi x)cos(2 pi y), u=0.5+0.05 cos(2 pi x)sin(2 pi y),
 *         v=0.3+0.05 sin(2 pi x+1), p=1/1.4+0.1 cos(2 pi y) (Euler source only). */
#define AR 0.9
#define BR 0.04
#define CR (-2.0)
#define DR 1.0
#define AU 0.1
#define BU 0.02
#define CU 1.0
#define DU 1.0
#define AV 0.05
#define BV (-0.1)
#define CV 0.7
#define DV 1.3
#define AP 1.0
#define BP 0.05
#define CP 2.0
#define DP (-1.0)

static double m_rho(double x, double y) { return AR + BR * sin(CR * x + DR * y); }
static double m_drdx(double x, double y) { return BR * CR * cos(CR * x + DR * y); }
static double m_d2rdx2(double x, double y) { return -BR * (CR * CR) * sin(CR * x + DR * y); }
static double m_drdy(double x, double y) { return BR * DR * cos(CR * x + DR * y); }
static double m_d2rdy2(double x, double y) { return -BR * (DR * DR) * sin(CR * x + DR * y); }
static double m_u(double x, double y) { return AU + BU * cos(CU * x + DU * y); }
static double m_dudx(double x, double y) { return -BU * CU * sin(CU * x + DU * y); }
static double m_d2udxy(double x, double y) { return -BU * CU * DU * cos(CU * x + DU * y); }
static double m_d2udx2(double x, double y) { return -BU * (CU * CU) * cos(CU * x + DU * y); }
static double m_dudy(double x, double y) { return -BU * DU * sin(CU * x + DU * y); }
static double m_d2udy2(double x, double y) { return -BU * (DU * DU) * cos(CU * x + DU * y); }
static double m_v(double x, double y) { return AV + BV * cos(CV * x + DV * y); }
static double m_dvdx(double x, double y) { return -BV * CV * sin(CV * x + DV * y); }
static double m_dvdy(double x, double y) { return -BV * DV * sin(CV * x + DV * y); }
static double m_d2vdx2(double x, double y) { return -BV * (CV * CV) * cos(CV * x + DV * y); }
static double m_d2vdy2(double x, double y) { return -BV * (DV * DV) * cos(CV * x + DV * y); }
static double m_d2vdxy(double x, double y) { return -BV * CV * DV * cos(CV * x + DV * y); }
static double m_p(double x, double y) { return AP + BP * sin(CP * x + DP * y); }
static double m_dpdx(double x, double y) { return BP * CP * cos(CP * x + DP * y); }
static double m_d2pdx2(double x, double y) { return -BP * (CP * CP) * sin(CP * x + DP * y); }
static double m_dpdy(double x, double y) { return BP * DP * cos(CP * x + DP * y); }
static double m_d2pdy2(double x, double y) { return -BP * (DP * DP) * sin(CP * x + DP * y); }

/* manufacturedsolution.d:244-254 */
static void ref_solution(double x, double y, double q[4])
{
    q[0] = m_rho(x, y);
    q[1] = m_rho(x, y) * m_u(x, y);
    q[2] = m_rho(x, y) * m_v(x, y);
    double uu = m_u(x, y), vv = m_v(x, y);
    q[3] = m_p(x, y) / (GAMMA - 1.0) + 0.5 * m_rho(x, y) * (uu * uu + vv * vv);
}

/* manufacturedsolution.d:256-282 */
static void ref_solutionGradient(double x, double y, double g[4][2])
{
    g[0][0] = m_drdx(x, y);
    g[0][1] = m_drdy(x, y);
    g[1][0] = m_u(x, y) * m_drdx(x, y) + m_rho(x, y) * m_dudx(x, y);
    g[1][1] = m_u(x, y) * m_drdy(x, y) + m_rho(x, y) * m_dudy(x, y);
    g[2][0] = m_v(x, y) * m_drdx(x, y) + m_rho(x, y) * m_dvdx(x, y);
    g[2][1] = m_v(x, y) * m_drdy(x, y) + m_rho(x, y) * m_dvdy(x, y);
    double uu = m_u(x, y), vv = m_v(x, y);
    double dru2dx = 2.0 * m_rho(x, y) * m_u(x, y) * m_dudx(x, y) + (uu * uu) * m_drdx(x, y);
    double dru2dy = 2.0 * m_rho(x, y) * m_u(x, y) * m_dudy(x, y) + (uu * uu) * m_drdy(x, y);
    double drv2dx = 2.0 * m_rho(x, y) * m_v(x, y) * m_dvdx(x, y) + (vv * vv) * m_drdx(x, y);
    double drv2dy = 2.0 * m_rho(x, y) * m_v(x, y) * m_dvdy(x, y) + (vv * vv) * m_drdy(x, y);
    g[3][0] = 1.0 / (GAMMA - 1.0) * m_dpdx(x, y) + 0.5 * (dru2dx + drv2dx);
    g[3][1] = 1.0 / (GAMMA - 1.0) * m_dpdy(x, y) + 0.5 * (dru2dy + drv2dy);
}

/* manufacturedsolution.d:158-242 */
static void ref_sourceTerm(double x, double y, const ocfg *cfg, double S[4])
{
    double q[4], dq[4][2];
    ref_solution(x, y, q);
    ref_solutionGradient(x, y, dq);
    double r = q[0], u = q[1] / q[0], v = q[2] / q[0], ru = q[1], rv = q[2];
    double drdx = dq[0][0], drdy = dq[0][1], drudx = dq[1][0], drvdy = dq[2][1];
    double p = getPressure(q);
    double dudx = m_dudx(x, y), dudy = m_dudy(x, y), dvdy = m_dvdy(x, y), dvdx = m_dvdx(x, y);
    double dpdx = m_dpdx(x, y), dpdy = m_dpdy(x, y);
    double dredx = dq[3][0], dredy = dq[3][1], rE = q[3];
    double Fx[4], Fy[4];
    Fx[0] = drudx;
    Fx[1] = 2.0 * ru * dudx + (u * u) * drdx + dpdx;
    Fx[2] = u * v * drdx + r * u * dvdx + r * v * dudx;
    Fx[3] = u * dredx + rE * dudx + u * dpdx + p * dudx;
    Fy[0] = drvdy;
    Fy[1] = u * v * drdy + r * u * dvdy + r * v * dudy;
    Fy[2] = 2.0 * rv * dvdy + (v * v) * drdy + dpdy;
    Fy[3] = v * dredy + rE * dvdy + v * dpdy + p * dvdy;
    for (int c = 0; c < 4; c++) S[c] = Fx[c] + Fy[c];
    if (cfg->viscosity) {
        double Gx[4] = {0, 0, 0, 0}, Gy[4] = {0, 0, 0, 0};
        double R = cfg->R, mu = cfg->mu, Pr = cfg->Pr;
        double k = (GAMMA * R * mu) / ((GAMMA - 1) * Pr);
        double d2udx2 = m_d2udx2(x, y), d2udy2 = m_d2udy2(x, y), d2udxy = m_d2udxy(x, y);
        double d2vdx2 = m_d2vdx2(x, y), d2vdy2 = m_d2vdy2(x, y), d2vdxy = m_d2vdxy(x, y);
        double d2pdx2 = m_d2pdx2(x, y), d2pdy2 = m_d2pdy2(x, y);
        double d2rdx2 = m_d2rdx2(x, y), d2rdy2 = m_d2rdy2(x, y);
        Gx[1] = mu * (2.0 / 3.0) * (2 * d2udx2 - d2vdxy);
        Gx[2] = mu * (d2udxy + d2vdx2);
        Gx[3] = mu * (2.0 / 3.0) * (2 * (u * d2udx2 + dudx * dudx) - (u * d2vdxy + dudx * dvdy));
        Gx[3] += mu * ((v * d2udxy + dvdx * dudy) + (v * d2vdx2 + dvdx * dvdx));
        double d2Tdx2 = (1.0 / R) * ((1.0 / r) * d2pdx2 + (1.0 / (r * r)) * drdx * dpdx -
                                     (1.0 / (r * r * r)) * (r * dpdx - 2.0 * p * drdx) * drdx - (p / (r * r)) * d2rdx2);
        Gx[3] += k * d2Tdx2;
        Gy[1] = mu * (d2udy2 + d2vdxy);
        Gy[2] = mu * (2.0 / 3.0) * (2 * d2vdy2 - d2udxy);
        Gy[3] = mu * (2.0 / 3.0) * (2.0 * (v * d2vdy2 + dvdy * dvdy) - (v * d2udxy + dvdy * dudx));
        Gy[3] += mu * (u * d2udy2 + dudy * dudy + u * d2vdxy + dudy * dvdx);
        double d2Tdy2 = (1.0 / R) * ((1.0 / r) * d2pdy2 + (1.0 / (r * r)) * drdy * dpdy -
                                     (1.0 / (r * r * r)) * (r * dpdy - 2.0 * p * drdy) * drdy - (p / (r * r)) * d2rdy2);
        Gy[3] += k * d2Tdy2;
        for (int c = 0; c < 4; c++) S[c] -= (Gx[c] + Gy[c]);
    }
}

#define TWO_PI 6.283185307179586
static void sin_solution(double x, double y, double q[4])
{
    double r = 1.0 + 0.1 * sin(TWO_PI * x) * cos(TWO_PI * y);
    double u = 0.5 + 0.05 * cos(TWO_PI * x) * sin(TWO_PI * y);
    double v = 0.3 + 0.05 * sin(TWO_PI * x + 1.0);
    double p = 1.0 / 1.4 + 0.1 * cos(TWO_PI * y);
    q[0] = r;
    q[1] = r * u;
    q[2] = r * v;
    q[3] = p / (GAMMA - 1.0) + 0.5 * r * (u * u + v * v);
}

static void sin_prims(double x, double y, double w[4], double wx[4], double wy[4])
{
    double sx = sin(TWO_PI * x), cx = cos(TWO_PI * x), sy = sin(TWO_PI * y), cy = cos(TWO_PI * y);
    double s1 = sin(TWO_PI * x + 1.0), c1 = cos(TWO_PI * x + 1.0);
    w[0] = 1.0 + 0.1 * sx * cy;
    w[1] = 0.5 + 0.05 * cx * sy;
    w[2] = 0.3 + 0.05 * s1;
    w[3] = 1.0 / 1.4 + 0.1 * cy;
    wx[0] = 0.1 * TWO_PI * cx * cy;
    wy[0] = -0.1 * TWO_PI * sx * sy;
    wx[1] = -0.05 * TWO_PI * sx * sy;
    wy[1] = 0.05 * TWO_PI * cx * cy;
    wx[2] = 0.05 * TWO_PI * c1;
    wy[2] = 0.0;
    wx[3] = 0.0;
    wy[3] = -0.1 * TWO_PI * sy;
}

static void sin_gradient(double x, double y, double g[4][2])
{
    double w[4], wx[4], wy[4];
    sin_prims(x, y, w, wx, wy);
    double r = w[0], u = w[1], v = w[2];
    double d[2][4] = {{wx[0], wx[1], wx[2], wx[3]}, {wy[0], wy[1], wy[2], wy[3]}};
    for (int k = 0; k < 2; k++) {
        double rk = d[k][0], uk = d[k][1], vk = d[k][2], pk = d[k][3];
        g[0][k] = rk;
        g[1][k] = rk * u + r * uk;
        g[2][k] = rk * v + r * vk;
        g[3][k] = pk / (GAMMA - 1.0) + 0.5 * rk * (u * u + v * v) + r * (u * uk + v * vk);
    }
}

static void sin_source(double x, double y, double S[4])
{
    double w[4], wx[4], wy[4];
    sin_prims(x, y, w, wx, wy);
    double r = w[0], u = w[1], v = w[2], p = w[3];
    double rx = wx[0], ry = wy[0], ux = wx[1], uy = wy[1], vx = wx[2], vy = wy[2], px = wx[3], py = wy[3];
    double rE = p / (GAMMA - 1.0) + 0.5 * r * (u * u + v * v);
    double rEx = px / (GAMMA - 1.0) + 0.5 * rx * (u * u + v * v) + r * (u * ux + v * vx);
    double rEy = py / (GAMMA - 1.0) + 0.5 * ry * (u * u + v * v) + r * (u * uy + v * vy);
    double H = rE + p, Hx = rEx + px, Hy = rEy + py;
    S[0] = rx * u + r * ux + ry * v + r * vy;
    S[1] = rx * u * u + 2.0 * r * u * ux + px + ry * u * v + r * uy * v + r * u * vy;
    S[2] = rx * u * v + r * ux * v + r * u * vx + ry * v * v + 2.0 * r * v * vy + py;
    S[3] = ux * H + u * Hx + vy * H + v * Hy;
}

static void mms_solution(int kind, double x, double y, double q[4])
{
    if (kind == 1)
        ref_solution(x, y, q);
    else
        sin_solution(x, y, q);
}
static void mms_gradient(int kind, double x, double y, double g[4][2])
{
    if (kind == 1)
        ref_solutionGradient(x, y, g);
    else
        sin_gradient(x, y, g);
}
static void mms_source(int kind, double x, double y, const ocfg *cfg, double S[4])
{
    if (kind == 1)
        ref_sourceTerm(x, y, cfg, S);
    else
        sin_source(x, y, S);
}

void o_mms_eval(int kind, int n, const double *xy, double *q, double *grad, double *src, const ocfg *cfg)
{
    for (int i = 0; i < n; i++) {
        double g[4][2];
        mms_solution(kind, xy[2 * i], xy[2 * i + 1], q + 4 * i);
        mms_gradient(kind, xy[2 * i], xy[2 * i + 1], g);
        for (int c = 0; c < 4; c++) {
            grad[8 * i + 2 * c] = g[c][0];
            grad[8 * i + 2 * c + 1] = g[c][1];
        }
        mms_source(kind, xy[2 * i], xy[2 * i + 1], cfg, src + 4 * i);
    }
}

/* ------------------------------------------------------------------------- */
/* Edge hash keyed on the sorted node pair (restates the mir.sparse maps of
   mesh.d:220-227; only membership and stored values matter). */
typedef struct {
    uint64_t *keys;
    int *vals;
    size_t cap;
} OHash;

static uint64_t hkey(uint32_t a, uint32_t b)
{
    uint32_t n1 = a > b ? b : a, n2 = a > b ? a : b;
    return ((uint64_t)n1 << 32) | n2;
}
static size_t hslot(const OHash *h, uint64_t k)
{
    uint64_t x = k * 0x9E3779B97F4A7C15ull;
    return (size_t)(x >> 17) & (h->cap - 1);
}
static void hinit(OHash *h, size_t n)
{
    size_t cap = 16;
    while (cap < 2 * n + 16) cap <<= 1;
    h->cap = cap;
    h->keys = (uint64_t *)malloc(cap * sizeof(uint64_t));
    h->vals = (int *)calloc(cap, sizeof(int));
    for (size_t i = 0; i < cap; i++) h->keys[i] = ~0ull;
}
static int hget(const OHash *h, uint64_t k)
{
    size_t s = hslot(h, k);
    while (h->keys[s] != ~0ull) {
        if (h->keys[s] == k) return h->vals[s];
        s = (s + 1) & (h->cap - 1);
    }
    return 0;
}
static void hset(OHash *h, uint64_t k, int v)
{
    size_t s = hslot(h, k);
    while (h->keys[s] != ~0ull && h->keys[s] != k) s = (s + 1) & (h->cap - 1);
    h->keys[s] = k;
    h->vals[s] = v;
}
static void hfree(OHash *h)
{
    free(h->keys);
    free(h->vals);
}

static int push_edge(OMesh *m, const OEdge *e)
{
    if (m->nEdges == m->capEdges) {
        m->capEdges = m->capEdges ? 2 * m->capEdges : 1024;
        m->edges = (OEdge *)realloc(m->edges, (size_t)m->capEdges * sizeof(OEdge));
    }
    m->edges[m->nEdges] = *e;
    return m->nEdges++;
}

/* mesh.d:217-643 (single rank: no comm edges, so the hasCommNeighbor split and the
   extra-neighbour search for boundary triangles never trigger: every boundary
   edge already has its ghost cell as neighbour when gradMat is built). */
OMesh *o_mesh_create(int nNodes, const double *xy, int nElem, const int *elemOff, const int *elemNodes, int nB,
                     const int *bNodes, int nGroups, const int *bGroupStart, const int *groupBc)
{
    OMesh *m = (OMesh *)calloc(1, sizeof(OMesh));
    m->nNodes = nNodes;
    m->nodes = (double(*)[2])malloc(sizeof(double) * 2 * (size_t)nNodes);
    memcpy(m->nodes, xy, sizeof(double) * 2 * (size_t)nNodes);
    m->nElem = nElem;
    m->elemOff = (int *)malloc(sizeof(int) * (size_t)(nElem + 1));
    memcpy(m->elemOff, elemOff, sizeof(int) * (size_t)(nElem + 1));
    m->elemNodes = (int *)malloc(sizeof(int) * (size_t)elemOff[nElem]);
    memcpy(m->elemNodes, elemNodes, sizeof(int) * (size_t)elemOff[nElem]);
    m->nB = nB;
    m->bNodes = (int(*)[2])malloc(sizeof(int) * 2 * (size_t)(nB > 0 ? nB : 1));
    memcpy(m->bNodes, bNodes, sizeof(int) * 2 * (size_t)nB);
    m->nGroups = nGroups;
    m->bGroupStart = (int *)malloc(sizeof(int) * (size_t)(nGroups + 1));
    memcpy(m->bGroupStart, bGroupStart, sizeof(int) * (size_t)nGroups);
    m->groupBc = (int *)malloc(sizeof(int) * (size_t)(nGroups + 1));
    memcpy(m->groupBc, groupBc, sizeof(int) * (size_t)nGroups);

    int C = nElem;
    int cap = C + nB + 16;
    m->cells = (OCell *)calloc((size_t)cap * 2, sizeof(OCell));
    m->nInterior = C;

    OHash edgeHash, bHash;
    hinit(&edgeHash, (size_t)elemOff[nElem]);
    hinit(&bHash, (size_t)nB);
    for (int i = 0; i < nB; i++) hset(&bHash, hkey((uint32_t)bNodes[2 * i], (uint32_t)bNodes[2 * i + 1]), i + 1);

    int *bGroupCount = (int *)calloc((size_t)nGroups + 1, sizeof(int));
    int *edgeGroup = NULL; /* group of each boundary edge, in creation order */
    int nBndCap = 0;
    m->interiorEdges = (int *)malloc(sizeof(int) * (size_t)elemOff[nElem]);
    m->boundaryEdges = (int *)malloc(sizeof(int) * (size_t)elemOff[nElem]);

    for (int i = 0; i < C; i++) {
        OCell *c = &m->cells[i];
        int ne = elemOff[i + 1] - elemOff[i];
        const int *el = elemNodes + elemOff[i];
        c->nEdges = (uint32_t)ne;
        for (int j = 0; j < MAX_EDGES; j++) {
            c->edges[j] = 0;
            c->fluxMultiplier[j] = 1.0;
        }
        c->area = 0.0;
        c->d = 0.0;
        c->perim = 0;
        c->centroid[0] = c->centroid[1] = 0;
        c->nNb = 0;
        for (int k = 0; k < 4; k++) c->lim[k][0] = c->lim[k][1] = 1.0;
        c->dt = NAN;

        for (int j = 0; j < ne; j++) {
            uint32_t ni0 = (uint32_t)(el[j] - 1), ni1 = (uint32_t)(el[(j + 1) % ne] - 1);
            int edgeidx;
            int bi = hget(&bHash, hkey(ni0, ni1));
            double x0 = m->nodes[ni0][0], y0 = m->nodes[ni0][1], x1 = m->nodes[ni1][0], y1 = m->nodes[ni1][1];
            if (bi == 0) {
                int hv = hget(&edgeHash, hkey(ni0, ni1));
                if (hv != 0) {
                    edgeidx = hv - 1;
                    m->edges[edgeidx].cellIdx[1] = (uint32_t)i;
                    c->fluxMultiplier[j] = -1.0;
                } else {
                    OEdge e;
                    memset(&e, 0, sizeof e);
                    e.nodeIdx[0] = ni0;
                    e.nodeIdx[1] = ni1;
                    e.cellIdx[0] = (uint32_t)i;
                    double dx = x0 - x1, dy = y0 - y1;
                    e.len = sqrt(dx * dx + dy * dy);
                    double nx = y1 - y0, ny = x0 - x1;
                    double mag = sqrt(nx * nx + ny * ny);
                    e.normal[0] = nx / mag;
                    e.normal[1] = ny / mag;
                    e.mid[0] = 0.5 * (x0 + x1);
                    e.mid[1] = 0.5 * (y0 + y1);
                    e.bGroup = -1;
                    c->fluxMultiplier[j] = 1.0;
                    edgeidx = push_edge(m, &e);
                    hset(&edgeHash, hkey(ni0, ni1), edgeidx + 1);
                    m->interiorEdges[m->nInt++] = edgeidx;
                }
            } else {
                int bIdx0 = bi - 1;
                int bGroup = 0;
                for (int g = 0; g < nGroups - 1; g++)
                    if (bIdx0 >= bGroupStart[g] && bIdx0 < bGroupStart[g + 1]) bGroup = g;
                if (bIdx0 >= bGroupStart[nGroups - 1]) bGroup = nGroups - 1;
                OEdge e;
                memset(&e, 0, sizeof e);
                e.nodeIdx[0] = ni0;
                e.nodeIdx[1] = ni1;
                e.cellIdx[0] = (uint32_t)i;
                double dx = x0 - x1, dy = y0 - y1;
                e.len = sqrt(dx * dx + dy * dy);
                double inv = 1.0 / e.len;
                e.normal[0] = inv * (y1 - y0);
                e.normal[1] = inv * (x0 - x1);
                e.mid[0] = 0.5 * (x0 + x1);
                e.mid[1] = 0.5 * (y0 + y1);
                e.isBoundary = 1;
                e.bGroup = bGroup;
                c->fluxMultiplier[j] = 1.0;
                edgeidx = push_edge(m, &e);
                m->boundaryEdges[m->nBnd++] = edgeidx;
                if (m->nBnd > nBndCap) {
                    nBndCap = nBndCap ? 2 * nBndCap : 1024;
                    edgeGroup = (int *)realloc(edgeGroup, sizeof(int) * (size_t)nBndCap);
                }
                edgeGroup[m->nBnd - 1] = bGroup;
                bGroupCount[bGroup]++;
            }
            c->edges[j] = (uint32_t)edgeidx;
            c->perim += m->edges[edgeidx].len;
            double det = x0 * y1 - x1 * y0;
            c->area += det;
            c->centroid[0] += (x0 + x1) * (x0 * y1 - x1 * y0);
            c->centroid[1] += (y0 + y1) * (x0 * y1 - x1 * y0);
        }
        c->area *= 0.5;
        if (!(c->area > 0)) {
            m->errIndex = i;
        }
        c->d = (2 * c->area) / c->perim;
        c->centroid[0] *= 1 / (6 * c->area);
        c->centroid[1] *= 1 / (6 * c->area);
    }
    hfree(&edgeHash);
    hfree(&bHash);

    /* bGroups: per-group boundary edge lists in creation order */
    m->groupEdgeOff = (int *)calloc((size_t)nGroups + 1, sizeof(int));
    for (int g = 0; g < nGroups; g++) m->groupEdgeOff[g + 1] = m->groupEdgeOff[g] + bGroupCount[g];
    m->groupEdges = (int *)malloc(sizeof(int) * (size_t)(m->nBnd + 1));
    {
        int *fill = (int *)calloc((size_t)nGroups + 1, sizeof(int));
        for (int b = 0; b < m->nBnd; b++) {
            int g = edgeGroup[b];
            m->groupEdges[m->groupEdgeOff[g] + fill[g]++] = m->boundaryEdges[b];
        }
        free(fill);
    }
    free(edgeGroup);
    free(bGroupCount);

    /* ghost cells (mesh.d:329-381) */
    m->nCells = C + m->nBnd;
    for (int b = 0; b < m->nBnd; b++) {
        int be = m->boundaryEdges[b];
        OEdge *e = &m->edges[be];
        OCell *g = &m->cells[C + b];
        memset(g, 0, sizeof *g);
        for (int j = 0; j < MAX_EDGES; j++) g->fluxMultiplier[j] = -1.0;
        const OCell *other = &m->cells[e->cellIdx[0]];
        double xr, yr;
        double nx0 = m->nodes[e->nodeIdx[0]][0], ny0 = m->nodes[e->nodeIdx[0]][1];
        double nx1 = m->nodes[e->nodeIdx[1]][0], ny1 = m->nodes[e->nodeIdx[1]][1];
        if (nx0 != nx1) {
            double x1 = other->centroid[0], y1 = other->centroid[1];
            double mm = (ny0 - ny1) / (nx0 - nx1);
            double x = nx0, y = ny0;
            double cc = y - mm * x;
            double d = (x1 + (y1 - cc) * mm) / (1.0 + mm * mm);
            xr = 2.0 * d - x1;
            yr = 2.0 * d * mm - y1 + 2.0 * cc;
        } else {
            double x = nx0;
            double d = other->centroid[0] - x;
            double x1 = other->centroid[0];
            xr = -(2.0 * d - x1);
            yr = other->centroid[1];
        }
        g->centroid[0] = xr;
        g->centroid[1] = yr;
        g->nNb = 1;
        for (int k = 0; k < 4; k++) g->lim[k][0] = g->lim[k][1] = 1.0;
        g->nb[0] = e->cellIdx[0];
        g->edges[0] = (uint32_t)be;
        g->nEdges = 0;
        g->dt = NAN;
        e->cellIdx[1] = (uint32_t)(C + b);
    }

    /* neighbours and least-squares pseudo-inverse (mesh.d:481-642) */
    for (int i = 0; i < C; i++) {
        OCell *c = &m->cells[i];
        double tmp[MAX_EDGES][2];
        memset(tmp, 0, sizeof tmp);
        memset(c->gradMat, 0, sizeof c->gradMat);
        c->nNb = 0;
        for (uint32_t j = 0; j < c->nEdges; j++) {
            const OEdge *e = &m->edges[c->edges[j]];
            uint32_t idx = (e->cellIdx[0] == (uint32_t)i) ? e->cellIdx[1] : e->cellIdx[0];
            c->nb[c->nNb] = idx;
            tmp[c->nNb][0] = m->cells[idx].centroid[0] - c->centroid[0];
            tmp[c->nNb][1] = m->cells[idx].centroid[1] - c->centroid[1];
            c->nNb++;
        }
        /* b = A^T A, c = b^-1, gradMat = c A^T */
        double b[2][2];
        for (int r = 0; r < 2; r++)
            for (int s = 0; s < 2; s++) {
                double acc = 0.0;
                for (int k = 0; k < MAX_EDGES; k++) acc += tmp[k][r] * tmp[k][s];
                b[r][s] = acc;
            }
        double det = b[0][0] * b[1][1] - b[0][1] * b[1][0];
        double id = 1.0 / det;
        double ci[2][2] = {{b[1][1] * id, -b[0][1] * id}, {-b[1][0] * id, b[0][0] * id}};
        for (int r = 0; r < 2; r++)
            for (int k = 0; k < MAX_EDGES; k++) c->gradMat[r][k] = ci[r][0] * tmp[k][0] + ci[r][1] * tmp[k][1];
    }

    size_t NC = (size_t)m->nCells;
    m->q = (double(*)[4])calloc(NC, sizeof(double[4]));
    m->R = (double(*)[4])calloc(NC, sizeof(double[4]));
    m->tmp = (double(*)[4])calloc(NC, sizeof(double[4]));
    m->k1 = (double(*)[4])calloc(NC, sizeof(double[4]));
    m->k2 = (double(*)[4])calloc(NC, sizeof(double[4]));
    m->k3 = (double(*)[4])calloc(NC, sizeof(double[4]));
    m->k4 = (double(*)[4])calloc(NC, sizeof(double[4]));
    m->qFE = (double(*)[4])calloc(NC, sizeof(double[4]));
    for (int k = 0; k < 4; k++) m->last[k] = (double *)calloc(NC, sizeof(double));
    return m;
}

void o_mesh_free(OMesh *m)
{
    if (!m) return;
    free(m->nodes);
    free(m->elemOff);
    free(m->elemNodes);
    free(m->bNodes);
    free(m->bGroupStart);
    free(m->groupBc);
    free(m->cells);
    free(m->edges);
    free(m->interiorEdges);
    free(m->boundaryEdges);
    free(m->groupEdgeOff);
    free(m->groupEdges);
    free(m->q);
    free(m->R);
    free(m->tmp);
    free(m->k1);
    free(m->k2);
    free(m->k3);
    free(m->k4);
    free(m->qFE);
    for (int k = 0; k < 4; k++) free(m->last[k]);
    free(m);
}

void o_mesh_sizes(const OMesh *m, int *out)
{
    out[0] = m->nInterior;
    out[1] = m->nCells - m->nInterior;
    out[2] = m->nEdges;
    out[3] = m->nInt;
    out[4] = m->nBnd;
    out[5] = (int)m->errIndex;
}

/* Geometry export for the parity tests. cellGeo per interior cell:
   area, perim, d, cx, cy, nEdges, gradMat[2][6]. edgeGeo per edge: len, nx, ny, mx, my,
   cellL, cellR, isBoundary. cellTopo per cell: edges[6], nb[6], fluxMultiplier sign[6]. */
void o_mesh_geometry(const OMesh *m, double *cellGeo, double *edgeGeo, int *cellTopo, double *ghostCentroid)
{
    for (int i = 0; i < m->nInterior; i++) {
        const OCell *c = &m->cells[i];
        double *g = cellGeo + 18 * i;
        g[0] = c->area;
        g[1] = c->perim;
        g[2] = c->d;
        g[3] = c->centroid[0];
        g[4] = c->centroid[1];
        g[5] = c->nEdges;
        for (int k = 0; k < 6; k++) {
            g[6 + k] = c->gradMat[0][k];
            g[12 + k] = c->gradMat[1][k];
        }
        int *t = cellTopo + 18 * i;
        for (int k = 0; k < 6; k++) {
            t[k] = (int)c->edges[k];
            t[6 + k] = (k < (int)c->nNb) ? (int)c->nb[k] : -1;
            t[12 + k] = c->fluxMultiplier[k] > 0 ? 1 : -1;
        }
    }
    for (int e = 0; e < m->nEdges; e++) {
        const OEdge *E = &m->edges[e];
        double *g = edgeGeo + 8 * e;
        g[0] = E->len;
        g[1] = E->normal[0];
        g[2] = E->normal[1];
        g[3] = E->mid[0];
        g[4] = E->mid[1];
        g[5] = E->cellIdx[0];
        g[6] = E->cellIdx[1];
        g[7] = E->isBoundary;
    }
    for (int b = 0; b < m->nBnd; b++) {
        ghostCentroid[2 * b] = m->cells[m->nInterior + b].centroid[0];
        ghostCentroid[2 * b + 1] = m->cells[m->nInterior + b].centroid[1];
    }
}

/* ------------------------------------------------------------------------- */
/* ufvmSetup (solve.d:175-279) with the MMS variant of app/ms.d:236-298. */
void o_setup(OMesh *m, const ocfg *cfg)
{
    m->cfg = *cfg;
    ocfg *c = &m->cfg;
    double M = c->ic[0], aoa = c->ic[1] * (M_PI / 180), rho = c->ic[3];
    double U = 1.0, a = U / M, p = (rho * (a * a)) / GAMMA, u = U * cos(aoa), v = U * sin(aoa);
    if (c->viscosity)
        c->mu = (rho * U * c->L) / c->Re;
    else
        c->mu = NAN; /* PhysicalConfig.mu is never set without viscosity (D initialises doubles to NaN) */

    for (int i = 0; i < m->nInterior; i++) {
        if (c->mms) {
            mms_solution(c->mms, m->cells[i].centroid[0], m->cells[i].centroid[1], m->q[i]);
        } else {
            m->q[i][0] = rho;
            m->q[i][1] = rho * u;
            m->q[i][2] = rho * v;
            m->q[i][3] = p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v);
        }
        for (int k = 0; k < 4; k++) m->last[k][i] = m->q[i][k];
    }

    for (int g = 0; g < m->nGroups; g++) {
        int bcIdx = m->groupBc[g];
        for (int j = m->groupEdgeOff[g]; j < m->groupEdgeOff[g + 1]; j++) {
            OEdge *e = &m->edges[m->groupEdges[j]];
            e->type = c->bcType[bcIdx];
            e->bIdx = bcIdx;
            if (e->type == BC_FULLSTATE) {
                double bM = c->bcData[bcIdx][0], baoa = c->bcData[bcIdx][1] * (M_PI / 180), brho = c->bcData[bcIdx][3];
                double ba = 1.0 / bM, bp = (brho * (ba * ba)) / GAMMA, bu = 1.0 * cos(baoa), bv = 1.0 * sin(baoa);
                e->q[1][0] = brho;
                e->q[1][1] = brho * bu;
                e->q[1][2] = brho * bv;
                e->q[1][3] = bp / (GAMMA - 1.0) + 0.5 * brho * (bu * bu + bv * bv);
            } else if (e->type == BC_CONSTP || e->type == BC_TPINFLOW) {
                for (int k = 0; k < c->bcNData[bcIdx] && k < 4; k++) e->bData[k] = c->bcData[bcIdx][k];
            } else if (e->type == BC_DIRICHLET) {
                mms_solution(c->mms ? c->mms : 1, e->mid[0], e->mid[1], e->q[1]);
            }
        }
    }
    m->t = 0;
    m->dt = c->dt;
    m->iterations = 0;
    m->residRhoLast = INFINITY;
    m->residIncIters = 0;
}

void o_get_state(const OMesh *m, double *q)
{
    memcpy(q, m->q, sizeof(double) * 4 * (size_t)m->nInterior);
}
void o_set_state(OMesh *m, const double *q)
{
    memcpy(m->q, q, sizeof(double) * 4 * (size_t)m->nInterior);
    for (int i = 0; i < m->nInterior; i++)
        for (int k = 0; k < 4; k++) m->last[k][i] = m->q[i][k];
}
void o_get_cfg(const OMesh *m, ocfg *c) { *c = m->cfg; }
void o_set_cfl(OMesh *m, double cfl) { m->cfg.CFL = cfl; }

/* ------------------------------------------------------------------------- */
static void reflectVel(const OMesh *m, const OEdge *e, const double v[2], double out[2])
{
    double x1 = m->nodes[e->nodeIdx[0]][0], y1 = m->nodes[e->nodeIdx[0]][1];
    double x2 = m->nodes[e->nodeIdx[1]][0], y2 = m->nodes[e->nodeIdx[1]][1];
    if (x1 != x2) {
        double mm = (y2 - y1) / (x2 - x1);
        double den = 1 + mm * mm;
        double r00 = (1 - mm * mm) * 1.0 / den, r01 = 2.0 * mm * 1.0 / den, r10 = 2.0 * mm * 1.0 / den,
               r11 = (mm * mm - 1) * 1.0 / den;
        out[0] = r00 * v[0] + r01 * v[1];
        out[1] = r10 * v[0] + r11 * v[1];
    } else {
        out[0] = -v[0];
        out[1] = v[1];
    }
}

/* LP!m (solve.d:37-173) */
static void lp_solve(int mrows, double A[][2], const double *b, const double c[2], double xk[2])
{
    int Wk[2] = {0, 1};
    double Ak[4] = {A[Wk[0]][0], A[Wk[0]][1], A[Wk[1]][0], A[Wk[1]][1]};
    double pk[2] = {0, 0}, lam[2] = {0, 0}, e[2] = {0, 0};
    int D[12];
    double gam[12];
    int k = 0;
    for (;;) {
        double det = Ak[0] * Ak[3] - Ak[1] * Ak[2];
        double id = 1.0 / det;
        double inv[4] = {Ak[3] * id, -Ak[2] * id, -Ak[1] * id, Ak[0] * id}; /* invertTrans */
        lam[0] = inv[0] * c[0] + inv[1] * c[1];
        lam[1] = inv[2] * c[0] + inv[3] * c[1];
        if ((lam[0] >= -10e-9) && (lam[1] >= -10e-9)) break;
        int qi = (lam[0] < lam[1]) ? Wk[0] : Wk[1];
        if (lam[0] < lam[1]) {
            e[0] = 1;
            e[1] = 0;
        } else {
            e[0] = 0;
            e[1] = 1;
        }
        double inv2[4] = {Ak[3] * id, -Ak[1] * id, -Ak[2] * id, Ak[0] * id}; /* invert */
        pk[0] = inv2[0] * e[0] + inv2[1] * e[1];
        pk[1] = inv2[2] * e[0] + inv2[3] * e[1];
        int Dlen = 0;
        for (int i = 0; i < mrows; i++)
            if (i != Wk[0] && i != Wk[1])
                if (A[i][0] * pk[0] + A[i][1] * pk[1] < -1e-11) D[Dlen++] = i;
        double alpha = INFINITY;
        for (int i = 0; i < Dlen; i++) {
            double aixk = A[D[i]][0] * xk[0] + A[D[i]][1] * xk[1];
            double aipk = A[D[i]][0] * pk[0] + A[D[i]][1] * pk[1];
            gam[i] = (aixk - b[D[i]]) / (-aipk);
            alpha = fmin(alpha, gam[i]);
        }
        int t = 0;
        for (int i = 0; i < Dlen; i++)
            if (gam[i] == alpha) {
                t = D[i];
                break;
            }
        if (qi == Wk[0])
            Wk[0] = t;
        else if (qi == Wk[1])
            Wk[1] = t;
        Ak[0] = A[Wk[0]][0];
        Ak[1] = A[Wk[0]][1];
        Ak[2] = A[Wk[1]][0];
        Ak[3] = A[Wk[1]][1];
        xk[0] += alpha * pk[0];
        xk[1] += alpha * pk[1];
        k++;
        if (k > 15) break;
    }
}

/* buildGradients (solve.d:324-508) for one cell */
static void build_gradient(OMesh *m, double (*q)[4], int i, int limit)
{
    OCell *c = &m->cells[i];
    const ocfg *cfg = &m->cfg;
    double du[4][MAX_EDGES];
    memset(du, 0, sizeof du);
    for (int k = 0; k < 4; k++) {
        c->minQ[k] = q[i][k];
        c->maxQ[k] = q[i][k];
        c->lim[k][0] = c->lim[k][1] = 1.0;
    }
    for (uint32_t j = 0; j < c->nNb; j++) {
        uint32_t idx = c->nb[j];
        for (int k = 0; k < 4; k++) {
            c->minQ[k] = fmin(c->minQ[k], q[idx][k]);
            c->maxQ[k] = fmax(c->maxQ[k], q[idx][k]);
            du[k][j] = q[idx][k] - q[i][k];
        }
    }
    for (int k = 0; k < 4; k++)
        for (int r = 0; r < 2; r++) {
            double acc = 0.0;
            for (int j = 0; j < MAX_EDGES; j++) acc += c->gradMat[r][j] * du[k][j];
            c->grad[k][r] = acc;
        }
    if (cfg->limited && limit) {
        for (uint32_t j = 0; j < c->nNb; j++) {
            const OCell *nbc = &m->cells[c->nb[j]];
            double dx = nbc->centroid[0] - c->centroid[0];
            double dy = nbc->centroid[1] - c->centroid[1];
            for (int k = 0; k < 4; k++) {
                double s = 1.0;
                double qE = q[i][k] + (c->grad[k][0] * dx + c->grad[k][1] * dy);
                if (qE < c->minQ[k])
                    s = (c->minQ[k] - q[i][k]) / (c->grad[k][0] * dx + c->grad[k][1] * dy);
                else if (qE > c->maxQ[k])
                    s = (c->maxQ[k] - q[i][k]) / (c->grad[k][0] * dx + c->grad[k][1] * dy);
                c->lim[k][0] = fmin(c->lim[k][0], s);
                c->lim[k][1] = c->lim[k][0];
            }
        }
        if (cfg->lpThresh > 0) {
            for (int k = 0; k < 4; k++) {
                if (c->lim[k][0] < cfg->lpThresh && (c->nNb == 3 || c->nNb == 4)) {
                    int mr = 4 + 2 * (int)c->nNb;
                    double A[12][2];
                    double b[12];
                    memset(A, 0, sizeof A);
                    memset(b, 0, sizeof b);
                    double cc[2] = {-fabs(c->grad[k][0]), -fabs(c->grad[k][1])};
                    double xk[2] = {0, 0};
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
                    for (uint32_t j = 0, ci = 0; j < c->nNb; j++, ci += 2) {
                        const OCell *nbc = &m->cells[c->nb[j]];
                        A[ci + 4][0] = (nbc->centroid[0] - c->centroid[0]) * c->grad[k][0];
                        A[ci + 4][1] = (nbc->centroid[1] - c->centroid[1]) * c->grad[k][1];
                        b[ci + 4] = c->minQ[k] - q[i][k];
                        A[ci + 5][0] = -(nbc->centroid[0] - c->centroid[0]) * c->grad[k][0];
                        A[ci + 5][1] = -(nbc->centroid[1] - c->centroid[1]) * c->grad[k][1];
                        b[ci + 5] = q[i][k] - c->maxQ[k];
                    }
                    lp_solve(mr, A, b, cc, xk);
                    c->lim[k][0] = xk[0];
                    c->lim[k][1] = xk[1];
                }
            }
        }
    }
}

/* face reconstruction, interior form (solve.d:980-1011) */
static void reconstruct(OMesh *m, double (*q)[4], uint32_t ci, const double mid[2], double out[4], int bndQuirk)
{
    const OCell *c = &m->cells[ci];
    double dx = mid[0] - c->centroid[0];
    double dy = mid[1] - c->centroid[1];
    for (int j = 0; j < 4; j++) out[j] = q[ci][j] + c->lim[j][0] * c->grad[j][0] * dx + c->lim[j][1] * c->grad[j][1] * dy;
    if (getPressure(out) < 0) {
        double l0 = 1.0, l1 = 1.0;
        for (int j = 0; j < 4; j++) {
            l0 = fmin(l0, c->lim[j][0]);
            l1 = fmin(l1, c->lim[j][1]);
        }
        if (bndQuirk) l1 = l0; /* solve.d:311,315: boundary fallback uses lim[0] in both directions */
#pragma omp atomic
        m->nFallback[bndQuirk ? 1 : 0]++;
        for (int j = 0; j < 4; j++) out[j] = q[ci][j] + l0 * c->grad[j][0] * dx + l1 * c->grad[j][1] * dy;
    }
}

static int has_nan4(const double f[4]) { return isnan(f[0]) || isnan(f[1]) || isnan(f[2]) || isnan(f[3]); }

/* ufvmSolver (solve.d:322-1122).  Returns 0 or O_ERR_NAN_EDGE (m->errIndex = edge id). */
int o_solver(OMesh *m, double (*R)[4], double (*q)[4], double *newDt, double *Rmax, int limit, int dtUpdate)
{
    m->nFallback[0] = m->nFallback[1] = 0;
    const ocfg *cfg = &m->cfg;
    int C = m->nInterior;
    /* ghost states (solve.d:521-689) */
    int firstBad = INT_MAX;
#pragma omp parallel for schedule(static) reduction(min : firstBad)
    for (int b = 0; b < m->nBnd; b++) {
        int gi = C + b;
        OEdge *e = &m->edges[m->cells[gi].edges[0]];
        uint32_t ci = e->cellIdx[0];
        uint32_t c2 = e->cellIdx[1];
        switch (e->type) {
        case BC_DIRICHLET:
            mms_solution(cfg->mms ? cfg->mms : 1, m->cells[gi].centroid[0], m->cells[gi].centroid[1], q[gi]);
            break;
        case BC_FULLSTATE:
            for (int k = 0; k < 4; k++) q[c2][k] = q[ci][k];
            break;
        case BC_INVWALL:
        case BC_SYMMETRY: {
            double v[2] = {q[ci][1] / q[ci][0], q[ci][2] / q[ci][0]}, nv[2];
            reflectVel(m, e, v, nv);
            q[c2][0] = q[ci][0];
            q[c2][1] = q[ci][0] * nv[0];
            q[c2][2] = q[ci][0] * nv[1];
            q[c2][3] = q[ci][3];
            break;
        }
        case BC_VISCWALL:
            q[c2][0] = q[ci][0];
            q[c2][1] = -q[ci][1];
            q[c2][2] = -q[ci][2];
            q[c2][3] = q[ci][3];
            break;
        case BC_CONSTP: {
            double rhop = q[ci][0], up = q[ci][1] / q[ci][0], vp = q[ci][2] / q[ci][0];
            double pp = getPressure(q[ci]);
            double ap = sqrt(GAMMA * (pp / rhop));
            double Jp = up + (2.0 * ap) / (GAMMA - 1);
            double Sp = pp / pow(rhop, GAMMA);
            double pb = e->bData[0];
            double rhob = pow(pb / Sp, 1.0 / GAMMA);
            double ab = sqrt(GAMMA * (pb / rhob));
            double ub = Jp - (2.0 * ab) / (GAMMA - 1);
            double vb = vp;
            double mag = sqrt(ub * ub + vb * vb);
            double rEb = pb / (GAMMA - 1) + 0.5 * rhob * (mag * mag);
            const double *n = e->normal;
            double vpn = up * n[0] + vp * n[1];
            double vbn = ub * n[0] + vb * n[1];
            double Vbg0 = up - vpn * n[0] + vbn * n[0];
            double Vbg1 = vp - vpn * n[1] + vbn * n[1];
            q[c2][0] = rhob;
            q[c2][1] = rhob * Vbg0;
            q[c2][2] = rhob * Vbg1;
            q[c2][3] = rEb;
            break;
        }
        case BC_TPINFLOW: {
            double Tt = e->bData[0], Pt = e->bData[1], aoa = e->bData[2] * M_PI / 180;
            double rhop = q[ci][0], up = q[ci][1] / q[ci][0];
            double pp = getPressure(q[ci]);
            double ap = sqrt(GAMMA * (pp / rhop));
            double Jp = up + (2.0 * ap) / (GAMMA - 1);
            double nin[2] = {cos(aoa), sin(aoa)};
            double d = nin[0] * e->normal[0] + nin[1] * e->normal[1];
            double Rg = cfg->R;
            double aa = GAMMA * Rg * Tt * (d * d) - 0.5 * (GAMMA - 1) * (Jp * Jp);
            double bb = (4.0 * GAMMA * Rg * Tt * d) / (GAMMA - 1);
            double cc = (4.0 * GAMMA * Rg * Tt) / ((GAMMA - 1) * (GAMMA - 1)) - Jp * Jp;
            double M1 = (-bb + sqrt(bb * bb - 4 * aa * cc)) / (2.0 * aa);
            double M2 = (-bb - sqrt(bb * bb - 4 * aa * cc)) / (2.0 * aa);
            double Mb = 0;
            if (M1 >= 0 && M2 >= 0)
                Mb = fmin(M1, M2);
            else if (M1 >= 0 && M2 < 0)
                Mb = M1;
            else if (M1 < 0 && M2 >= 0)
                Mb = M2;
            else {
                if (b < firstBad) firstBad = b;
                break;
            }
            double Tb = Tt / (1 + 0.5 * (GAMMA - 1) * (Mb * Mb));
            double pb = Pt * pow(Tb / Tt, GAMMA / (GAMMA - 1));
            double rhob = pb / (Rg * Tb);
            double ab = sqrt(GAMMA * (pb / rhob));
            double vb0 = Mb * ab * nin[0], vb1 = Mb * ab * nin[1];
            double mag = sqrt(vb0 * vb0 + vb1 * vb1);
            double rEb = pb / (GAMMA - 1) + 0.5 * rhob * (mag * mag);
            (void)rhob;
            /* solve.d:678-681 writes every value into component 0; the last one stays */
            q[c2][0] = rEb;
            break;
        }
        default:
            break;
        }
    }

    if (firstBad != INT_MAX) {
        m->errIndex = m->cells[C + firstBad].edges[0];
        return O_ERR_BC;
    }

    if (cfg->order > 1) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++) build_gradient(m, q, i, limit);
    }

    /* boundary edges (solve.d:769-968) */
#pragma omp parallel for schedule(static) reduction(min : firstBad)
    for (int bb = 0; bb < m->nBnd; bb++) {
        int ei = m->boundaryEdges[bb];
        OEdge *e = &m->edges[ei];
        if (cfg->order == 1) {
            for (int k = 0; k < 4; k++) e->q[0][k] = q[e->cellIdx[0]][k];
        } else {
            reconstruct(m, q, e->cellIdx[0], e->mid, e->q[0], 1);
        }
        const double *n = e->normal;
        int type = e->type;
        if (type == BC_DIRICHLET) {
            OCell *g = &m->cells[e->cellIdx[1]];
            mms_gradient(cfg->mms ? cfg->mms : 1, g->centroid[0], g->centroid[1], g->grad);
            mms_solution(cfg->mms ? cfg->mms : 1, e->mid[0], e->mid[1], e->q[1]);
            type = BC_FULLSTATE;
        }
        switch (type) {
        case BC_FULLSTATE: {
            double F[4];
            invFlux(cfg->flux, e->q[0], e->q[1], n, F, &e->sMax);
            if (cfg->viscosity) {
                double qAve[4], dq[4][2], Fv[4];
                const OCell *g1 = &m->cells[e->cellIdx[0]], *g2 = &m->cells[e->cellIdx[1]];
                for (int k = 0; k < 4; k++) {
                    qAve[k] = 0.5 * (e->q[0][k] + e->q[1][k]);
                    dq[k][0] = 0.5 * (g1->grad[k][0] + g2->grad[k][0]);
                    dq[k][1] = 0.5 * (g1->grad[k][1] + g2->grad[k][1]);
                }
                diffusiveFlux(cfg->Pr, cfg->mu, qAve, dq, n, Fv);
                for (int k = 0; k < 4; k++) F[k] -= Fv[k];
            }
            memcpy(e->flux, F, sizeof F);
            break;
        }
        case BC_INVWALL: {
            double inv = 1 / e->q[0][0];
            double vp[2] = {inv * e->q[0][1], inv * e->q[0][2]};
            double vn = vp[0] * n[0] + vp[1] * n[1];
            double t0 = vp[0] - vn * n[0], t1 = vp[1] - vn * n[1];
            double vel = sqrt(t0 * t0 + t1 * t1);
            double p = (GAMMA - 1) * (e->q[0][3] - 0.5 * e->q[0][0] * (vel * vel));
            double a = sqrt(GAMMA * (p / e->q[0][0]));
            if (p < 0) p = 1.0e-12;
            e->flux[0] = 0;
            e->flux[1] = p * n[0];
            e->flux[2] = p * n[1];
            e->flux[3] = 0;
            e->sMax = fabs(a);
            for (int k = 0; k < 4; k++) e->q[1][k] = q[e->cellIdx[1]][k];
            break;
        }
        case BC_VISCWALL: {
            double vel = 0.0;
            double p = (GAMMA - 1) * (e->q[0][3] - 0.5 * e->q[0][0] * (vel * vel));
            double a = sqrt(GAMMA * (p / e->q[0][0]));
            if (p < 0) p = 1.0e-12;
            double qR[4] = {e->q[0][0], -e->q[0][1], -e->q[0][2], e->q[0][3]};
            qR[1] = e->q[0][1] * -1;
            qR[2] = e->q[0][2] * -1;
            memcpy(e->q[1], qR, sizeof qR);
            double qAve[4];
            for (int k = 0; k < 4; k++) qAve[k] = 0.5 * (e->q[0][k] + qR[k]);
            qAve[1] = 0.0;
            qAve[2] = 0.0;
            double dq[4][2];
            memcpy(dq, m->cells[e->cellIdx[0]].grad, sizeof dq);
            dq[3][0] = (qAve[3] / qAve[0]) * dq[0][0];
            dq[3][1] = (qAve[3] / qAve[0]) * dq[0][1];
            double Fv[4];
            diffusiveFlux(cfg->Pr, cfg->mu, qAve, dq, n, Fv);
            double F0[4] = {0, p * n[0], p * n[1], 0};
            for (int k = 0; k < 4; k++) e->flux[k] = F0[k] - Fv[k];
            e->sMax = fabs(a);
            break;
        }
        case BC_CONSTP: {
            const double *qg = q[e->cellIdx[1]];
            double p = getPressure(qg);
            double u = qg[1] / qg[0], v = qg[2] / qg[0];
            double a = sqrt(GAMMA * (p / qg[0]));
            for (int k = 0; k < 4; k++) e->q[1][k] = qg[k];
            convectiveFlux(p, u, v, qg[0], qg[3], n, e->flux);
            e->sMax = fabs(a);
            break;
        }
        case BC_SYMMETRY: {
            double v[2] = {e->q[0][1] / e->q[0][0], e->q[0][2] / e->q[0][0]}, nv[2];
            reflectVel(m, e, v, nv);
            e->q[1][0] = e->q[0][0];
            e->q[1][1] = e->q[0][0] * nv[0];
            e->q[1][2] = e->q[0][0] * nv[1];
            e->q[1][3] = e->q[0][3];
            double F[4];
            invFlux(cfg->flux, e->q[0], e->q[1], n, F, &e->sMax);
            if (cfg->viscosity) {
                double qAve[4];
                for (int k = 0; k < 4; k++) qAve[k] = 0.5 * (e->q[0][k] + e->q[1][k]);
                const double(*gp)[2] = m->cells[e->cellIdx[0]].grad;
                double nO[2][2] = {{n[0] * n[0], n[0] * n[1]}, {n[1] * n[0], n[1] * n[1]}};
                double A[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
                double V[2][2] = {{1 - nO[0][0], 0 - nO[0][1]}, {0 - nO[1][0], 1 - nO[1][1]}};
                A[1][1] = V[0][0];
                A[1][2] = V[0][1];
                A[2][1] = V[1][0];
                A[2][2] = V[1][1];
                double t1[4][2], t3[4][2], bG[4][2];
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 2; j++) {
                        double acc = 0.0;
                        for (int k = 0; k < 4; k++) acc += A[i][k] * gp[k][j];
                        t1[i][j] = acc;
                    }
                double t2[2][2] = {{1 - 2 * nO[0][0], 0 - 2 * nO[0][1]}, {0 - 2 * nO[1][0], 1 - 2 * nO[1][1]}};
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 2; j++) {
                        double acc = 0.0;
                        for (int k = 0; k < 2; k++) acc += t1[i][k] * t2[k][j];
                        t3[i][j] = acc;
                    }
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 2; j++) {
                        double acc = 0.0;
                        for (int k = 0; k < 2; k++) acc += gp[i][k] * nO[k][j];
                        bG[i][j] = acc + t3[i][j];
                    }
                double Fv[4];
                diffusiveFlux(cfg->Pr, cfg->mu, qAve, bG, n, Fv);
                for (int k = 0; k < 4; k++) F[k] -= Fv[k];
            }
            memcpy(e->flux, F, sizeof F);
            break;
        }
        case BC_TPINFLOW: {
            for (int k = 0; k < 4; k++) e->q[1][k] = q[e->cellIdx[1]][k];
            double F[4];
            invFlux(cfg->flux, e->q[0], e->q[1], n, F, &e->sMax);
            if (cfg->viscosity) {
                double qAve[4], Fv[4];
                for (int k = 0; k < 4; k++) qAve[k] = 0.5 * (e->q[0][k] + e->q[1][k]);
                diffusiveFlux(cfg->Pr, cfg->mu, qAve, m->cells[e->cellIdx[0]].grad, n, Fv);
                for (int k = 0; k < 4; k++) F[k] -= Fv[k];
            }
            memcpy(e->flux, F, sizeof F);
            break;
        }
        default:
            break;
        }
        if (has_nan4(e->flux) && bb < firstBad) firstBad = bb;
    }
    if (firstBad != INT_MAX) {
        m->errIndex = m->boundaryEdges[firstBad];
        return O_ERR_NAN_EDGE;
    }

    /* interior edges (solve.d:970-1033) */
#pragma omp parallel for schedule(static) reduction(min : firstBad)
    for (int ii = 0; ii < m->nInt; ii++) {
        int ei = m->interiorEdges[ii];
        OEdge *e = &m->edges[ei];
        if (cfg->order == 1) {
            for (int k = 0; k < 4; k++) {
                e->q[0][k] = q[e->cellIdx[0]][k];
                e->q[1][k] = q[e->cellIdx[1]][k];
            }
        } else {
            reconstruct(m, q, e->cellIdx[0], e->mid, e->q[0], 0);
            reconstruct(m, q, e->cellIdx[1], e->mid, e->q[1], 0);
        }
        double F[4];
        invFlux(cfg->flux, e->q[0], e->q[1], e->normal, F, &e->sMax);
        if (cfg->viscosity) {
            double qAve[4], dq[4][2], Fv[4];
            const OCell *g1 = &m->cells[e->cellIdx[0]], *g2 = &m->cells[e->cellIdx[1]];
            for (int k = 0; k < 4; k++) {
                qAve[k] = 0.5 * (e->q[0][k] + e->q[1][k]);
                dq[k][0] = 0.5 * (g1->grad[k][0] + g2->grad[k][0]);
                dq[k][1] = 0.5 * (g1->grad[k][1] + g2->grad[k][1]);
            }
            diffusiveFlux(cfg->Pr, cfg->mu, qAve, dq, e->normal, Fv);
            for (int k = 0; k < 4; k++) F[k] -= Fv[k];
        }
        memcpy(e->flux, F, sizeof F);
        if (has_nan4(e->flux) && ii < firstBad) firstBad = ii;
    }
    if (firstBad != INT_MAX) {
        m->errIndex = m->interiorEdges[firstBad];
        return O_ERR_NAN_EDGE;
    }

    /* residual, dt, Rmax (solve.d:1080-1118) */
    double ndt = INFINITY, rmx = *Rmax;
#pragma omp parallel for schedule(static) reduction(min : ndt) reduction(max : rmx)
    for (int i = 0; i < C; i++) {
        OCell *c = &m->cells[i];
        double r[4] = {0, 0, 0, 0};
        double sAve = 0;
        for (uint32_t j = 0; j < c->nEdges; j++) {
            const OEdge *e = &m->edges[c->edges[j]];
            double ml = c->fluxMultiplier[j] * e->len;
            for (int k = 0; k < 4; k++) r[k] += ml * e->flux[k];
            sAve += e->len * e->sMax;
        }
        sAve /= c->perim;
        ndt = fmin(ndt, (cfg->CFL * c->d) / sAve);
        if (cfg->localTimestep && dtUpdate) {
            c->dt = cfg->CFL * c->d / sAve;
            if (isnan(c->dt)) c->dt = 0;
        }
        for (int k = 0; k < 4; k++)
            if (fabs(r[k]) > rmx) rmx = fabs(r[k]);
        double s = -(1.0 / c->area);
        for (int k = 0; k < 4; k++) R[i][k] = r[k] * s;
    }
    *newDt = ndt;
    *Rmax = rmx;
    return O_OK;
}

/* addSourceTerm (app/ms.d:131-141); the manufactured-solution solver is
   ufvmSolver followed by this. */
static void add_source(OMesh *m, double (*R)[4])
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m->nInterior; i++) {
        double S[4];
        mms_source(m->cfg.mms, m->cells[i].centroid[0], m->cells[i].centroid[1], &m->cfg, S);
        for (int k = 0; k < 4; k++) R[i][k] += S[k];
    }
}

static int solve(OMesh *m, double (*R)[4], double (*q)[4], double *newDt, double *Rmax, int limit, int dtUpdate)
{
    int st = o_solver(m, R, q, newDt, Rmax, limit, dtUpdate);
    if (st) return st;
    if (m->cfg.mms) add_source(m, R);
    return 0;
}

/* one residual evaluation on an external state (length nCells*4), for the parity tests */
int o_residual(OMesh *m, double *q, double *R, double *newDt, double *Rmax, int limit, int dtUpdate)
{
    return solve(m, (double(*)[4])R, (double(*)[4])q, newDt, Rmax, limit, dtUpdate);
}

/* integrators.d: Euler (29-48), RK4 (91-133), RK2_TVD (170-205), RK2 (242-269) */
int o_step(OMesh *m, double *dt, double *Rmax)
{
    const ocfg *cfg = &m->cfg;
    int C = m->nInterior;
    double newDt = INFINITY;
    double (*q)[4] = m->q;
    int st = 0;
    double h = *dt;
    switch (cfg->integrator) {
    case INT_EULER:
        st = solve(m, m->R, q, &newDt, Rmax, 1, 1);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++) {
            double hh = cfg->localTimestep ? m->cells[i].dt : h;
            for (int k = 0; k < 4; k++) q[i][k] = q[i][k] + hh * m->R[i][k];
        }
        break;
    case INT_RK4:
        st = solve(m, m->k1, q, &newDt, Rmax, 1, 1);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++)
            for (int k = 0; k < 4; k++) m->tmp[i][k] = q[i][k] + ((h / 2.0) * m->k1[i][k]);
        st = solve(m, m->k2, m->tmp, &newDt, Rmax, cfg->multistageLimiting, 0);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++)
            for (int k = 0; k < 4; k++) m->tmp[i][k] = q[i][k] + ((h / 2.0) * m->k2[i][k]);
        st = solve(m, m->k3, m->tmp, &newDt, Rmax, cfg->multistageLimiting, 0);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++)
            for (int k = 0; k < 4; k++) m->tmp[i][k] = q[i][k] + (h * m->k3[i][k]);
        st = solve(m, m->k4, m->tmp, &newDt, Rmax, cfg->multistageLimiting, 0);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++) {
            double hh = cfg->localTimestep ? m->cells[i].dt : h;
            for (int k = 0; k < 4; k++)
                q[i][k] = q[i][k] + (hh / 6.0) * (m->k1[i][k] + 2.0 * m->k2[i][k] + 2.0 * m->k3[i][k] + m->k4[i][k]);
        }
        break;
    case INT_RK2_TVD:
        st = solve(m, m->R, q, &newDt, Rmax, 1, cfg->localTimestep);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++) {
            double hh = cfg->localTimestep ? m->cells[i].dt : h;
            for (int k = 0; k < 4; k++) m->qFE[i][k] = q[i][k] + hh * m->R[i][k];
        }
        st = solve(m, m->k2, m->qFE, &newDt, Rmax, 0, !cfg->localTimestep);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++) {
            double hh = cfg->localTimestep ? m->cells[i].dt : h;
            for (int k = 0; k < 4; k++) q[i][k] = 0.5 * (q[i][k] + m->qFE[i][k] + hh * m->k2[i][k]);
        }
        break;
    case INT_RK2:
        st = solve(m, m->k1, q, &newDt, Rmax, 1, 1);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++)
            for (int k = 0; k < 4; k++) m->tmp[i][k] = q[i][k] + (h * m->k1[i][k]);
        st = solve(m, m->k2, m->tmp, &newDt, Rmax, cfg->multistageLimiting, 0);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < C; i++) {
            double hh = cfg->localTimestep ? m->cells[i].dt : h;
            for (int k = 0; k < 4; k++) q[i][k] = q[i][k] + (hh / 2.0) * (m->k1[i][k] + m->k2[i][k]);
        }
        break;
    }
    *dt = newDt;
    return 0;
}

/* runIntegrator loop body (app/solver.d:119-249) for nsteps steps or until t >= tEnd.
   rec (9 doubles per step): t, drag, lift, residRho, residU, residV, residE, Rmax, dt.
   Returns the number of steps run in *done; status 0 or an error code. */
int o_run(OMesh *m, int nsteps, double *rec, int *done)
{
    ocfg *cfg = &m->cfg;
    int C = m->nInterior;
    double aoa = cfg->ic[1] * (M_PI / 180);
    double rot[4] = {cos(aoa), -sin(aoa), sin(aoa), cos(aoa)};
    *done = 0;
    for (int s = 0; s < nsteps && m->t < cfg->tEnd; s++) {
        double Rmax = 0;
        double newDt = m->dt;
        int st = o_step(m, &newDt, &Rmax);
        if (st) return st;
        if (cfg->dynamicDt) m->dt = newDt;
        for (int i = 0; i < C; i++)
            if (isnan(m->q[i][0]) || isnan(m->q[i][1]) || isnan(m->q[i][2]) || isnan(m->q[i][3])) {
                m->errIndex = i;
                return O_ERR_NAN_CELL;
            }
        double resid[4];
        for (int k = 0; k < 4; k++) {
            double ss = 0, vs = 0;
            for (int i = 0; i < C; i++) {
                double d = m->q[i][k] - m->last[k][i];
                ss += d * d;
                vs += m->q[i][k];
            }
            resid[k] = sqrt((double)C * ss) / vs;
        }
        for (int k = 0; k < 4; k++)
            for (int i = 0; i < C; i++) m->last[k][i] = m->q[i][k];
        double f[2] = {0, 0};
        for (int fg = 0; fg < cfg->nForceGroups; fg++) {
            int g = cfg->forceGroups[fg];
            if (g < 0 || g >= m->nGroups) continue;
            for (int j = m->groupEdgeOff[g]; j < m->groupEdgeOff[g + 1]; j++) {
                const OEdge *e = &m->edges[m->groupEdges[j]];
                f[0] += e->flux[1] * e->len;
                f[1] += e->flux[2] * e->len;
            }
        }
        double ld0 = rot[0] * f[0] + rot[1] * f[1];
        double ld1 = rot[2] * f[0] + rot[3] * f[1];
        double residMax = fmax(fmax(resid[0], resid[1]), fmax(resid[2], resid[3]));
        if (cfg->cflAdjust) {
            if (m->residRhoLast < residMax)
                m->residIncIters++;
            else if (m->residIncIters >= 1)
                m->residIncIters--;
            if (m->residIncIters >= 2000) {
                cfg->CFL *= 0.99;
                m->residIncIters = 0;
            }
        }
        m->residRhoLast = residMax;
        double *r = rec + 9 * s;
        r[0] = m->t;
        r[1] = ld0;
        r[2] = ld1;
        r[3] = resid[0];
        r[4] = resid[1];
        r[5] = resid[2];
        r[6] = resid[3];
        r[7] = Rmax;
        r[8] = m->dt;
        m->t += m->dt;
        m->iterations++;
        (*done)++;
    }
    return 0;
}

/* Pseudo-steady manufactured-solution loop (app/ms.d:324-361): forward Euler with the
   source term until max(R) <= tol or maxIter.  Returns iterations; L2 of (q - exact)
   per component (app/ms.d:162-188) in l2[4]. */
long o_ms_converge(OMesh *m, long maxIter, double tol, double *l2, double *rmaxOut)
{
    const ocfg *cfg = &m->cfg;
    int C = m->nInterior;
    double Rmax = -INFINITY, newDt = INFINITY;
    double dt = cfg->dt;
    long it = 0;
    while (fabs(Rmax) > tol && it < maxIter) {
        int st = solve(m, m->R, m->q, &newDt, &Rmax, cfg->limited, 1);
        if (st) return -st;
        for (int i = 0; i < C; i++) {
            double hh = cfg->localTimestep ? m->cells[i].dt : dt;
            for (int k = 0; k < 4; k++) m->q[i][k] = m->q[i][k] + hh * m->R[i][k];
        }
        Rmax = 0;
        for (int i = 0; i < C; i++)
            for (int k = 0; k < 4; k++) Rmax = fmax(m->R[i][k], Rmax);
        dt = newDt;
        it++;
    }
    double s[4] = {0, 0, 0, 0};
    for (int i = 0; i < C; i++) {
        double qe[4];
        mms_solution(cfg->mms, m->cells[i].centroid[0], m->cells[i].centroid[1], qe);
        for (int k = 0; k < 4; k++) {
            double d = fabs(qe[k] - m->q[i][k]);
            s[k] += d * d;
        }
    }
    for (int k = 0; k < 4; k++) l2[k] = sqrt(s[k] / (double)C);
    *rmaxOut = Rmax;
    return it;
}

/* Face states of the last residual evaluation, per interior cell and local edge,
   as written to .esln (io.d:100-134). out: sum(nEdges)*4 doubles in cell order. */
void o_face_states(const OMesh *m, double *out)
{
    size_t o = 0;
    for (int i = 0; i < m->nInterior; i++) {
        const OCell *c = &m->cells[i];
        for (uint32_t j = 0; j < c->nEdges; j++) {
            const OEdge *e = &m->edges[c->edges[j]];
            const double *qq = (e->cellIdx[0] == (uint32_t)i) ? e->q[0] : e->q[1];
            for (int k = 0; k < 4; k++) out[o++] = qq[k];
        }
    }
}

/* Edge fluxes of the last residual evaluation, len * flux per edge in edge order: the
   terms the residual sums (solve.d:1086-1096) and computeBoundaryForces adds up for
   the force tags (mesh.d:645-671).  out: nEdges*4 doubles. */
void o_edge_fluxes(const OMesh *m, double *out)
{
    for (int i = 0; i < m->nEdges; i++)
        for (int k = 0; k < 4; k++) out[4 * i + k] = m->edges[i].flux[k] * m->edges[i].len;
}

/* Gradient and limiter of the last residual evaluation (interior cells). */
void o_grad_lim(const OMesh *m, double *grad, double *lim)
{
    for (int i = 0; i < m->nInterior; i++)
        for (int k = 0; k < 4; k++) {
            grad[8 * i + 2 * k] = m->cells[i].grad[k][0];
            grad[8 * i + 2 * k + 1] = m->cells[i].grad[k][1];
            lim[8 * i + 2 * k] = m->cells[i].lim[k][0];
            lim[8 * i + 2 * k + 1] = m->cells[i].lim[k][1];
        }
}

/* ebb-reconstruct (app/reconstruct.d:79-424): one ufvmSolver evaluation of the current
   state limited as config.limited, without dt update (reconstruct.d:165-176), then the
   refined triangulation's values: node values for the nodes the elements use, in node
   order (interior nodes: the average over the node's elements, in element order, of
   q + lim0*g0*dx + lim1*g1*dy at the node, reconstruct.d:303-324; boundary nodes: the
   average of the values of the boundary edges of those elements that touch the node,
   reconstruct.d:326-346), edge values 0.5*(q[0] + q[1]) in edge order
   (reconstruct.d:290-294), and the cell averages.  out holds (n_nodes_used + nEdges +
   nInterior) x 4 values; sizes[0..2] receive the three counts.  Returns 0, or an error
   status (NaN flux; NaN node value: O_ERR_NAN_CELL with the node index). */
int o_reconstruct(OMesh *m, double *out, int *sizes)
{
    const int C = m->nInterior;
    double newDt = INFINITY, Rmax = 0.0;
    int st = o_solver(m, m->R, m->q, &newDt, &Rmax, m->cfg.limited, 0);
    if (st) return st;
    /* node -> elements (ascending), used nodes, boundary nodes */
    int *cnt = calloc((size_t)m->nNodes + 1, sizeof(int));
    for (int c = 0; c < m->nElem; c++)
        for (int k = m->elemOff[c]; k < m->elemOff[c + 1]; k++) cnt[m->elemNodes[k] - 1 + 1]++;
    for (int n = 0; n < m->nNodes; n++) cnt[n + 1] += cnt[n];
    int *fill = calloc((size_t)m->nNodes, sizeof(int));
    int *ncell = malloc(sizeof(int) * (size_t)(cnt[m->nNodes] > 0 ? cnt[m->nNodes] : 1));
    for (int c = 0; c < m->nElem; c++)
        for (int k = m->elemOff[c]; k < m->elemOff[c + 1]; k++) {
            int n = m->elemNodes[k] - 1;
            ncell[cnt[n] + fill[n]++] = c;
        }
    char *isB = calloc((size_t)m->nNodes, 1);
    for (int b = 0; b < m->nB; b++) {
        isB[m->bNodes[b][0]] = 1;
        isB[m->bNodes[b][1]] = 1;
    }
    double (*ev)[4] = malloc(sizeof(double[4]) * (size_t)(m->nEdges > 0 ? m->nEdges : 1));
    for (int e = 0; e < m->nEdges; e++)
        for (int k = 0; k < 4; k++) ev[e][k] = 0.5 * (m->edges[e].q[0][k] + m->edges[e].q[1][k]);
    int nUsed = 0, status = 0;
    for (int n = 0; n < m->nNodes && !status; n++) {
        int nc = cnt[n + 1] - cnt[n];
        if (nc == 0) continue; /* orphaned node (reconstruct.d:247-268) */
        double v[4] = {0, 0, 0, 0};
        if (!isB[n]) {
            for (int a = cnt[n]; a < cnt[n + 1]; a++) {
                const OCell *c = &m->cells[ncell[a]];
                double dx = m->nodes[n][0] - c->centroid[0];
                double dy = m->nodes[n][1] - c->centroid[1];
                for (int k = 0; k < 4; k++)
                    v[k] += m->q[ncell[a]][k] + c->lim[k][0] * c->grad[k][0] * dx + c->lim[k][1] * c->grad[k][1] * dy;
            }
            for (int k = 0; k < 4; k++) v[k] *= (1.0 / nc);
        } else {
            int ne = 0;
            for (int a = cnt[n]; a < cnt[n + 1]; a++) {
                int ci = ncell[a];
                const OCell *c = &m->cells[ci];
                for (uint32_t j = 0; j < c->nEdges; j++) {
                    int n1 = m->elemNodes[m->elemOff[ci] + (int)j] - 1;
                    int n2 = m->elemNodes[m->elemOff[ci] + (int)((j + 1) % c->nEdges)] - 1;
                    const OEdge *e = &m->edges[c->edges[j]];
                    if (e->isBoundary && (n1 == n || n2 == n)) {
                        for (int k = 0; k < 4; k++) v[k] += ev[c->edges[j]][k];
                        ne++;
                    }
                }
            }
            for (int k = 0; k < 4; k++) v[k] *= (1.0 / ne);
        }
        if (isnan(v[0]) || isnan(v[1]) || isnan(v[2]) || isnan(v[3])) {
            m->errIndex = n;
            status = O_ERR_NAN_CELL;
        }
        for (int k = 0; k < 4; k++) out[4 * nUsed + k] = v[k];
        nUsed++;
    }
    if (!status) {
        memcpy(out + 4 * (size_t)nUsed, ev, sizeof(double[4]) * (size_t)m->nEdges);
        memcpy(out + 4 * ((size_t)nUsed + m->nEdges), m->q, sizeof(double[4]) * (size_t)C);
        sizes[0] = nUsed;
        sizes[1] = m->nEdges;
        sizes[2] = C;
    }
    free(cnt);
    free(fill);
    free(ncell);
    free(isB);
    free(ev);
    return status;
}

/* Thread count of the parallel loops (default 1).  Per-cell and per-edge work is
   independent, min/max reductions are exact, and errors report the first index in
   loop order, so results do not depend on it except for the last bits of the RMS
   residual sums of o_run. */
void o_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

int o_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

/* Faces of the last residual evaluation that took the negative-pressure fallback
   (solve.d:996-1009 interior, solve.d:306-318 boundary). */
void o_fallback_counts(const OMesh *m, long *out)
{
    out[0] = m->nFallback[0];
    out[1] = m->nFallback[1];
}

double o_time(const OMesh *m) { return m->t; }
double o_dt(const OMesh *m) { return m->dt; }
long o_err_index(const OMesh *m) { return m->errIndex; }
