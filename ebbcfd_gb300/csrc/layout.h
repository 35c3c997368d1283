// layout.h -- device-resident mesh and solver state, shared by host and kernels.
//
// HBM layout (C interior cells in Hilbert-curve order, G ghost cells = boundary edges ordered by
// owner, Eint interior edges sorted by first cell, Cs = C rounded up to 32):
//   state   q64 double[4] per cell (32 B, one sector) = the solution; stage inputs qs1/qs
//           in the arithmetic type T (double: qs1 aliases q64; float: a float[4] shadow),
//           ghosts at [C, C+G)
//   slots   ELL, slot (i, j) at j*Cs + i, j < nedge[i] in the reference's local edge order:
//           nbr int32, edge int32 (bit 31 = fluxMultiplier -1), gm T[2] (gradMat column),
//           nd T[2] (neighbour centroid - centroid), fd T[2] (edge midpoint - centroid),
//           face T[4] (reconstructed face state)
//   edges   slot int32[2], cell int32[2], n T[2], len T; fluxes fl T[4] (len*F) and fs T
//           (len*sMax) for interior edges then boundary edges
//   cells   nedge int32, neg_inv_area, perim, d, src T[4] (manufactured source)
// All geometry is computed on the host in FP64; the split path stores FP32 copies.
#pragma once
#include <stdint.h>

#include "dfloat.h"

#define EBB_NOERR 0xFFFFFFFFFFFFFFFFull
#define EBB_REC_CAP 4096
#define EBB_RED_THREADS 256

// real-valued mesh arrays, in the arithmetic type of a precision form
struct DGeo {
    const void *s_gm, *s_nd, *s_fd;             // T[2] per slot
    const void *neg_inv_area, *perim, *dlen;     // T per cell
    const void *src;                             // T[4] per cell or null
    const void *e_n, *e_len;                     // T[2], T per interior edge
    const void *s_en, *s_elen;                   // split path: T[2], T per slot, a copy of
                                                 // the slot's edge normal and length
    const void *b_n, *b_len;                     // T[2], T per boundary edge
    const void *b_refl, *b_data, *b_dq, *b_dmid; // T[4] per boundary edge
};

struct DMesh {
    int32_t C, G, Cs, Eint, maxJ;
    int32_t uniform;                   // every interior cell has exactly maxJ edges
    const int32_t *nedge;
    const int32_t *s_nbr, *s_edge;
    const int32_t *e_slot, *e_cell;    // int2 per interior edge
    const int32_t *b_cell, *b_slot, *b_type;
    const int32_t *e_ref, *b_ref;      // reference edge ids (error reports)
    const int32_t *cell_ref;           // reference cell id per device cell
    const int32_t *force_b;            // boundary indices summed for forces
    int32_t n_force;
    DGeo g;                            // arrays in the kernels' arithmetic type
    // batched arena of n_inst independent instances (all null when n_inst == 1):
    int32_t n_inst;
    int32_t n_upd_blocks;              // k_update grid size
    const int32_t *cell_inst;          // instance of each interior cell
    const int32_t *blk_first, *blk_end, *blk_inst;  // k_update block -> cell range, instance
    const int32_t *inst_c0;            // n_inst+1 interior-cell offsets
    const int32_t *inst_blk;           // n_inst+1 k_update block offsets
    const int32_t *force_off;          // n_inst+1 offsets into force_b
    const double *inst_mu;             // viscosity per instance
    const float *inst_muf;             // its FP32 rounding (split path)
};

struct DPhys {
    int32_t flux, limited, order, viscous, mms, local_ts, lp;
    double lp_thresh, pr, mu, r_gas;
    int32_t need_grad;  // write raw gradients (viscous terms or viscous walls)
    float prf, muf;     // FP32 roundings of pr and mu: the split kernels read these, so no
                        // thread spends FP64-pipe time converting the doubles
    double gP, c43gP, m1gP, p43mgP, omgP;  // 1.4/pr, -4/3 + gP, -1 + gP, 4/3 - gP, 1 - gP (FP64
                                           // viscous flux constants, rounded once on the host)
    ebbdf::df gPw, c43gPw, m1gPw, p43mgPw, omgPw, muw;  // the same as double-floats (df path)
};

// device-resident scalar state of the time loop
struct DState {
    double dt, t, cfl, t_end;
    double dt_half, dt_sixth;
    unsigned long long newdt_bits;  // atomicMin over non-negative doubles
    unsigned long long rmax_bits;   // atomicMax over non-negative doubles
    unsigned long long err_key;     // atomicMin: (phase << 48) | (code << 40) | index
    double resid_last;
    int32_t resid_inc;
    int32_t done;
    int64_t iter;
    int32_t dynamic_dt, cfl_adjust;
    double rot[4];
    int64_t n_rec;
    int32_t rec_enabled;
    float dtf, dt_half_f, dt_sixth_f;  // FP32 copies for the split path's increments
    int64_t max_steps;                 // > 0: done after this many iterations
    double stop_drop;                  // > 0: done once the density residual <= stop_drop * its first value
    double resid_first;                // density residual of the first iteration (< 0: not yet seen)
    double last[7];                    // drag, lift, resid[4], Rmax of the latest iteration
    float cflf;                        // FP32 rounding of cfl (split path)
    int64_t stall_steps;               // > 0: done once the density residual, after falling at
                                       // least 1000-fold from its first iteration, has made no
                                       // new minimum for this many iterations (a stalled solve)
    int64_t resid_min_iter;            // iteration of the smallest density residual so far
    double resid_min;                  // that residual
    ebbdf::df dtw, dt_half_w;          // double-float copies (the df path's stage states)
};

// dt and what is derived from it: the halves and sixths of the RK stages and their FP32
// (split path) and double-float (df path) copies
EBB_DF_HD void set_step(DState &h, double dt)
{
    h.dt = dt;
    h.dt_half = dt / 2.0;
    h.dt_sixth = dt / 6.0;
    h.dtf = (float)dt;
    h.dt_half_f = (float)h.dt_half;
    h.dt_sixth_f = (float)h.dt_sixth;
    h.dtw = ebbdf::df(dt);
    h.dt_half_w = ebbdf::df(h.dt_half);
}

// record layout matches ebb_step_record
struct DRecord {
    double t, drag, lift, resid[4], rmax, dt, cfl;
};

enum StageKind {
    ST_RESID = 0,  // residual only (ebb_residual): write R
    ST_EULER = 1,
    ST_RK2_1 = 2,
    ST_RK2_2 = 3,
    ST_TVD_1 = 4,
    ST_TVD_2 = 5,
    ST_RK4_1 = 6,
    ST_RK4_2 = 7,
    ST_RK4_3 = 8,
    ST_RK4_4 = 9
};

struct DArrays {
    double *q64;          // solution, FP64, C (+G) x 4
    void *qs1;            // stage-1 input in T (FP64 path: == q64)
    void *qs;             // later-stage input in T
    void *aux;            // k1 / R1 / RK4 accumulator in T
    void *face, *grad, *fl, *fs, *cdt, *R;
    void *lim;            // T[8] per cell (lim[k][0], lim[k][1]) when exported, else null
    double *red;          // per-block partial sums (8 per block)
    DState *st;
    DRecord *rec;
};

#ifdef __cplusplus
extern "C++" {
// launch wrappers; T = double (k_fp64.cu) or float (k_split.cu)
template <typename T>
int launch_cell(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, int limit, void *stream);
template <typename T> int launch_flux(const DMesh &M, const DPhys &P, const DArrays &A, const T *qin, void *stream);
template <typename T>
int launch_update(const DMesh &M, const DPhys &P, const DArrays &A, int stage, const T *qin, T *qout, int dt_update,
                  int need_dt, int final_stage, void *stream);
template <> int launch_cell<double>(const DMesh &, const DPhys &, const DArrays &, const double *, int, void *);
template <> int launch_cell<float>(const DMesh &, const DPhys &, const DArrays &, const float *, int, void *);
template <> int launch_flux<double>(const DMesh &, const DPhys &, const DArrays &, const double *, void *);
template <> int launch_flux<float>(const DMesh &, const DPhys &, const DArrays &, const float *, void *);
template <>
int launch_update<double>(const DMesh &, const DPhys &, const DArrays &, int, const double *, double *, int, int, int,
                          void *);
template <>
int launch_update<float>(const DMesh &, const DPhys &, const DArrays &, int, const float *, float *, int, int, int,
                         void *);
template <> int launch_cell<ebbdf::df>(const DMesh &, const DPhys &, const DArrays &, const ebbdf::df *, int, void *);
template <> int launch_flux<ebbdf::df>(const DMesh &, const DPhys &, const DArrays &, const ebbdf::df *, void *);
template <>
int launch_update<ebbdf::df>(const DMesh &, const DPhys &, const DArrays &, int, const ebbdf::df *, ebbdf::df *, int,
                             int, int, void *);
// precision: EBB_PREC_FP64, EBB_PREC_SPLIT or EBB_PREC_DF (the type of the stored edge fluxes)
int launch_step_end(const DMesh &M, const DArrays &A, int nred_blocks, int precision, void *stream);
// ebb-reconstruct: edge values (reference edge order) and node values
template <typename T>
int launch_recon(const DMesh &M, const DArrays &A, const T *qs, double *edge_out, int n_nodes, const int32_t *off,
                 const int32_t *items, const uint8_t *is_b, const double *nxy, const double *cxy, double *node_out,
                 unsigned long long *err, void *stream);
template <>
int launch_recon<double>(const DMesh &, const DArrays &, const double *, double *, int, const int32_t *,
                         const int32_t *, const uint8_t *, const double *, const double *, double *,
                         unsigned long long *, void *);
template <>
int launch_recon<float>(const DMesh &, const DArrays &, const float *, double *, int, const int32_t *,
                        const int32_t *, const uint8_t *, const double *, const double *, double *,
                        unsigned long long *, void *);
template <>
int launch_recon<ebbdf::df>(const DMesh &, const DArrays &, const ebbdf::df *, double *, int, const int32_t *,
                            const int32_t *, const uint8_t *, const double *, const double *, double *,
                            unsigned long long *, void *);
int update_grid(const DMesh &M);
int launch_flux_batch(int kind, int64_t n, const double *qL, const double *qR, const double *nrm, double *F,
                      double *s, void *stream);
int update_blocks(int C);
// reference-order <-> device-order state copies; conversions for the split path
int launch_permute4(const double *src, double *dst, const int32_t *idx, int64_t n, int gather, void *stream);
int launch_to_float4(const double *src, float *dst, int64_t n, void *stream);
int launch_to_double4(const float *src, double *dst, int64_t n, void *stream);
// q64 (device order) -> its double-float shadow (dst: 4 double-floats per cell)
int launch_to_df4(const double *src, void *dst, int64_t n, void *stream);
int launch_from_df4(const void *src, double *dst, int64_t n, void *stream);
// state in reference order (src, possibly page-locked host memory) -> device order
// q64[iperm[j]] = src[j], plus its FP32 copy when qs1 is given; and back
int launch_load_state(const double *src, double *q64, float *qs1, const int32_t *iperm, int64_t n, void *stream);
int launch_store_state(const double *q64, double *dst, const int32_t *iperm, int64_t n, void *stream);
}
#endif
