// layout.h -- device-resident mesh and solver state, shared by host and kernels.
//
// HBM layout (C interior cells in RCM order, G ghost cells = boundary edges ordered by
// owner, Eint interior edges sorted by first cell, Cs = C rounded up to 32):
//   state   q, qs, aux           double[4] per cell (32 B, one sector), ghosts at [C, C+G)
//   slots   ELL, slot (i, j) at j*Cs + i, j < nedge[i] in the reference's local edge order:
//           nbr int32, edge int32 (bit 31 = fluxMultiplier -1), gm double[2] (gradMat
//           column), nd double[2] (neighbour centroid - centroid), fd double[2] (edge
//           midpoint - centroid), face double[4] (reconstructed face state)
//   edges   slot int32[2], cell int32[2], n double[2], len double; fluxes fl double[4]
//           (len*F) and fs double (len*sMax) for interior edges then boundary edges
//   cells   nedge int32, neg_inv_area, perim, d, src double[4] (manufactured source)
#pragma once
#include <stdint.h>

#define EBB_NOERR 0xFFFFFFFFFFFFFFFFull
#define EBB_REC_CAP 4096
#define EBB_RED_THREADS 256

struct DMesh {
    int32_t C, G, Cs, Eint, maxJ;
    const int32_t *nedge;
    const int32_t *s_nbr, *s_edge;
    const double *s_gm, *s_nd, *s_fd;  // double2 per slot
    const double *neg_inv_area, *perim, *dlen, *src;  // src: double4 per cell or null
    const int32_t *e_slot, *e_cell;    // int2 per interior edge
    const double *e_n, *e_len;         // double2, double
    const int32_t *b_cell, *b_slot, *b_type;
    const double *b_n, *b_len;         // double2, double
    const double *b_refl;              // double4: reflection matrix (r00, r01, r10, r11)
    const double *b_data;              // double4: FullState q_inf | ConstP pb | TPInflow Tt, Pt, nin0, nin1
    const double *b_dq, *b_dmid;       // double4: Dirichlet state at ghost centroid / edge midpoint
    const int32_t *e_ref, *b_ref;      // reference edge ids (error reports)
    const int32_t *cell_ref;           // reference cell id per device cell
    const int32_t *force_b;            // boundary indices summed for forces
    int32_t n_force;
};

struct DPhys {
    int32_t flux, limited, order, viscous, mms, local_ts, lp;
    double lp_thresh, pr, mu, r_gas;
    int32_t need_grad;  // write raw gradients (viscous terms or viscous walls)
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
    int32_t pad;
};

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
    double *q, *qs, *aux, *face, *grad, *fl, *fs, *cdt, *R;
    double *red;  // per-block partial sums (8 per block)
    DState *st;
    DRecord *rec;
};

#ifdef __cplusplus
extern "C++" {
// launch wrappers (k_fp64.cu)
int launch_cell_fp64(const DMesh &M, const DPhys &P, const DArrays &A, const double *qin, double *qin_ghost_out,
                     int limit, void *stream);
int launch_flux_fp64(const DMesh &M, const DPhys &P, const DArrays &A, const double *qin, void *stream);
int launch_update_fp64(const DMesh &M, const DPhys &P, const DArrays &A, int stage, const double *qin, double *qout,
                       int dt_update, int need_dt, int final_stage, void *stream);
int launch_step_end(const DMesh &M, const DArrays &A, int nred_blocks, void *stream);
int launch_flux_batch(int kind, int64_t n, const double *qL, const double *qR, const double *nrm, double *F,
                      double *s, void *stream);
int update_blocks(int C);
}
#endif

#ifdef __cplusplus
extern "C++" {
// reference-order <-> device-order state copies (k_fp64.cu)
int launch_permute4(const double *src, double *dst, const int32_t *idx, int64_t n, int gather, void *stream);
}
#endif
