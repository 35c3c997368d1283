// k_fp64.cu -- plain FP64 instantiation of the stage kernels, plus the time-loop
// epilogue, the flux seam and the state copy kernels (sm_103a).
//
// Compiled with -fmad=false: every multiply and add rounds separately, in the
// reference's left-to-right order, so results are bitwise those of the FP64 CPU
// path (up to the sign of exact zeros) except where CUDA's pow() is used
// (constant-pressure ghost states).
#include "../../include/ebb_gb300.h"
#include "kernels.cuh"

EBB_INSTANTIATE(double)

using namespace ebbdev;

namespace {

// end of one runIntegrator iteration (app/solver.d:126-249), one block; FP64 sums in
// a fixed tree order
template <typename T> __global__ void __launch_bounds__(EBB_RED_THREADS) k_step_end(DMesh M, DArrays A, int nblk)
{
    // one block per instance
    const int inst = blockIdx.x;
    DState *st = A.st + inst;
    const int b0 = M.inst_blk ? M.inst_blk[inst] : 0, b1 = M.inst_blk ? M.inst_blk[inst + 1] : nblk;
    const int fb0 = M.force_off ? M.force_off[inst] : 0, fb1 = M.force_off ? M.force_off[inst + 1] : M.n_force;
    const int ncell = M.inst_c0 ? M.inst_c0[inst + 1] - M.inst_c0[inst] : M.C;
    grid_dep_release();
    grid_dep_wait();
    if (st->done) return;
    if (st->err_key != EBB_NOERR) {
        if (threadIdx.x == 0) st->done = 1;
        return;
    }
    __shared__ double sh[EBB_RED_THREADS][10];
    double s[10];
    for (int k = 0; k < 10; k++) s[k] = 0.0;
    for (int b = b0 + threadIdx.x; b < b1; b += EBB_RED_THREADS)
        for (int k = 0; k < 8; k++) s[k] = s[k] + A.red[8 * (size_t)b + k];
    const T *fl = reinterpret_cast<const T *>(A.fl);
    for (int f = fb0 + threadIdx.x; f < fb1; f += EBB_RED_THREADS) {
        const size_t e = (size_t)M.Eint + M.force_b[f];
        s[8] = s[8] + (double)fl[4 * e + 1];
        s[9] = s[9] + (double)fl[4 * e + 2];
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
    for (int k = 0; k < 4; k++) resid[k] = sqrt((double)ncell * sh[0][k]) / sh[0][4 + k];
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
            st->cflf = (float)st->cfl;
            st->resid_inc = 0;
        }
    }
    st->resid_last = residMax;
    if (st->resid_first < 0) st->resid_first = resid[0];
    if (resid[0] < st->resid_min) {
        st->resid_min = resid[0];
        st->resid_min_iter = st->iter;
    }
    st->last[0] = drag;
    st->last[1] = lift;
    for (int k = 0; k < 4; k++) st->last[2 + k] = resid[k];
    st->last[6] = rmax;
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
    st->done = !(st->t < st->t_end) || (st->max_steps > 0 && st->iter >= st->max_steps) ||
               (st->stop_drop > 0 && resid[0] <= st->stop_drop * st->resid_first) ||
               (st->stall_steps > 0 && st->resid_min <= 1e-3 * st->resid_first &&
                st->iter - st->resid_min_iter > st->stall_steps);
    set_step(*st, st->dt);
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

__global__ void k_to_float4(const double *__restrict__ src, float *__restrict__ dst, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    ld4(src + 4 * i, v);
    float f[4] = {(float)v[0], (float)v[1], (float)v[2], (float)v[3]};
    st4(dst + 4 * i, f);
}

__global__ void k_to_double4(const float *__restrict__ src, double *__restrict__ dst, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float f[4];
    ld4(src + 4 * i, f);
    double v[4] = {(double)f[0], (double)f[1], (double)f[2], (double)f[3]};
    st4(dst + 4 * i, v);
}

// State in and out in the caller's cell order.  The reference-order side is read or
// written in sequence (the device side through the inverse permutation), so when it
// is a page-locked host buffer the link carries whole contiguous lines.
__global__ void k_load_state(const double *__restrict__ src, double *__restrict__ q64, float *__restrict__ qs1,
                             const int32_t *__restrict__ iperm, int64_t n)
{
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double v[4];
    ld4(src + 4 * j, v);
    const size_t i = (size_t)iperm[j];
    st4(q64 + 4 * i, v);
    if (qs1) {
        float f[4] = {(float)v[0], (float)v[1], (float)v[2], (float)v[3]};
        st4(qs1 + 4 * i, f);
    }
}

__global__ void k_store_state(const double *__restrict__ q64, double *__restrict__ dst,
                              const int32_t *__restrict__ iperm, int64_t n)
{
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double v[4];
    ld4(q64 + 4 * (size_t)iperm[j], v);
    st4(dst + 4 * j, v);
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int update_blocks(int C) { return (C + UPD_THREADS - 1) / UPD_THREADS; }

int update_grid(const DMesh &M) { return M.n_upd_blocks; }

int launch_step_end(const DMesh &M, const DArrays &A, int nred_blocks, int precision, void *stream)
{
    const int n = M.n_inst > 0 ? M.n_inst : 1;
    cudaError_t e;
    if (precision == EBB_PREC_SPLIT)
        e = launch_dep(k_step_end<float>, dim3(n), dim3(EBB_RED_THREADS), (cudaStream_t)stream, M, A, nred_blocks);
    else if (precision == EBB_PREC_DF)
        e = launch_dep(k_step_end<ebbdf::df>, dim3(n), dim3(EBB_RED_THREADS), (cudaStream_t)stream, M, A, nred_blocks);
    else
        e = launch_dep(k_step_end<double>, dim3(n), dim3(EBB_RED_THREADS), (cudaStream_t)stream, M, A, nred_blocks);
    return ret(e);
}

int launch_flux_batch(int kind, int64_t n, const double *qL, const double *qR, const double *nrm, double *F, double *s,
                      void *stream)
{
    if (n <= 0) return 0;
    k_flux_batch<<<nblk(n, 128), 128, 0, (cudaStream_t)stream>>>(kind, n, qL, qR, nrm, F, s);
    return ret(cudaGetLastError());
}

int launch_permute4(const double *src, double *dst, const int32_t *idx, int64_t n, int gather, void *stream)
{
    if (n <= 0) return 0;
    k_permute4<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(src, dst, idx, n, gather);
    return ret(cudaGetLastError());
}

int launch_to_float4(const double *src, float *dst, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    k_to_float4<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(src, dst, n);
    return ret(cudaGetLastError());
}

int launch_to_double4(const float *src, double *dst, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    k_to_double4<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(src, dst, n);
    return ret(cudaGetLastError());
}

int launch_load_state(const double *src, double *q64, float *qs1, const int32_t *iperm, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    k_load_state<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(src, q64, qs1, iperm, n);
    return ret(cudaGetLastError());
}

int launch_store_state(const double *q64, double *dst, const int32_t *iperm, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    k_store_state<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>(q64, dst, iperm, n);
    return ret(cudaGetLastError());
}
