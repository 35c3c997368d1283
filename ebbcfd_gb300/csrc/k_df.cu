// k_df.cu -- double-float instantiation of the stage kernels (sm_103a): face, flux,
// gradient and limiter arithmetic on (hi, lo) pairs of FP32 numbers (dfloat.h, ~46
// significant bits) on the FP32 pipe, which GB300 runs at 64 times its FP64 rate; the
// solution update and the reductions inside k_update run in FP64 as on the plain path.
// Compiled with IEEE FP32 division and square root and FP32 denormals kept: the
// double-word algorithms need every FP32 operation correctly rounded.
#include "kernels.cuh"

EBB_INSTANTIATE(ebbdf::df)

namespace {

// q64 (FP64, device order) -> its double-float shadow
__global__ void k_to_df4(const double *__restrict__ src, ebbdf::df *__restrict__ dst, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[4];
    ebbdev::ld4(src + 4 * i, v);
    const ebbdf::df w[4] = {ebbdf::df(v[0]), ebbdf::df(v[1]), ebbdf::df(v[2]), ebbdf::df(v[3])};
    ebbdev::st4(dst + 4 * i, w);
}

}  // namespace

int launch_to_df4(const double *src, void *dst, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    k_to_df4<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(src, reinterpret_cast<ebbdf::df *>(dst), n);
    return ebbdev::ret(cudaGetLastError());
}

namespace {

// double-floats -> doubles (4 per item), e.g. a residual evaluated on the df path
__global__ void k_from_df4(const ebbdf::df *__restrict__ src, double *__restrict__ dst, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ebbdf::df w[4];
    ebbdev::ld4(src + 4 * i, w);
    const double v[4] = {(double)w[0], (double)w[1], (double)w[2], (double)w[3]};
    ebbdev::st4(dst + 4 * i, v);
}

}  // namespace

int launch_from_df4(const void *src, double *dst, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    k_from_df4<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const ebbdf::df *>(src), dst, n);
    return ebbdev::ret(cudaGetLastError());
}
