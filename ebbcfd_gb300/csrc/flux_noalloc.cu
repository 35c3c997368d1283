// flux_noalloc.cu -- batched face-flux evaluation that allocates no device memory.
//
// ebb_flux stages its host arrays through device buffers it allocates on every call.
// This variant stages them through one fixed array compiled into the library
// (EBB_FLUX_NOALLOC_MAX faces, 15 doubles per face: 3.75 MiB on every GPU that loads
// the library, held until the process exits), so a caller that cannot allocate
// device memory at call time can still evaluate fluxes.  Compiled with -fmad=false
// like the plain FP64 kernels: results are bitwise those of ebb_flux.
//
// The array is shared by every call on a device and keeps the last call's contents;
// each call overwrites the whole region it reads, so nothing needs clearing.  Calls
// that overlap on the same GPU (several host threads) race on it: serialise them.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ebb_gb300.h"
#include "kernels.cuh"

namespace {

constexpr int64_t kMax = EBB_FLUX_NOALLOC_MAX;
constexpr int kMaxDevices = 64;
// per face: qL 4, qR 4, normal 2, F 4, sMax 1 (region offsets in units of kMax)
__device__ __align__(256) double g_flux_scratch[15 * EBB_FLUX_NOALLOC_MAX];

std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {};

__global__ void k_flux_scratch(int kind, int64_t n, double *base)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *qL = base, *qR = base + 4 * kMax, *nrm = base + 8 * kMax;
    double *F = base + 10 * kMax, *s = base + 14 * kMax;
    double a[4], b[4], f[4], sm;
    ebbdev::ld4(qL + 4 * i, a);
    ebbdev::ld4(qR + 4 * i, b);
    ebbdev::inviscid_flux(kind, a, b, nrm[2 * i], nrm[2 * i + 1], f, sm);
    ebbdev::st4(F + 4 * i, f);
    s[i] = sm;
}

// Device address of the scratch array on the current device: the host-side symbol
// is only a stand-in, so the address is looked up once per device with that device
// current and cached.
int scratch_for_current_device(double **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return EBB_ERR_NO_DEVICE;
    if (dev >= kMaxDevices) return EBB_ERR_LIMIT;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        if (cudaGetSymbolAddress((void **)&p, g_flux_scratch) != cudaSuccess || !p) return EBB_ERR_CUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return EBB_OK;
}

}  // namespace

extern "C" int ebb_flux_noalloc(int32_t kind, int64_t n, const double *qL, const double *qR, const double *normal,
                                double *F, double *s_max)
{
    if (n < 0 || (n && (!qL || !qR || !normal || !F || !s_max))) return EBB_ERR_ARG;
    if (n > kMax) return EBB_ERR_LIMIT;
    if (n == 0) return EBB_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return EBB_ERR_NO_DEVICE;
    double *base = nullptr;
    int r = scratch_for_current_device(&base);
    if (r) return r;
    cudaError_t e = cudaMemcpy(base, qL, sizeof(double) * 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(base + 4 * kMax, qR, sizeof(double) * 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(base + 8 * kMax, normal, sizeof(double) * 2 * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return EBB_ERR_CUDA;
    const int T = 128;
    k_flux_scratch<<<(unsigned)((n + T - 1) / T), T>>>(kind, n, base);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(F, base + 10 * kMax, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(s_max, base + 14 * kMax, sizeof(double) * n, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? EBB_OK : EBB_ERR_CUDA;
}
