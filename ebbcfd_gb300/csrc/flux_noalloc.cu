// flux_noalloc.cu -- batched face-flux evaluation that allocates no device memory.
//
// ebb_flux stages its host arrays through device buffers it allocates and frees on
// every call.  Some callers cannot do that: a process that shares the GPU with
// running solves (cudaFree synchronises the whole device, stalling every stream the
// solves run on), or one whose device memory is already reserved, e.g. by a request
// server's HBM budget.  This variant stages through one fixed array compiled into the
// library (EBB_FLUX_NOALLOC_MAX faces, 15 doubles per face: 3.75 MiB on every GPU
// that loads the library, held until the process exits).  Compiled with -fmad=false
// like the plain FP64 kernels: results are bitwise those of ebb_flux.
//
// Set-up, once per device on the first call with that device current: the array's
// device address (cudaGetSymbolAddress: in host code the array's name is only a
// stand-in) and a non-blocking stream the copies and the kernel run on.  Every later
// call on the device only copies, launches and waits on that stream.
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
struct DeviceScratch {
    double *base = nullptr;
    cudaStream_t stream = nullptr;
};
DeviceScratch g_dev[kMaxDevices];

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

// The scratch array's device address and the stream of the current device, set up
// on the device's first call (with that device current) and cached.
int scratch_for_current_device(DeviceScratch *out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return EBB_ERR_NO_DEVICE;
    if (dev >= kMaxDevices) return EBB_ERR_LIMIT;
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceScratch &d = g_dev[dev];
    if (!d.base) {
        double *p = nullptr;
        if (cudaGetSymbolAddress((void **)&p, g_flux_scratch) != cudaSuccess || !p) return EBB_ERR_CUDA;
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return EBB_ERR_CUDA;
        d.stream = st;
        d.base = p;
    }
    *out = d;
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
    DeviceScratch d;
    int r = scratch_for_current_device(&d);
    if (r) return r;
    double *base = d.base;
    cudaStream_t st = d.stream;
    cudaError_t e = cudaMemcpyAsync(base, qL, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + 4 * kMax, qR, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + 8 * kMax, normal, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const int T = 128;
        k_flux_scratch<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(kind, n, base);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(F, base + 10 * kMax, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s_max, base + 14 * kMax, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
    // wait for whatever was enqueued, also after a failed enqueue, so that no copy into
    // the caller's buffers is still pending when the call returns
    const cudaError_t w = cudaStreamSynchronize(st);
    return (e == cudaSuccess && w == cudaSuccess) ? EBB_OK : EBB_ERR_CUDA;
}
