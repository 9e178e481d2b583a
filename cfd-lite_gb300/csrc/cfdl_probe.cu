// cfdl_probe.cu -- the device's FP64 instruction rate, measured.
//
// The assembly kernels of the outer iteration are bound by the FP64 pipe, not
// by HBM: GB300 issues about two FP64 thread-instructions per SM per clock
// (against 128 FP32).  The roofline of those kernels is therefore their FP64
// instruction count over this rate.  The probe runs independent chains of
// DFMA in every thread of a grid that fills every SM (8 chains a thread, so
// the pipe never waits on a dependency) and times one launch with CUDA
// events after a warm-up launch.
#include "cfdl_internal.h"

namespace {

constexpr int kProbeChains = 8;
constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) k_probe_dfma(double *out, int iters, double a, double b) {
    double x[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; k++) x[k] = 1e-3 * (double)threadIdx.x + (double)k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < kProbeChains; k++) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kProbeChains; k++) s += x[k];
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace

// FP64 FMA thread-instructions per second of the current device.  The
// kernel's sum s of each thread is kept in a device buffer so the chains are
// not optimised away; *fma_per_s receives the rate (multiply by 2 for
// flop/s) and *ms (optional) the timed launch's duration.
extern "C" int cfdl_probe_fp64(double *fma_per_s, double *ms) {
    if (!fma_per_s) return CFDL_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return CFDL_ERR_NO_DEVICE; }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cfdl::cuda_status(e);
    const int blocks = sms * 8, iters = 4096;
    double *buf = nullptr;
    e = cudaMalloc(&buf, (size_t)blocks * kProbeThreads * sizeof(double));
    if (e != cudaSuccess) { cudaGetLastError(); return CFDL_ERR_OOM; }
    cudaStream_t s = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    float elapsed = 0.f;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e == cudaSuccess) {
        k_probe_dfma<<<blocks, kProbeThreads, 0, s>>>(buf, iters, 0.999999, 1e-7);   // warm-up
        cudaEventRecord(t0, s);
        k_probe_dfma<<<blocks, kProbeThreads, 0, s>>>(buf, iters, 0.999999, 1e-7);
        cudaEventRecord(t1, s);
        e = cudaEventSynchronize(t1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&elapsed, t0, t1);
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (s) cudaStreamDestroy(s);
    cudaFree(buf);
    if (e != cudaSuccess) return cfdl::cuda_status(e);
    if (!(elapsed > 0.f)) return CFDL_ERR_CUDA;
    const double fmas = (double)blocks * kProbeThreads * kProbeChains * iters;
    *fma_per_s = fmas / (elapsed * 1e-3);
    if (ms) *ms = elapsed;
    return CFDL_OK;
}
