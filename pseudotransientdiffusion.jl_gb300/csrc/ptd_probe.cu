// ptd_probe.cu -- the FP64 instruction throughput of the current GPU, the
// roofline of the native-FP64 PT kernels (GB300 runs FP64 at a small fraction
// of its FP32 rate, so those kernels are bound by this number, not by HBM).
//
// Every thread runs 8 independent chains of dependent FP64 FMAs (enough to
// cover the pipe latency), 8 CTAs of 256 threads per SM; the chains' sum is
// written out so the compiler keeps them.  Timed with CUDA events on a private
// stream after one warm-up launch.  No reference counterpart (diagnostic).
#include "../../include/ptd.h"
#include "ptd_internal.h"

namespace ptd {

__global__ void __launch_bounds__(256) dfma_chains_kernel(double* out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace ptd

using namespace ptd;

extern "C" int ptd_measure_fp64_rate(double* ops_per_s)
{
    if (!ops_per_s) return set_error(PTD_EINVAL, "ptd_measure_fp64_rate: NULL output");
    *ops_per_s = 0.0;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    const int blocks = 8 * sms, threads = 256, iters = 4096;
    double* out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = PTD_OK;
    e = cudaMalloc(&out, sizeof(double) * blocks * threads);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        // a = 1 - 2^-30, b = 2^-20: the chains stay finite and normal
        dfma_chains_kernel<<<blocks, threads, 0, s>>>(out, iters, 1.0 - 0x1p-30, 0x1p-20);
        e = cudaEventRecord(e0, s);
    }
    if (e == cudaSuccess) {
        dfma_chains_kernel<<<blocks, threads, 0, s>>>(out, iters, 1.0 - 0x1p-30, 0x1p-20);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) rc = cuda_fail(e, "ptd_measure_fp64_rate");
    else *ops_per_s = (double)blocks * threads * iters * 8 / (ms * 1e-3);
    if (e1) cudaEventDestroy(e1);
    if (e0) cudaEventDestroy(e0);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    return rc;
}
