// k_peak.cu -- the FP64 pipe's rate on this device, measured: the denominator of the element
// pass's FP64 roofline (the pass is bound by FP64 instruction issue, not by HBM, on GB300).
//
// Every thread runs eight independent chains of dependent fused multiply-adds (a fixed point
// of x -> x a + b with |a| < 1, so the values stay finite); 16 warps per SM keep every SM's
// FP64 pipe fed. The rate is the executed DFMA warp instructions (and FLOPs, two per lane
// per DFMA) over the kernel's CUDA-event duration, best of a few launches after a warm-up.
#include "nf_internal.h"

namespace nf {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_BLOCKS_PER_SM = 2;
constexpr int PEAK_CHAINS = 8;

__global__ void __launch_bounds__(PEAK_THREADS) k_dfma_rate(double *out, int iters, double a,
                                                            double b) {
    double x[PEAK_CHAINS];
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) x[c] = (double)(threadIdx.x + c) * 1.0e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < PEAK_CHAINS; c++) x[c] = fma(x[c], a, b);
    }
    double t = 0.0;
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; c++) t += x[c];
    out[blockIdx.x * PEAK_THREADS + threadIdx.x] = t;
}

}  // namespace nf

using namespace nf;

extern "C" nf_status nf_device_fp64_rate(double *warp_instructions_per_second,
                                         double *flops_per_second) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms < 1) {
        (void)cudaGetLastError();
        set_thread_error("no usable CUDA device");
        return NF_EDEVICE;
    }
    const int blocks = sms * PEAK_BLOCKS_PER_SM;
    const int iters = 1 << 16;
    double *out = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float best = 0.0f;
    cudaError_t e = cudaMalloc(&out, sizeof(double) * (size_t)blocks * PEAK_THREADS);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(e0, st);
        k_dfma_rate<<<blocks, PEAK_THREADS, 0, st>>>(out, iters, 0.999999, 1.0e-6);
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (out) cudaFree(out);
    if (e != cudaSuccess || !(best > 0.0f)) {
        (void)cudaGetLastError();
        set_thread_error(e != cudaSuccess ? cudaGetErrorString(e) : "no duration measured");
        return NF_EDEVICE;
    }
    const double warpInst = (double)blocks * (PEAK_THREADS / 32) * (double)iters * PEAK_CHAINS;
    const double seconds = best * 1.0e-3;
    if (warp_instructions_per_second) *warp_instructions_per_second = warpInst / seconds;
    if (flops_per_second) *flops_per_second = warpInst * 32.0 * 2.0 / seconds;
    return NF_OK;
}
