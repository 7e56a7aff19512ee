// k_peaks.cu -- the arithmetic rates the FP64 path's roofline is quoted against.
//
// The plain FP64 drop-in is bound by the FP64 pipe, not by HBM (GB300 issues FP64
// at a small fraction of its FP32 rate), so its roofline denominator is the
// device's own DFMA rate, measured here: every thread runs 8 independent FMA
// chains (no dependency stalls at full occupancy) over a grid of 4 CTAs of 256
// threads per SM, timed with CUDA events, best of 5 launches.  The FP32 FFMA
// rate is measured the same way for comparison.  No counterpart in the
// reference (it reports no rates).
#include <cuda_runtime.h>

#include <string>

#include "clv_internal.cuh"

namespace clv {
int record_failure(int status, const std::string &msg);
}

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <class T>
__global__ void __launch_bounds__(256) fma_rate_kernel(T *sink, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = (T)(threadIdx.x + c);
#pragma unroll 4
    for (int i = 0; i < kIters; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == (T)-1.2345) sink[blockIdx.x] = s;  // never true for the inputs below; keeps the chains live
}

template <class T>
int measure(int sms, double *tflops) {
    T *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t rc = cudaMalloc(&sink, sizeof(T) * 4 * sms);
    if (rc == cudaSuccess) rc = cudaEventCreate(&e0);
    if (rc == cudaSuccess) rc = cudaEventCreate(&e1);
    float best = 0.f;
    const int grid = 4 * sms;
    for (int rep = 0; rep < 6 && rc == cudaSuccess; ++rep) {
        cudaEventRecord(e0);
        fma_rate_kernel<T><<<grid, 256>>>(sink, (T)0.999999, (T)1e-7);
        cudaEventRecord(e1);
        rc = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (rc == cudaSuccess) rc = cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
    }
    if (sink) cudaFree(sink);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc != cudaSuccess)
        return clv::record_failure(CLV_ERR_CUDA, std::string("clv_measure_peaks: ") + cudaGetErrorString(rc));
    const double flops = 2.0 * kChains * (double)kIters * 256.0 * grid;
    *tflops = flops / (best * 1e-3) / 1e12;
    return CLV_OK;
}

}  // namespace

extern "C" int clv_measure_peaks(int device, double *fp64_tflops, double *fp32_tflops) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess)
        return clv::record_failure(CLV_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int rc = CLV_OK;
    if (fp64_tflops) rc = measure<double>(sms, fp64_tflops);
    if (rc == CLV_OK && fp32_tflops) rc = measure<float>(sms, fp32_tflops);
    cudaSetDevice(prev);
    return rc;
}
