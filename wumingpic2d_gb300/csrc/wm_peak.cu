// wm_peak.cu -- a measured FP64 rate, the denominator of the FP64 path's roofline.
//
// The FP64 particle kernels are bound by GB300's FP64 pipe, whose rate is far below its FP32 and
// tensor rates and for which no library figure is measured beside the HBM copy and the BF16 GEMM.
// k_fp64_fma runs eight independent dependency chains of fused multiply-adds per thread (enough
// to cover the FMA latency) on a grid of whole waves of the SMs; the rate is the FMAs it issued
// times two flops over its CUDA-event time.
#include "wm_launch.cuh"

namespace {

constexpr int FMA_CHAINS = 8;
constexpr int FMA_THREADS = 256;
__device__ double g_fma_sink;

// x <- x * a + b keeps every chain bounded (|a| < 1) and data-dependent, so nothing is folded.
__global__ void __launch_bounds__(FMA_THREADS) k_fp64_fma(double a, double b, int iters)
{
    double x[FMA_CHAINS];
#pragma unroll
    for (int k = 0; k < FMA_CHAINS; ++k) x[k] = 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < FMA_CHAINS; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < FMA_CHAINS; ++k) s += x[k];
    if (s == -1.0) g_fma_sink = s;  // never true (x > 0 for a, b > 0): keeps the chains live
}

}  // namespace

extern "C" int wm_fp64_fma_rate(double *tflops, double *ms_out)
{
    if (!tflops) return WM_ERR_BAD_ARG;
    int dev = 0, nsm = 0, per_sm = 0;
    WM_CUDA(cudaGetDevice(&dev));
    WM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    WM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_fma, FMA_THREADS, 0));
    const int blocks = nsm * (per_sm > 0 ? per_sm : 1);
    const int iters = 1 << 14;
    cudaStream_t st;
    WM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    WM_CUDA(cudaEventCreate(&e0));
    WM_CUDA(cudaEventCreate(&e1));
    k_fp64_fma<<<blocks, FMA_THREADS, 0, st>>>(0.999999, 1e-7, iters / 8);  // warm-up
    WM_TRY(wm_check_launch("k_fp64_fma"));
    WM_CUDA(cudaEventRecord(e0, st));
    k_fp64_fma<<<blocks, FMA_THREADS, 0, st>>>(0.999999, 1e-7, iters);
    WM_TRY(wm_check_launch("k_fp64_fma"));
    WM_CUDA(cudaEventRecord(e1, st));
    WM_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    WM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    WM_CUDA(cudaEventDestroy(e0));
    WM_CUDA(cudaEventDestroy(e1));
    WM_CUDA(cudaStreamDestroy(st));
    const double fmas = (double)blocks * FMA_THREADS * FMA_CHAINS * iters;
    *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
    return WM_OK;
}
