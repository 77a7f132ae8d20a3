// FP64 pipe rate of the current GPU, measured with independent fused multiply-add chains.
//
// The FP64 ("plain") step kernel is bound by the FP64 pipe on GB300 rather than by HBM, so
// its roofline needs this GPU's FP64 rate; the peaks the bench reads hold only a copy
// bandwidth and a bf16 GEMM rate.  Each thread runs CHAINS independent dependency chains of
// `fma(a, b, c)` (CHAINS x ITERS DFMA, 2 flops each), enough warps per SM to hide the pipe's
// latency; the result is the best of three CUDA-event-timed launches.
#include "../../include/csadv.h"
#include "internal.h"

namespace csadv {

constexpr int PK_CHAINS = 8;
constexpr int PK_THREADS = 256;
constexpr int PK_BLOCKS_PER_SM = 8;

__global__ void __launch_bounds__(PK_THREADS) k_dfma_rate(int iters, double b, double c, double *sink) {
    double a[PK_CHAINS];
#pragma unroll
    for (int k = 0; k < PK_CHAINS; ++k) a[k] = 1e-3 * (threadIdx.x + 1) + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < PK_CHAINS; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < PK_CHAINS; ++k) s += a[k];
    if (s == -1.0) sink[0] = s;  // the chains stay positive: keeps them live without a store
}

}  // namespace csadv

using namespace csadv;

extern "C" int csadv_fp64_rate(int iters, double *flops_per_s, void *stream) {
    if (!flops_per_s || iters < 1 || iters > (1 << 24)) return CSADV_ERR_ARG;
    *flops_per_s = 0.0;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    CSADV_CUDA(cudaGetDevice(&dev));
    CSADV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) {
        (void)cudaGetLastError();
        return CSADV_ERR_OOM;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = CSADV_OK;
    const int blocks = sms * PK_BLOCKS_PER_SM;
    const double flops = 2.0 * PK_CHAINS * (double)iters * blocks * PK_THREADS;
    float best = 0.f;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = cuda_fail(cudaGetLastError(), "cudaEventCreate", __FILE__, __LINE__);
    } else {
        k_dfma_rate<<<blocks, PK_THREADS, 0, st>>>(iters, 0.9999999, 1e-7, sink);  // warm-up
        for (int r = 0; r < 3 && rc == CSADV_OK; ++r) {
            cudaEventRecord(e0, st);
            k_dfma_rate<<<blocks, PK_THREADS, 0, st>>>(iters, 0.9999999, 1e-7, sink);
            cudaEventRecord(e1, st);
            cudaError_t e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "k_dfma_rate", __FILE__, __LINE__);
            } else if (best == 0.f || ms < best) {
                best = ms;
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    if (rc == CSADV_OK && best > 0.f) *flops_per_s = flops / (best * 1e-3);
    return rc;
}
