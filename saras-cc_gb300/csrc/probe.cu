// Measurement entry point: the FP64 instruction rate of this GPU, the
// denominator of the FP64 form's arithmetic roofline.  Every thread of a
// full-occupancy grid runs eight independent dependency chains, either of
// fused multiply-adds or of separately rounded adds and multiplies (the
// operations the reference-order arithmetic uses), so the FP64 pipe, not
// latency, sets the rate.  The chains converge to a fixed point (b < 1), and
// their sum is compared with a value they never reach, so the compiler keeps
// every operation and nothing is stored.
#include <cuda_runtime.h>

#include "common.cuh"

namespace {

constexpr int PROBE_CHAINS = 8;
constexpr int PROBE_THREADS = 256;

__global__ void __launch_bounds__(PROBE_THREADS) k_fp64_fma_chains(double *sink, int iters, double b, double c) {
    double a[PROBE_CHAINS];
#pragma unroll
    for (int q = 0; q < PROBE_CHAINS; q++) a[q] = 1e-3 * (threadIdx.x + q);
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int q = 0; q < PROBE_CHAINS; q++) a[q] = __fma_rn(a[q], b, c);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < PROBE_CHAINS; q++) s += a[q];
    if (s == -1.0) sink[0] = s;  // never true: the chains stay positive
}

__global__ void __launch_bounds__(PROBE_THREADS) k_fp64_addmul_chains(double *sink, int iters, double b, double c) {
    double a[PROBE_CHAINS];
#pragma unroll
    for (int q = 0; q < PROBE_CHAINS; q++) a[q] = 1e-3 * (threadIdx.x + q);
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int q = 0; q < PROBE_CHAINS; q++) a[q] = __dmul_rn(__dadd_rn(a[q], c), b);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < PROBE_CHAINS; q++) s += a[q];
    if (s == -1.0) sink[0] = s;
}

}  // namespace

extern "C" saras_status saras_measure_fp64_rate(void *stream, double *fma_per_s, double *addmul_per_s) {
    if (!fma_per_s || !addmul_per_s) {
        saras::set_error("null argument");
        return SARAS_BAD_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0, per_sm = 0;
    SARAS_CUDA(cudaGetDevice(&dev));
    SARAS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SARAS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_fma_chains, PROBE_THREADS, 0));
    const int blocks = sms * (per_sm > 0 ? per_sm : 1);
    const int iters = 4096;
    double *sink = nullptr;
    SARAS_CUDA(cudaMalloc(&sink, sizeof(double)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    saras_status st = SARAS_OK;
    float ms[2] = {0.f, 0.f};
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        st = SARAS_CUDA_ERR;
    } else {
        for (int kind = 0; kind < 2 && st == SARAS_OK; kind++) {
            for (int rep = 0; rep < 2; rep++) {  // the first launch warms up
                cudaEventRecord(e0, s);
                if (kind == 0)
                    k_fp64_fma_chains<<<blocks, PROBE_THREADS, 0, s>>>(sink, iters, 0.9999999, 1e-7);
                else
                    k_fp64_addmul_chains<<<blocks, PROBE_THREADS, 0, s>>>(sink, iters, 0.9999999, 1e-7);
                cudaEventRecord(e1, s);
            }
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms[kind], e0, e1) != cudaSuccess)
                st = SARAS_CUDA_ERR;
        }
    }
    const double ops = (double)blocks * PROBE_THREADS * PROBE_CHAINS * iters;
    if (st == SARAS_OK && ms[0] > 0.f && ms[1] > 0.f) {
        *fma_per_s = ops / (ms[0] * 1e-3);
        *addmul_per_s = 2.0 * ops / (ms[1] * 1e-3);
    } else if (st == SARAS_OK) {
        st = SARAS_CUDA_ERR;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    if (st != SARAS_OK) {
        cudaGetLastError();
        saras::set_error("FP64 rate measurement failed");
    }
    return st;
}
