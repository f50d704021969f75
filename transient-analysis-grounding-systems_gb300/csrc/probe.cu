// FP64 throughput probes (diagnostic entry point tags_probe_fp64): the rates
// of the two FP64 paths the plain form could use, measured on the device the
// library runs on, so that the plain form's roofline has a measured
// denominator and the choice between them (k_gemm_update<double2> runs on
// DFMA) rests on numbers taken here:
//   * DFMA: eight independent FMA chains per thread on the CUDA cores;
//   * DMMA: four independent accumulators per warp of mma.sync m8n8k4 f64 on
//     the FP64 tensor path (512 flops per warp instruction).
// Each probe is timed with CUDA events over a launch of some tens of ms; the
// best of three launches (after one warm-up launch) is kept.
#include <cuda_runtime.h>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

constexpr int PROBE_THREADS = 256;

__global__ void __launch_bounds__(PROBE_THREADS) k_probe_dfma(double* out, int iters, double mul, double add) {
    double a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = 1.0 + 1e-3 * (threadIdx.x + j);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fma(a[j], mul, add);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == 123.456) out[0] = s;          // keeps the chains live; never true for these inputs
}

__global__ void __launch_bounds__(PROBE_THREADS) k_probe_dmma(double* out, int iters) {
    const double a = 1.0 + 1e-6 * threadIdx.x, b = 1.0 - 1e-6 * threadIdx.x;
    double c[4][2];
#pragma unroll
    for (int q = 0; q < 4; ++q) c[q][0] = c[q][1] = 0.0;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(c[q][0]), "+d"(c[q][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1];
    if (s == 123.456) out[0] = s;
}

}  // namespace

extern "C" int tags_probe_fp64(double* dfma_tflops, double* dmma_tflops) {
    if (!dfma_tflops || !dmma_tflops) return tags_fail(TAGS_E_ARG, "tags_probe_fp64: null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    int sms = 0;
    TAGS_CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    // the probes never store (their sums cannot equal the test value); the
    // pointer only keeps the chains from being optimised away
    double* d_out = reinterpret_cast<double*>(c->scratch(15, sizeof(double)));
    if (!d_out) return tags_fail(TAGS_E_NOMEM, "tags_probe_fp64: scratch allocation failed");
    cudaStream_t st = c->stream;
    cudaEvent_t e0, e1;
    TAGS_CUDA_OK(cudaEventCreate(&e0));
    TAGS_CUDA_OK(cudaEventCreate(&e1));
    const int blocks = 8 * sms;
    double best[2] = {0.0, 0.0};
    int err = 0;
    for (int kind = 0; kind < 2 && !err; ++kind) {
        const int iters = kind == 0 ? 8192 : 4096;
        for (int rep = 0; rep < 4; ++rep) {
            cudaError_t ce = cudaEventRecord(e0, st);
            if (kind == 0) k_probe_dfma<<<blocks, PROBE_THREADS, 0, st>>>(d_out, iters, 0.9999999, 1e-9);
            else k_probe_dmma<<<blocks, PROBE_THREADS, 0, st>>>(d_out, iters);
            if (ce == cudaSuccess) ce = cudaGetLastError();
            if (ce == cudaSuccess) ce = cudaEventRecord(e1, st);
            if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
            if (ce != cudaSuccess) {
                err = tags_fail_cuda(ce, "tags_probe_fp64", __FILE__, __LINE__);
                break;
            }
            const double threads = (double)blocks * PROBE_THREADS;
            const double flops = kind == 0 ? threads * iters * 8.0 * 2.0 : threads / 32.0 * iters * 4.0 * 512.0;
            const double tf = flops / (1e-3 * ms) / 1e12;
            if (rep > 0 && tf > best[kind]) best[kind] = tf;
        }
    }
    tags_note_launch(8);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err) return err;
    *dfma_tflops = best[0];
    *dmma_tflops = best[1];
    return 0;
}
