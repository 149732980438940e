// Measured FP32 FMA throughput of the GPU, the denominator of the pruning
// kernel's roofline.
//
// The fused pruning kernel keeps every conditional likelihood on chip, so HBM
// does not bound it; FP32 issue does.  Nominal figures assume the maximum SM
// clock, which a power- or thermally-limited part may not hold, so the bench
// measures the rate instead: a grid of 4 blocks of 256 threads per SM, each
// thread running 8 independent FMA chains (enough independent work to cover
// the FMA pipe's latency), timed with CUDA events on the library's stream.
// No reference counterpart.
#include <cuda_runtime.h>
#include "p4g_internal.h"

namespace p4g {

namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;

__global__ void __launch_bounds__(256) k_fmaPeak(float *sink, int iters, float seed)
{
    float a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = seed + 1e-3f * (float)(threadIdx.x + c);
    const float b = 0.9999f, d = 1e-4f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < kUnroll; u++) {
#pragma unroll
            for (int c = 0; c < kChains; c++) a[c] = __fmaf_rn(a[c], b, d);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += a[c];
    // never true for these inputs; keeps the chains live
    if (s == 1234567.0f) sink[0] = s;
}

}  // namespace

}  // namespace p4g

using namespace p4g;

#define RET(call)                      \
    do {                               \
        int rc_ = (call);              \
        if (rc_ != P4G_OK) return rc_; \
    } while (0)

extern "C" int p4g_fp32FmaPeak(int iters, double *tflops, double *ms)
{
    if (!tflops || !ms || iters <= 0) return setError(P4G_EINVAL, "fp32FmaPeak: bad arguments");
    RET(ensureCtx());
    static DevBuf sink;
    RET(sink.ensure(sizeof(float)));
    cudaStream_t s = ctx().stream;
    const int blocks = 4 * ctx().nSM, threads = 256;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    P4G_CUDA(cudaEventCreate(&e0));
    P4G_CUDA(cudaEventCreate(&e1));
    int rc = P4G_OK;
    float best = -1.0f;
    for (int rep = 0; rep < 4 && rc == P4G_OK; rep++) {   // first repetition warms the clocks up
        cudaEventRecord(e0, s);
        k_fmaPeak<<<blocks, threads, 0, s>>>(sink.as<float>(), iters, 1.0f + rep);
        cudaEventRecord(e1, s);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            rc = setError(P4G_ECUDA, "fp32FmaPeak: %s", cudaGetErrorString(e));
            break;
        }
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && (best < 0.0f || t < best)) best = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != P4G_OK) return rc;
    const double flops = 2.0 * blocks * threads * (double)iters * kUnroll * kChains;
    *ms = best;
    *tflops = flops / (best * 1e-3) / 1e12;
    return P4G_OK;
}
