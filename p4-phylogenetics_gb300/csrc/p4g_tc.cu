// Self-test of the tensor-core datapath the protein pruning kernel uses:
// one CTA computes D (128 x 32, FP32) = A (128 x 8, TF32, in tensor memory)
// * B^T (B: 32 x 8, TF32, shared memory, K-major core matrices) with one
// tcgen05.mma, reads D back through tcgen05.ld and writes it out.  The host
// compares with an FP64 product of the same (TF32-exact) inputs.
#include <cuda_runtime.h>
#include <math.h>
#include <vector>
#include "p4g_internal.h"
#include "p4g_tc.cuh"

namespace p4g {

namespace {

constexpr int ST_M = 128, ST_N = 32, ST_K = 8;
constexpr uint32_t ST_LBO = 128;   // bytes between core matrices along K
constexpr uint32_t ST_SBO = 256;   // bytes between 8-row groups along N

// B occupies 1 KB; the region is 8 KB so that either reading of the
// descriptor's two strides stays inside it.
__global__ void __launch_bounds__(128) k_tcSelfTest(const float *__restrict__ A, const float *__restrict__ B,
                                                    float *__restrict__ D, int *__restrict__ status, int variant)
{
    __shared__ __align__(1024) unsigned char sB[8192];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t sTmem;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        tc::tmemAlloc(&sTmem, 64);
        tc::tmemRelinquish();
    }
    if (tid == 0) {
        tc::mbarInit(&mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < 8192 / 4; i += 128) ((float *)sB)[i] = 0.f;
    __syncthreads();
    for (int i = tid; i < ST_N * ST_K; i += 128) {
        const int n = i / ST_K, k = i % ST_K;
        const int off = (n / 8) * ST_SBO + (k / 4) * ST_LBO + (n % 8) * 16 + (k % 4) * 4;
        *(float *)(sB + off) = B[i];
    }
    tc::fenceProxyAsync();
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t base = sTmem;
    const uint32_t aCol = 0, dCol = 32;
    const uint32_t laneBase = (uint32_t)(32 * warp) << 16;
    {
        float v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = A[tid * ST_K + k];
        tc::st8(base + laneBase + aCol, v);
        tc::waitSt();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (tid == 0) {
        const uint64_t bd = variant == 0 ? tc::sdesc(tc::smemAddr(sB), ST_LBO, ST_SBO)
                                         : tc::sdesc(tc::smemAddr(sB), ST_SBO, ST_LBO);
        tc::mmaTf32TS(base + dCol, base + aCol, bd, tc::idescTf32(ST_M, ST_N), false);
        tc::commit(&mbar);
    }
    const bool ok = tc::mbarWait(&mbar, 0);
    if (!ok && (tid & 31) == 0) atomicOr(status, 1);
    tc::fenceAfterSync();
    if (__syncthreads_and(ok)) {
#pragma unroll
        for (int c = 0; c < ST_N; c += 8) {
            float v[8];
            tc::ld8(base + laneBase + dCol + c, v);
            tc::waitLd();
#pragma unroll
            for (int j = 0; j < 8; j++) D[tid * ST_N + c + j] = v[j];
        }
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (warp == 0) tc::tmemDealloc(base, 64);
}

}  // namespace

int tensorSelfTest(int variant, double *maxAbsErr)
{
    {
        int rc = ensureCtx();
        if (rc != P4G_OK) return rc;
    }
    std::vector<float> hA(ST_M * ST_K), hB(ST_N * ST_K), hD(ST_M * ST_N, 0.f);
    uint32_t x = 12345u;
    auto rnd = [&]() {   // multiples of 2^-8 in [-1, 1): exact in TF32, products exact in FP32
        x = x * 1664525u + 1013904223u;
        return (float)((int)(x >> 23) - 256) / 256.0f;
    };
    for (auto &v : hA) v = rnd();
    for (auto &v : hB) v = rnd();
    float *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int *dS = nullptr;
    int rc = P4G_OK;
    if (cudaMalloc(&dA, sizeof(float) * hA.size()) != cudaSuccess ||
        cudaMalloc(&dB, sizeof(float) * hB.size()) != cudaSuccess ||
        cudaMalloc(&dD, sizeof(float) * hD.size()) != cudaSuccess || cudaMalloc(&dS, sizeof(int)) != cudaSuccess) {
        rc = setError(P4G_ENOMEM, "tensorSelfTest: cudaMalloc failed");
    } else {
        cudaStream_t s = ctx().stream;
        cudaMemcpyAsync(dA, hA.data(), sizeof(float) * hA.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dB, hB.data(), sizeof(float) * hB.size(), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(dD, 0, sizeof(float) * hD.size(), s);
        cudaMemsetAsync(dS, 0, sizeof(int), s);
        k_tcSelfTest<<<1, 128, 0, s>>>(dA, dB, dD, dS, variant);
        cudaError_t e = cudaGetLastError();
        int st = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(hD.data(), dD, sizeof(float) * hD.size(), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&st, dS, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = setError(P4G_ECUDA, "tensorSelfTest: %s", cudaGetErrorString(e));
        } else if (st) {
            rc = setError(P4G_ETIMEOUT, "tensorSelfTest: the MMA completion wait gave up");
        } else {
            double worst = 0.0;
            for (int m = 0; m < ST_M; m++)
                for (int n = 0; n < ST_N; n++) {
                    double ref = 0.0;
                    for (int k = 0; k < ST_K; k++) ref += (double)hA[m * ST_K + k] * (double)hB[n * ST_K + k];
                    worst = fmax(worst, fabs(ref - (double)hD[m * ST_N + n]));
                }
            *maxAbsErr = worst;
        }
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dS);
    return rc;
}

}  // namespace p4g

extern "C" int p4g_tensorSelfTest(int variant, double *maxAbsErr)
{
    if (!maxAbsErr || variant < 0 || variant > 1) return p4g::setError(P4G_EINVAL, "tensorSelfTest: bad arguments");
    return p4g::tensorSelfTest(variant, maxAbsErr);
}
