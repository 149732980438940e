// The learned-proposal network: a 3-layer MLP (dIn -> H -> H -> dOut, tanh
// hidden activations) with BF16 weights, FP32 accumulation, FP32 master
// weights and Adam, trained on the GPU by these kernels.
//
// It has no counterpart in the reference (p4's proposals are all hand-made).
// The network is a block-conditional density over the chain's whitened
// continuous coordinates (p4gpu/learned.py): its input is the coordinates with
// one block zeroed plus the block's mask, its output the conditional mean and
// log standard deviation of every coordinate.  The MCMC uses only the learned
// scale, in a symmetric random walk on the block whose step size depends on
// the untouched coordinates alone, so the move needs no proposal-density term.
// Output layout per row: mu[0:d], s[d:2d]; the training loss is the Gaussian
// negative log density of the targets (NaN targets left out), mean over the
// batch: sum_i s_i + (t_i - mu_i)^2 exp(-2 s_i) / 2.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <vector>
#include "p4g_internal.h"

namespace p4g {

constexpr float S_MIN = -12.f, S_MAX = 6.f;

struct Mlp {
    int dIn, H, dOut, maxB;
    int nW1, nW2, nW3, nParams;
    size_t oW1, ob1, oW2, ob2, oW3, ob3;   // offsets into the parameter vector
    DevBuf params, grads, m1, m2;         // FP32
    DevBuf wbf;                            // BF16 copies of W1, W2, W3
    DevBuf wmap;                           // parameter index -> BF16 copy index or -1
    DevBuf X, H1, H2, Y, T, dY, dH2, dH1, loss;
    int step = 0;
};

// ---------------------------------------------------------------- kernels
// out[b][n] = act(bias[n] + sum_k in[b][k] * W[n][k]); one block per row b.
template <bool TANH>
__global__ void k_linear(const float *__restrict__ in, const __nv_bfloat16 *__restrict__ W,
                         const float *__restrict__ bias, float *__restrict__ out, int K, int N)
{
    extern __shared__ float row[];
    const int b = blockIdx.x;
    for (int k = threadIdx.x; k < K; k += blockDim.x) row[k] = in[(size_t)b * K + k];
    __syncthreads();
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const __nv_bfloat16 *w = W + (size_t)n * K;
        float acc = bias[n];
        for (int k = 0; k < K; k++) acc = fmaf(row[k], __bfloat162float(w[k]), acc);
        out[(size_t)b * N + n] = TANH ? tanhf(acc) : acc;
    }
}

// Gaussian NLL and its gradient w.r.t. the outputs (mu, s).
__global__ void k_nll(const float *__restrict__ Y, const float *__restrict__ T, float *__restrict__ dY,
                      float *__restrict__ loss, int B, int d)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (idx < B * d) {
        const int b = idx / d, i = idx % d;
        const float t = T[(size_t)b * d + i];
        if (t != t) {   // NaN target: coordinate not scored in this row
            dY[(size_t)b * 2 * d + i] = 0.f;
            dY[(size_t)b * 2 * d + d + i] = 0.f;
        } else {
            const float mu = Y[(size_t)b * 2 * d + i];
            const float sr = Y[(size_t)b * 2 * d + d + i];
            const float s = fminf(fmaxf(sr, S_MIN), S_MAX);
            const float e = expf(-s);
            const float r = (t - mu) * e;
            l = s + 0.5f * r * r;
            dY[(size_t)b * 2 * d + i] = -r * e / B;
            dY[(size_t)b * 2 * d + d + i] = (sr > S_MIN && sr < S_MAX) ? (1.f - r * r) / B : 0.f;
        }
    }
    for (int o = 16; o; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / B);
}

// dIn[b][k] = (sum_n dOut[b][n] W[n][k]) * (1 - h[b][k]^2)   (tanh' at the layer input)
__global__ void k_linear_back_in(const float *__restrict__ dOut, const __nv_bfloat16 *__restrict__ W,
                                 const float *__restrict__ h, float *__restrict__ dIn, int B, int K, int N)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B * K) return;
    const int b = idx / K, k = idx % K;
    float acc = 0.f;
    for (int n = 0; n < N; n++) acc = fmaf(dOut[(size_t)b * N + n], __bfloat162float(W[(size_t)n * K + k]), acc);
    const float hv = h[idx];
    dIn[idx] = acc * (1.f - hv * hv);
}

// dW[n][k] = sum_b dOut[b][n] in[b][k];  db[n] = sum_b dOut[b][n]  (fixed order)
__global__ void k_linear_back_w(const float *__restrict__ dOut, const float *__restrict__ in,
                                float *__restrict__ dW, float *__restrict__ db, int B, int K, int N)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * (K + 1)) return;
    const int n = idx / (K + 1), k = idx % (K + 1);
    float acc = 0.f;
    if (k < K) {
        for (int b = 0; b < B; b++) acc = fmaf(dOut[(size_t)b * N + n], in[(size_t)b * K + k], acc);
        dW[(size_t)n * K + k] = acc;
    } else {
        for (int b = 0; b < B; b++) acc += dOut[(size_t)b * N + n];
        db[n] = acc;
    }
}

// Adam on the FP32 masters, then refresh the BF16 weight copies.
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float c1,
                       float c2, const int *__restrict__ wmap, __nv_bfloat16 *__restrict__ wbf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    const int w = wmap[i];
    if (w >= 0) wbf[w] = __float2bfloat16_rn(pi);
}

__global__ void k_to_bf16(const float *__restrict__ p, const int *__restrict__ wmap,
                          __nv_bfloat16 *__restrict__ wbf, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int w = wmap[i];
    if (w >= 0) wbf[w] = __float2bfloat16_rn(p[i]);
}

// ---------------------------------------------------------------- host
static inline Mlp *M(p4g_mlp *m) { return reinterpret_cast<Mlp *>(m); }

static int forward(Mlp *m, int B)
{
    cudaStream_t s = ctx().stream;
    const __nv_bfloat16 *w = m->wbf.as<__nv_bfloat16>();
    const float *P = m->params.as<float>();
    k_linear<true><<<B, 128, sizeof(float) * m->dIn, s>>>(m->X.as<float>(), w, P + m->ob1, m->H1.as<float>(),
                                                          m->dIn, m->H);
    k_linear<true><<<B, 128, sizeof(float) * m->H, s>>>(m->H1.as<float>(), w + m->nW1, P + m->ob2,
                                                         m->H2.as<float>(), m->H, m->H);
    k_linear<false><<<B, 128, sizeof(float) * m->H, s>>>(m->H2.as<float>(), w + m->nW1 + m->nW2, P + m->ob3,
                                                          m->Y.as<float>(), m->H, m->dOut);
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

static int backward(Mlp *m, int B)
{
    cudaStream_t s = ctx().stream;
    const int d = m->dOut / 2;
    const __nv_bfloat16 *w = m->wbf.as<__nv_bfloat16>();
    float *G = m->grads.as<float>();
    P4G_CUDA(cudaMemsetAsync(m->loss.ptr, 0, sizeof(float), s));
    k_nll<<<(B * d + 127) / 128, 128, 0, s>>>(m->Y.as<float>(), m->T.as<float>(), m->dY.as<float>(),
                                              m->loss.as<float>(), B, d);
    // layer 3
    k_linear_back_w<<<(m->dOut * (m->H + 1) + 127) / 128, 128, 0, s>>>(m->dY.as<float>(), m->H2.as<float>(),
                                                                       G + m->oW3, G + m->ob3, B, m->H, m->dOut);
    k_linear_back_in<<<(B * m->H + 127) / 128, 128, 0, s>>>(m->dY.as<float>(), w + m->nW1 + m->nW2,
                                                            m->H2.as<float>(), m->dH2.as<float>(), B, m->H, m->dOut);
    // layer 2
    k_linear_back_w<<<(m->H * (m->H + 1) + 127) / 128, 128, 0, s>>>(m->dH2.as<float>(), m->H1.as<float>(),
                                                                    G + m->oW2, G + m->ob2, B, m->H, m->H);
    k_linear_back_in<<<(B * m->H + 127) / 128, 128, 0, s>>>(m->dH2.as<float>(), w + m->nW1, m->H1.as<float>(),
                                                            m->dH1.as<float>(), B, m->H, m->H);
    // layer 1
    k_linear_back_w<<<(m->H * (m->dIn + 1) + 127) / 128, 128, 0, s>>>(m->dH1.as<float>(), m->X.as<float>(),
                                                                      G + m->oW1, G + m->ob1, B, m->dIn, m->H);
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

static int upload(Mlp *m, const float *x, int B, const float *t)
{
    cudaStream_t s = ctx().stream;
    if (B < 1 || B > m->maxB) return setError(P4G_EINVAL, "mlp: batch %d not in [1, %d]", B, m->maxB);
    P4G_CUDA(cudaMemcpyAsync(m->X.ptr, x, sizeof(float) * B * m->dIn, cudaMemcpyHostToDevice, s));
    if (t) P4G_CUDA(cudaMemcpyAsync(m->T.ptr, t, sizeof(float) * B * (m->dOut / 2), cudaMemcpyHostToDevice, s));
    return P4G_OK;
}

}  // namespace p4g

using namespace p4g;

static uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

extern "C" p4g_mlp *p4g_mlpNew(int dIn, int hidden, int dOut, int maxBatch, unsigned long long seed)
{
    if (dIn < 1 || hidden < 1 || dOut < 2 || (dOut & 1) || maxBatch < 1) {
        setError(P4G_EINVAL, "mlpNew: dIn=%d hidden=%d dOut=%d (even) maxBatch=%d", dIn, hidden, dOut, maxBatch);
        return nullptr;
    }
    if (ensureCtx() != P4G_OK) return nullptr;
    Mlp *m = new Mlp;
    m->dIn = dIn;
    m->H = hidden;
    m->dOut = dOut;
    m->maxB = maxBatch;
    m->nW1 = hidden * dIn;
    m->nW2 = hidden * hidden;
    m->nW3 = dOut * hidden;
    m->oW1 = 0;
    m->ob1 = m->oW1 + m->nW1;
    m->oW2 = m->ob1 + hidden;
    m->ob2 = m->oW2 + m->nW2;
    m->oW3 = m->ob2 + hidden;
    m->ob3 = m->oW3 + m->nW3;
    m->nParams = (int)(m->ob3 + dOut);
    // Xavier-uniform weights, zero biases; the output layer starts small and
    // its s half biased to log(0.1)
    std::vector<float> p(m->nParams, 0.f);
    uint64_t st = seed * 0x2545F4914F6CDD1DULL + 1;
    auto uni = [&](float a) { return (float)(((splitmix(st) >> 11) * (1.0 / 9007199254740992.0)) * 2 - 1) * a; };
    for (int i = 0; i < m->nW1; i++) p[m->oW1 + i] = uni(sqrtf(6.f / (dIn + hidden)));
    for (int i = 0; i < m->nW2; i++) p[m->oW2 + i] = uni(sqrtf(6.f / (2 * hidden)));
    for (int i = 0; i < m->nW3; i++) p[m->oW3 + i] = 0.01f * uni(sqrtf(6.f / (hidden + dOut)));
    for (int i = dOut / 2; i < dOut; i++) p[m->ob3 + i] = logf(0.1f);
    std::vector<int> wmap(m->nParams, -1);
    for (int i = 0; i < m->nW1; i++) wmap[m->oW1 + i] = i;
    for (int i = 0; i < m->nW2; i++) wmap[m->oW2 + i] = m->nW1 + i;
    for (int i = 0; i < m->nW3; i++) wmap[m->oW3 + i] = m->nW1 + m->nW2 + i;
    const size_t B = maxBatch;
    bool ok = m->params.ensure(sizeof(float) * m->nParams) == P4G_OK &&
              m->grads.ensure(sizeof(float) * m->nParams) == P4G_OK &&
              m->m1.ensure(sizeof(float) * m->nParams) == P4G_OK &&
              m->m2.ensure(sizeof(float) * m->nParams) == P4G_OK &&
              m->wbf.ensure(sizeof(__nv_bfloat16) * (m->nW1 + m->nW2 + m->nW3)) == P4G_OK &&
              m->wmap.ensure(sizeof(int) * m->nParams) == P4G_OK &&
              m->X.ensure(sizeof(float) * B * dIn) == P4G_OK && m->H1.ensure(sizeof(float) * B * hidden) == P4G_OK &&
              m->H2.ensure(sizeof(float) * B * hidden) == P4G_OK && m->Y.ensure(sizeof(float) * B * dOut) == P4G_OK &&
              m->T.ensure(sizeof(float) * B * dOut / 2) == P4G_OK && m->dY.ensure(sizeof(float) * B * dOut) == P4G_OK &&
              m->dH2.ensure(sizeof(float) * B * hidden) == P4G_OK &&
              m->dH1.ensure(sizeof(float) * B * hidden) == P4G_OK && m->loss.ensure(sizeof(float)) == P4G_OK;
    if (!ok) {
        delete m;
        return nullptr;
    }
    cudaStream_t s = ctx().stream;
    if (cudaMemcpyAsync(m->params.ptr, p.data(), sizeof(float) * m->nParams, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(m->wmap.ptr, wmap.data(), sizeof(int) * m->nParams, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(m->m1.ptr, 0, sizeof(float) * m->nParams, s) != cudaSuccess ||
        cudaMemsetAsync(m->m2.ptr, 0, sizeof(float) * m->nParams, s) != cudaSuccess) {
        setError(P4G_ECUDA, "mlpNew: upload failed");
        delete m;
        return nullptr;
    }
    k_to_bf16<<<(m->nParams + 255) / 256, 256, 0, s>>>(m->params.as<float>(), m->wmap.as<int>(),
                                                         m->wbf.as<__nv_bfloat16>(), m->nParams);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        setError(P4G_ECUDA, "mlpNew: init failed");
        delete m;
        return nullptr;
    }
    return reinterpret_cast<p4g_mlp *>(m);
}

extern "C" int p4g_mlpFree(p4g_mlp *mm)
{
    Mlp *m = M(mm);
    if (!m) return P4G_OK;
    cudaStreamSynchronize(ctx().stream);
    delete m;
    return P4G_OK;
}

extern "C" int p4g_mlpNumParams(p4g_mlp *mm, int *n)
{
    Mlp *m = M(mm);
    if (!m || !n) return setError(P4G_EINVAL, "mlpNumParams: null");
    *n = m->nParams;
    return P4G_OK;
}

extern "C" int p4g_mlpGetParams(p4g_mlp *mm, float *out)
{
    Mlp *m = M(mm);
    if (!m || !out) return setError(P4G_EINVAL, "mlpGetParams: null");
    P4G_CUDA(cudaStreamSynchronize(ctx().stream));
    P4G_CUDA(cudaMemcpy(out, m->params.ptr, sizeof(float) * m->nParams, cudaMemcpyDeviceToHost));
    return P4G_OK;
}

extern "C" int p4g_mlpSetParams(p4g_mlp *mm, const float *in)
{
    Mlp *m = M(mm);
    if (!m || !in) return setError(P4G_EINVAL, "mlpSetParams: null");
    cudaStream_t s = ctx().stream;
    P4G_CUDA(cudaMemcpyAsync(m->params.ptr, in, sizeof(float) * m->nParams, cudaMemcpyHostToDevice, s));
    k_to_bf16<<<(m->nParams + 255) / 256, 256, 0, s>>>(m->params.as<float>(), m->wmap.as<int>(),
                                                         m->wbf.as<__nv_bfloat16>(), m->nParams);
    P4G_CUDA(cudaGetLastError());
    P4G_CUDA(cudaStreamSynchronize(s));
    return P4G_OK;
}

extern "C" int p4g_mlpForward(p4g_mlp *mm, const float *x, int B, float *y)
{
    Mlp *m = M(mm);
    if (!m || !x || !y) return setError(P4G_EINVAL, "mlpForward: null");
    int rc = upload(m, x, B, nullptr);
    if (rc) return rc;
    rc = forward(m, B);
    if (rc) return rc;
    P4G_CUDA(cudaMemcpyAsync(y, m->Y.ptr, sizeof(float) * B * m->dOut, cudaMemcpyDeviceToHost, ctx().stream));
    P4G_CUDA(cudaStreamSynchronize(ctx().stream));
    return P4G_OK;
}

extern "C" int p4g_mlpGradients(p4g_mlp *mm, const float *x, const float *t, int B, float *grads, float *loss)
{
    Mlp *m = M(mm);
    if (!m || !x || !t) return setError(P4G_EINVAL, "mlpGradients: null");
    int rc = upload(m, x, B, t);
    if (!rc) rc = forward(m, B);
    if (!rc) rc = backward(m, B);
    if (rc) return rc;
    cudaStream_t s = ctx().stream;
    if (grads) P4G_CUDA(cudaMemcpyAsync(grads, m->grads.ptr, sizeof(float) * m->nParams, cudaMemcpyDeviceToHost, s));
    if (loss) P4G_CUDA(cudaMemcpyAsync(loss, m->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
    P4G_CUDA(cudaStreamSynchronize(s));
    return P4G_OK;
}

extern "C" int p4g_mlpTrainStep(p4g_mlp *mm, const float *x, const float *t, int B, float lr, float *loss)
{
    Mlp *m = M(mm);
    if (!m || !x || !t) return setError(P4G_EINVAL, "mlpTrainStep: null");
    int rc = upload(m, x, B, t);
    if (!rc) rc = forward(m, B);
    if (!rc) rc = backward(m, B);
    if (rc) return rc;
    m->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
    cudaStream_t s = ctx().stream;
    k_adam<<<(m->nParams + 255) / 256, 256, 0, s>>>(m->params.as<float>(), m->grads.as<float>(), m->m1.as<float>(),
                                                     m->m2.as<float>(), m->nParams, lr, b1, b2, 1e-8f, c1, c2,
                                                     m->wmap.as<int>(), m->wbf.as<__nv_bfloat16>());
    P4G_CUDA(cudaGetLastError());
    if (loss) {
        P4G_CUDA(cudaMemcpyAsync(loss, m->loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
        P4G_CUDA(cudaStreamSynchronize(s));
    }
    return P4G_OK;
}
