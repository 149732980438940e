// The plain FP64 GPU path: a direct restatement of the reference's pruning
// on the GPU, kept as the denominator of the FP32 path's speed-up and as an
// FP64 evaluation mode of the library (p4g_setPrecision(tree, 1)).
//
// Same structure as the reference: one launch per internal node in
// post-order, each computing cl[cat][state][pattern] in FP64 from its
// children exactly as p4_setConditionalLikelihoodsOfInternalNodePart
// (Pf/p4_node.c:636-857) does -- first child assigns, later children
// multiply, leaf children look up P[s][code] (1 for gap/?/N-like, a sum over
// members for other equates), internal children sum_j P[s][j] cl[j] -- and
// no rescaling.  The root reduction follows p4_partLogLikeLoop /
// p4_partLogLikeLoopRootLeaf (Pf/p4_tree.c:1029-1378): like = sum over
// (cat, state) of pi[s] cl[cat][s][p], pInvar term, /nCat, then
// count * log(like), with the -1e99 sentinel for like <= 0.
#include <cuda_runtime.h>
#include "p4g_internal.h"
#include "p4g_prune64.cuh"

namespace p4g {

template <int DIM>
__global__ void __launch_bounds__(128)
k_node64(const Node64Job *__restrict__ jobs, int nodeIdx)
{
    const Node64Job &J = jobs[blockIdx.y];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int nCat = J.nCat;
    if (p >= J.nPat * nCat) return;
    const int cat = p / J.nPat, pat = p % J.nPat;
    const int *node = J.table + J.nodeStart[nodeIdx];
    const int self = node[0], nKids = node[1];
    double cl[DIM];
    for (int k = 0; k < nKids; k++) {
        const int child = node[2 + 3 * k], kind = node[3 + 3 * k], ref = node[4 + 3 * k];
        const double *P = J.decks64 + ((size_t)child * nCat + cat) * DIM * DIM;
        double f[DIM];
        if (kind == 0) {  // leaf: raw p4 character code
            const int code = J.patterns[(size_t)ref * J.nPat + pat];
            if (code >= 0) {
                for (int s = 0; s < DIM; s++) f[s] = P[s * DIM + code];
            } else if (code == GAP_CODE || code == QMARK_CODE || code == N_LIKE) {
                for (int s = 0; s < DIM; s++) f[s] = 1.0;
            } else {
                const int e = code - EQUATES_BASE;
                const int *eq = J.equates + e * DIM;
                int isN = 1;
                for (int j = 0; j < DIM; j++)
                    if (!eq[j]) isN = 0;
                for (int s = 0; s < DIM; s++) {
                    double sum = 0.0;
                    if (isN) {
                        sum = 1.0;
                    } else {
                        for (int j = 0; j < DIM; j++)
                            if (eq[j]) sum = sum + P[s * DIM + j];
                    }
                    f[s] = sum;
                }
            }
        } else {  // internal child: ref = its internal index
            const double *x = J.cl + ((size_t)ref * nCat + cat) * DIM * J.nPatPad + pat;
            double xv[DIM];
            for (int j = 0; j < DIM; j++) xv[j] = x[(size_t)j * J.nPatPad];
            for (int s = 0; s < DIM; s++) {
                double sum = 0.0;
                for (int j = 0; j < DIM; j++) sum = sum + P[s * DIM + j] * xv[j];
                f[s] = sum;
            }
        }
        if (k == 0) {
            for (int s = 0; s < DIM; s++) cl[s] = f[s];
        } else {
            for (int s = 0; s < DIM; s++) cl[s] *= f[s];
        }
    }
    (void)self;
    double *out = J.cl + ((size_t)nodeIdx * nCat + cat) * DIM * J.nPatPad + pat;
    for (int s = 0; s < DIM; s++) out[(size_t)s * J.nPatPad] = cl[s];
}

template <int DIM>
__global__ void __launch_bounds__(128)
k_root64(const Node64Job *__restrict__ jobs)
{
    const Node64Job &J = jobs[blockIdx.y];
    const int pat = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = pat < J.nPat;
    double v = 0.0;
    int bad = 0;
    if (valid) {
        const double *root = J.cl + (size_t)J.rootInternal * J.nCat * DIM * J.nPatPad + pat;
        double like = 0.0;
        uint32_t mask = (DIM >= 32) ? 0xffffffffu : ((1u << DIM) - 1u);
        if (J.rootLeafRow >= 0) {
            int code = J.patterns[(size_t)J.rootLeafRow * J.nPat + pat];
            if (code >= 0) mask = 1u << code;
            else if (code != GAP_CODE && code != QMARK_CODE && code != N_LIKE) {
                const int *eq = J.equates + (code - EQUATES_BASE) * DIM;
                uint32_t m = 0;
                for (int j = 0; j < DIM; j++)
                    if (eq[j]) m |= 1u << j;
                mask = m;
            }
        }
        for (int c = 0; c < J.nCat; c++)
            for (int s = 0; s < DIM; s++)
                if ((mask >> s) & 1u)
                    like = __dadd_rn(like, __dmul_rn(J.rootComp[s], root[((size_t)c * DIM + s) * J.nPatPad]));
        if (J.pInvar != 0.0) {
            like = __dmul_rn(like, J.varScale);
            uint32_t im = J.invMask[pat];
            for (int s = 0; s < DIM; s++)
                if ((im >> s) & 1u) like = __dadd_rn(like, __dmul_rn(J.rootComp[s], J.pInvar));
        } else if (J.nCat > 1) {
            like = like / (double)J.nCat;
        }
        if (!(like > 0.0)) bad = 1;
        else v = J.counts[pat] * log(like);
    }
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __shared__ double red[4];
    __shared__ int sLast;
    int anyBad = __syncthreads_or(bad);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = red[0] + red[1] + red[2] + red[3];
        J.partials[blockIdx.x] = s;
        if (anyBad) atomicOr(J.badFlag, 1);
        __threadfence();
        sLast = (atomicAdd(J.ticket, 1) == (int)gridDim.x - 1);
    }
    __syncthreads();
    if (sLast && threadIdx.x < 32) {
        __threadfence();
        double s = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) s += __ldcg(J.partials + i);
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) {
            *J.out = atomicExch(J.badFlag, 0) ? -1.0e99 : s;
            atomicExch(J.ticket, 0);
        }
    }
}

template <int DIM>
static int launch64(const Node64Job *dJob, const Node64Job &h, cudaStream_t s)
{
    const int threads = 128;
    dim3 gridN((h.nPat * h.nCat + threads - 1) / threads, 1);
    for (int k = 0; k < h.nInternal; k++) {
        k_node64<DIM><<<gridN, threads, 0, s>>>(dJob, k);
        P4G_CUDA(cudaGetLastError());
    }
    dim3 gridR((h.nPat + threads - 1) / threads, 1);
    k_root64<DIM><<<gridR, threads, 0, s>>>(dJob);
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

int launchNode64(const Node64Job *dJob, const Node64Job &h, int nodeIdx, cudaStream_t s)
{
    if (nodeIdx < 0 || nodeIdx >= h.nInternal) return setError(P4G_EINVAL, "launchNode64: bad node %d", nodeIdx);
    const int threads = 128;
    dim3 grid((h.nPat * h.nCat + threads - 1) / threads, 1);
    switch (h.dim) {
    case 2: k_node64<2><<<grid, threads, 0, s>>>(dJob, nodeIdx); break;
    case 4: k_node64<4><<<grid, threads, 0, s>>>(dJob, nodeIdx); break;
    case 20: k_node64<20><<<grid, threads, 0, s>>>(dJob, nodeIdx); break;
    default: return setError(P4G_EUNSUPPORTED, "no FP64 pruning kernel for dim=%d", h.dim);
    }
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

int launchPrune64(const Node64Job *dJob, const Node64Job &h, cudaStream_t s)
{
    switch (h.dim) {
    case 2: return launch64<2>(dJob, h, s);
    case 4: return launch64<4>(dJob, h, s);
    case 20: return launch64<20>(dJob, h, s);
    default:
        return setError(P4G_EUNSUPPORTED, "no FP64 pruning kernel for dim=%d", h.dim);
    }
}

}  // namespace p4g
