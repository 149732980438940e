// Site-pattern compression on the GPU: the output of makePatterns
// (Pf/part.c:317-449) -- unique alignment columns in first-occurrence order,
// their counts and the site -> pattern index -- computed from the part's
// coded sequences in device memory.
//
//   k_colHash   one thread per site: 64-bit FNV-1a hash of the column
//   k_insert    open-addressing table (load <= 1/2); a slot's representative
//               is the smallest site holding that column (atomicCAS to claim
//               an empty slot, atomicMin once the columns compare equal
//               byte for byte, so hash collisions never merge columns)
//   k_resolve   every site finds its slot again: first[i] = representative
//   k_scanFirst one block: exclusive prefix sum of (first[i] == i), which
//               numbers the patterns in order of first occurrence
//   k_emit      seqPosIdx, counts, the representative site of each pattern
//   k_gather    patterns[taxon][pattern]
// The result is identical to the host's linear definition: pattern k is the
// k-th site (in site order) whose column has not occurred before.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <vector>
#include "p4g_internal.h"

using namespace p4g;

namespace {

constexpr int EMPTY = 0x7f7f7f7f;   // what a 0x7f byte fill leaves; above every site index

__global__ void k_colHash(const int8_t *__restrict__ S, int nTax, int nChar, uint64_t *__restrict__ hash)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nChar) return;
    uint64_t h = 1469598103934665603ULL;
    for (int t = 0; t < nTax; t++) h = (h ^ (uint32_t)(int)S[(size_t)t * nChar + i]) * 1099511628211ULL;
    hash[i] = h;
}

__device__ __forceinline__ bool sameColumn(const int8_t *__restrict__ S, int nTax, int nChar, int a, int b)
{
    for (int t = 0; t < nTax; t++)
        if (S[(size_t)t * nChar + a] != S[(size_t)t * nChar + b]) return false;
    return true;
}

__global__ void k_insert(const int8_t *__restrict__ S, int nTax, int nChar, const uint64_t *__restrict__ hash,
                         int *rep, uint32_t mask, int *overflow)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nChar) return;
    const uint64_t h = hash[i];
    uint32_t s = (uint32_t)h & mask;
    for (uint32_t probe = 0; probe <= mask; probe++) {
        int r = atomicAdd(&rep[s], 0);
        if (r == EMPTY) {
            r = atomicCAS(&rep[s], EMPTY, i);
            if (r == EMPTY) return;   // claimed
        }
        if (hash[r] == h && sameColumn(S, nTax, nChar, r, i)) {
            atomicMin(&rep[s], i);
            return;
        }
        s = (s + 1) & mask;
    }
    atomicOr(overflow, 1);
}

__global__ void k_resolve(const int8_t *__restrict__ S, int nTax, int nChar, const uint64_t *__restrict__ hash,
                          const int *__restrict__ rep, uint32_t mask, int *__restrict__ first,
                          int *__restrict__ isFirst, int *overflow)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nChar) return;
    const uint64_t h = hash[i];
    uint32_t s = (uint32_t)h & mask;
    for (uint32_t probe = 0; probe <= mask; probe++) {
        const int r = rep[s];
        if (r == EMPTY) break;
        if (hash[r] == h && sameColumn(S, nTax, nChar, r, i)) {
            first[i] = r;
            isFirst[i] = (r == i);
            return;
        }
        s = (s + 1) & mask;
    }
    atomicOr(overflow, 2);
    first[i] = i;
    isFirst[i] = 0;
}

// Exclusive prefix sum of flags[0, n) into out[], total into *total; one
// block of 1024 threads, each owning a contiguous chunk.
__global__ void __launch_bounds__(1024) k_scanFirst(const int *__restrict__ flags, int n, int *__restrict__ out,
                                                    int *__restrict__ total)
{
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int chunk = (n + 1023) / 1024;
    const int b = min(n, t * chunk), e = min(n, b + chunk);
    int s = 0;
    for (int i = b; i < e; i++) s += flags[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;   // exclusive prefix of this chunk
    for (int i = b; i < e; i++) {
        out[i] = run;
        run += flags[i];
    }
    if (t == 1023) *total = part[1023];
}

__global__ void k_emit(int nChar, const int *__restrict__ first, const int *__restrict__ isFirst,
                       const int *__restrict__ patOfSite, int *__restrict__ seqPosIdx, int *__restrict__ counts,
                       int *__restrict__ firstSite)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nChar) return;
    const int k = patOfSite[first[i]];
    seqPosIdx[i] = k;
    atomicAdd(&counts[k], 1);
    if (isFirst[i]) firstSite[k] = i;
}

__global__ void k_gather(const int8_t *__restrict__ S, int nTax, int nChar, int nPat,
                         const int *__restrict__ firstSite, int *__restrict__ patterns)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)nTax * nPat) return;
    const int t = (int)(idx / nPat), k = (int)(idx % nPat);
    patterns[idx] = S[(size_t)t * nChar + firstSite[k]];
}

}  // namespace

extern "C" int p4g_makePatternsDevice(p4g_part *pp)
{
    Part *p = reinterpret_cast<Part *>(pp);
    if (!p) return setError(P4G_EINVAL, "makePatternsDevice: null part");
    const int ctxRc = ensureCtx();
    if (ctxRc != P4G_OK) return ctxRc;
    const int nTax = p->nTax, nChar = p->nChar;
    if (nTax <= 0 || nChar <= 0) return setError(P4G_EINVAL, "makePatternsDevice: empty part");
    if ((int)p->sequences.size() != nTax * nChar)
        return setError(P4G_ESTATE, "makePatternsDevice: sequences not poked");
    std::vector<int8_t> s8((size_t)nTax * nChar);
    for (size_t k = 0; k < s8.size(); k++) s8[k] = (int8_t)p->sequences[k];   // p4 codes lie in [-64, 32)
    uint32_t cap = 1;
    while (cap < (uint32_t)nChar * 2u + 16u) cap <<= 1;
    DevBuf dS, dHash, dRep, dFirst, dIsFirst, dPatOf, dSeqPos, dCounts, dFirstSite, dPatterns, dMisc;
    const int n = nChar;
    if (dS.ensure(s8.size()) || dHash.ensure(sizeof(uint64_t) * n) || dRep.ensure(sizeof(int) * cap) ||
        dFirst.ensure(sizeof(int) * n) || dIsFirst.ensure(sizeof(int) * n) || dPatOf.ensure(sizeof(int) * n) ||
        dSeqPos.ensure(sizeof(int) * n) || dCounts.ensure(sizeof(int) * n) || dFirstSite.ensure(sizeof(int) * n) ||
        dMisc.ensure(sizeof(int) * 2))
        return P4G_ENOMEM;
    cudaStream_t st = ctx().stream;
    const int8_t *S = dS.as<int8_t>();
    const int B = 256, G = (n + B - 1) / B;
    P4G_CUDA(cudaMemcpyAsync(dS.ptr, s8.data(), s8.size(), cudaMemcpyHostToDevice, st));
    P4G_CUDA(cudaMemsetAsync(dRep.ptr, 0x7f, sizeof(int) * cap, st));   // every byte 0x7f: EMPTY
    P4G_CUDA(cudaMemsetAsync(dCounts.ptr, 0, sizeof(int) * n, st));
    P4G_CUDA(cudaMemsetAsync(dMisc.ptr, 0, sizeof(int) * 2, st));
    k_colHash<<<G, B, 0, st>>>(S, nTax, nChar, dHash.as<uint64_t>());
    k_insert<<<G, B, 0, st>>>(S, nTax, nChar, dHash.as<uint64_t>(), dRep.as<int>(), cap - 1, dMisc.as<int>());
    k_resolve<<<G, B, 0, st>>>(S, nTax, nChar, dHash.as<uint64_t>(), dRep.as<int>(), cap - 1, dFirst.as<int>(),
                               dIsFirst.as<int>(), dMisc.as<int>());
    k_scanFirst<<<1, 1024, 0, st>>>(dIsFirst.as<int>(), n, dPatOf.as<int>(), dMisc.as<int>() + 1);
    k_emit<<<G, B, 0, st>>>(n, dFirst.as<int>(), dIsFirst.as<int>(), dPatOf.as<int>(), dSeqPos.as<int>(),
                            dCounts.as<int>(), dFirstSite.as<int>());
    P4G_CUDA(cudaGetLastError());
    int misc[2] = {0, 0};
    P4G_CUDA(cudaMemcpyAsync(misc, dMisc.ptr, sizeof(misc), cudaMemcpyDeviceToHost, st));
    P4G_CUDA(cudaStreamSynchronize(st));
    if (misc[0]) return setError(P4G_ENUMERIC, "makePatternsDevice: hash table probe failed (%d)", misc[0]);
    const int nPat = misc[1];
    if (nPat <= 0 || nPat > nChar) return setError(P4G_ENUMERIC, "makePatternsDevice: bad pattern count %d", nPat);
    if (dPatterns.ensure(sizeof(int) * (size_t)nTax * nPat)) return P4G_ENOMEM;
    const size_t np = (size_t)nTax * nPat;
    k_gather<<<(unsigned)((np + B - 1) / B), B, 0, st>>>(S, nTax, nChar, nPat, dFirstSite.as<int>(),
                                                        dPatterns.as<int>());
    P4G_CUDA(cudaGetLastError());
    p->counts.assign(nPat, 0);
    p->seqPosIdx.assign(nChar, 0);
    p->patterns.assign(np, 0);
    P4G_CUDA(cudaMemcpyAsync(p->counts.data(), dCounts.ptr, sizeof(int) * nPat, cudaMemcpyDeviceToHost, st));
    P4G_CUDA(cudaMemcpyAsync(p->seqPosIdx.data(), dSeqPos.ptr, sizeof(int) * nChar, cudaMemcpyDeviceToHost, st));
    P4G_CUDA(cudaMemcpyAsync(p->patterns.data(), dPatterns.ptr, sizeof(int) * np, cudaMemcpyDeviceToHost, st));
    P4G_CUDA(cudaStreamSynchronize(st));
    p->nPatterns = nPat;
    p->patternsMade = true;
    p->invarMade = false;
    p->devValid = false;
    return P4G_OK;
}
