// Fused pruning for 20-state (protein) parts with 4 Gamma categories on the
// tensor cores: the same host-built program, tile staging and root
// reduction as k_prune (p4g_prune.cu), with every internal-child transform
// out[s] = sum_j P[s][j] x[j] computed as a split-precision TF32 product
// (3 x TF32, FP32 accumulate) by tcgen05.mma.
//
// Reference loop: p4_setConditionalLikelihoodsOfInternalNodePart
// (Pf/p4_node.c:636-857) per internal node in post-order, then the root
// reduction p4_partLogLike (Pf/p4_tree.c:924-1197).
//
// Block = 4 warpgroups (512 threads), warpgroup c = Gamma category c, thread
// row = pattern (tile of 128 patterns) = tensor-memory lane.  Per transform,
// warpgroup c writes its patterns' vectors x as A = [128 x 24] (K padded
// from 20 with zeros) into tensor memory, split as A = A_hi + A_lo with both
// parts TF32; writes P of its category as B = [32 x 24] (N padded from 20)
// split the same way into shared memory as K-major core matrices; one
// thread issues D = A_lo B_hi^T + A_hi B_lo^T + A_hi B_hi^T (three K-steps
// of 8 each, 9 MMAs of M 128 x N 32 x K 8) and commits to the warpgroup's
// mbarrier; the warpgroup waits (bounded) and reads D back.  The dropped
// A_lo B_lo term is below 2^-22 of each product.
//
// Tensor memory: 512 columns per block; warpgroup c uses columns
// [128c, 128c + 96): A_hi at +0, A_lo at +32, D at +64.
//
// B images: when setPrams has written each internal node's split-TF32 image
// (PruneJob::tcB, 6 KB per node and category), warpgroup c fetches the image
// of the NEXT transform it will run with one bulk copy (cp.async.bulk,
// completing on the warpgroup's B mbarrier) into the other of two B buffers,
// issued right after the current transform's MMAs: the copy's latency
// overlaps the MMAs, the read-back and the ops up to the next transform.  The
// order of transforms is the program's execution order (cherry tables skip
// their cherry's ops), tabulated once per job.
// Rescaling needs a pattern's maximum over all categories: the four
// warpgroups exchange their maxima through shared memory (double-buffered,
// one block barrier per rescale point).  The root chain over (category,
// state) runs in category order, handed from warpgroup to warpgroup.
#include <cuda_runtime.h>
#include <math.h>
#include "p4g_internal.h"
#include "p4g_prune_common.cuh"
#include "p4g_tc.cuh"

namespace p4g {

namespace {

constexpr int TD = 20;            // states
constexpr int TNC = 4;            // categories = warpgroups
constexpr int TTILE = 128;        // patterns per tile = tensor-memory lanes
constexpr int TK = 24;            // K padded to a multiple of 8
constexpr int TN = 32;            // N padded to a multiple of 16
constexpr uint32_t B_LBO = 128;                  // core matrices along K
constexpr uint32_t B_SBO = (TK / 4) * 128;       // 8-row groups along N: 768 B
constexpr int B_FLOATS = (TN / 8) * B_SBO / 4;   // 768 floats = 3 KB per hi or lo
constexpr uint32_t TMEM_COLS = 512;

struct TcLayout {
    int offB, offSlots, offProg, offNext, offCodes, offIdx, offCl, offClE, offPi, offMax, offChain, offRed, total;
    int dblB;      // two B buffers per warpgroup (the bulk-copy prefetch); one when two do not fit
    int clStage;   // clade-table indices staged, the next clade's entries copied ahead into shared memory
};

__host__ __device__ inline int a16(int x) { return (x + 15) & ~15; }

__host__ __device__ inline TcLayout tcLayoutB(int nProg, int nTax, int nSlots, int nClade, int dbl, int stage)
{
    TcLayout L;
    int o = 0;
    L.dblB = dbl;
    L.clStage = stage && nClade > 0;
    L.offB = o;
    o += (dbl ? 2 : 1) * TNC * 2 * B_FLOATS * 4;     // 24 KB per buffer, 1024-aligned at offset 0
    L.offSlots = o;
    o += nSlots * TNC * TD * TTILE * 4;
    L.offProg = o;
    o += nProg * 16;
    L.offNext = o;
    o += a16((nProg + 1) * 4);                       // next transform after each op, then the first
    L.offCodes = o;
    o += a16(nTax * TTILE);
    L.offIdx = o;                                    // clade-table index rows of the tile
    if (L.clStage) o += nClade * TTILE * 4;
    L.offCl = o;                                     // the next clade's entries, [category][pattern][20]
    if (L.clStage) o += TNC * TTILE * TD * 4;
    L.offClE = o;                                    // and their scale exponents, [category][pattern]
    if (L.clStage) o += TNC * TTILE * 4;
    L.offPi = o;
    o += a16(TD * 4);
    L.offMax = o;
    o += 2 * TNC * TTILE * 4;                        // double-buffered category maxima
    L.offChain = o;
    o += TTILE * 4;
    L.offRed = o;
    o += 8 * 8;
    L.total = o;
    return L;
}

// The largest layout that fits a block's 227 KB next to the kernel's static
// shared memory (its barriers, padded to the dynamic array's 1 KB alignment):
// both prefetches, then the B prefetch alone, then neither.
constexpr int TC_DYN_SMEM_MAX = 227 * 1024 - 1024;
__host__ __device__ inline TcLayout tcLayout(int nProg, int nTax, int nSlots, int nClade)
{
    TcLayout L = tcLayoutB(nProg, nTax, nSlots, nClade, 1, 1);
    if (L.total <= TC_DYN_SMEM_MAX) return L;
    L = tcLayoutB(nProg, nTax, nSlots, nClade, 1, 0);
    return L.total <= TC_DYN_SMEM_MAX ? L : tcLayoutB(nProg, nTax, nSlots, nClade, 0, 0);
}

__device__ __forceinline__ void namedBarrier(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__global__ void __launch_bounds__(512, 1)
k_prune_tc(const PruneJob *__restrict__ jobs, const BlockDesc *__restrict__ blocks, int nTiles,
           const int *__restrict__ nTilesDev)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t sBar[TNC];
    __shared__ __align__(8) uint64_t sBarB[TNC];   // B image bulk copies, one per warpgroup
    __shared__ uint32_t sTmem;
    __shared__ int sLast;
    __shared__ volatile int sAbort;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int c = tid >> 7;        // category handled by this warpgroup
    const int row = tid & 127;     // pattern in the tile = tensor-memory lane

    if (warp == 0) {
        tc::tmemAlloc(&sTmem, TMEM_COLS);
        tc::tmemRelinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < TNC; i++) {
            tc::mbarInit(&sBar[i], 1);
            tc::mbarInit(&sBarB[i], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sAbort = 0;
    }
    // B tiles: the padding (s >= 20 or j >= 20) stays zero for the whole
    // kernel (the bulk-copied images carry zero padding too)
    for (int i = tid; i < TNC * 2 * B_FLOATS; i += 512) ((float *)smem)[i] = 0.f;
    tc::fenceProxyAsync();   // the zeros before any bulk copy into the same bytes
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tLane = (uint32_t)(32 * (warp & 3)) << 16;
    const uint32_t tA = sTmem + 128u * c, tAlo = tA + 32u, tD = tA + 64u;
    // B buffer b of this warpgroup: hi at +0, lo at +B_FLOATS
    float *sB0 = (float *)smem + c * 2 * B_FLOATS;
    constexpr int B_BUF = TNC * 2 * B_FLOATS;   // floats between the two buffers
    float *sBhi = sB0;
    float *sBlo = sBhi + B_FLOATS;
    constexpr uint32_t idesc = tc::idescTf32(128, TN);
    uint32_t phase = 0;
    uint32_t bPhase = 0;     // phase of this warpgroup's B barrier
    int bufCur = 0;          // buffer the next transform's image is (being) copied into
    bool bPending = false;   // a bulk copy of this warpgroup not yet waited for
    bool timedOut = false;

    int curJob = -1;
    TcLayout L;
    int4 *sProg = nullptr;
    int *sNext = nullptr;
    uint8_t *sCodes = nullptr;
    uint32_t *sIdx = nullptr;
    float *sCl = nullptr;
    int *sClE = nullptr;
    int clPend = -1;         // the clade whose entries this thread's copies are bringing in
    float *sPi = nullptr, *sSlots = nullptr, *sMax = nullptr, *sChain = nullptr;
    double *sRed = nullptr;

    if (nTilesDev) nTiles = min(nTiles, *nTilesDev);
    for (int tile = blockIdx.x; tile < nTiles; tile += gridDim.x) {
        const BlockDesc bd = blocks[tile];
        const PruneJob &J = jobs[bd.job];
        const int nProg = J.nProg, nTax = J.nTax;
        __syncthreads();   // previous tile is done with the shared buffers
        if (bd.job != curJob) {
            L = tcLayout(nProg, nTax, J.nSlots, J.nClade);
            sProg = (int4 *)(smem + L.offProg);
            sNext = (int *)(smem + L.offNext);
            sCodes = smem + L.offCodes;
            sIdx = (uint32_t *)(smem + L.offIdx);
            sCl = (float *)(smem + L.offCl);
            sClE = (int *)(smem + L.offClE);
            sPi = (float *)(smem + L.offPi);
            sSlots = (float *)(smem + L.offSlots);
            sMax = (float *)(smem + L.offMax);
            sChain = (float *)(smem + L.offChain);
            sRed = (double *)(smem + L.offRed);
            for (int i = tid; i < nProg; i += 512) {
                const int ins = J.prog[i];
                const int op = ins & 15, a = (ins >> 4) & 0x3fff, b = ins >> 18;
                int4 d;
                d.x = op;
                d.y = (op == OP_PUSH || op == OP_MULSLOT) ? a * TNC * TD * TTILE : a * TNC * TD * TD;
                d.z = b * TTILE;
                d.w = a;
                if (op == OP_CHERRY) {   // table offset, both code rows
                    const int K = TD + 1 + J.nPartial;
                    d.y = a * K * K * TNC * TD;
                    d.w = (J.prog[i + 1] >> 18) * TTILE;
                }
                if (op == OP_CLADE) d.y = a * J.nPatPad;   // the clade's row of combination indices
                sProg[i] = d;
            }
            if (tid < TD && !J.cladeOut) sPi[tid] = (float)J.rootComp[tid];   // clade jobs have no root
            __syncthreads();
            if (tid == 0) {   // the transforms in execution order: sNext[op] = the next one, sNext[nProg] = first
                int prev = nProg;
                for (int i = 0; i <= nProg; i++) sNext[i] = -1;
                for (int i = 0; i < nProg;) {
                    const int op = sProg[i].x;
                    if (op == OP_XFORM || op == OP_SCALE_XFORM) {
                        sNext[prev] = i;
                        prev = i;
                    }
                    i += op == OP_CHERRY ? (J.cherryTab ? 5 : 2) : 1;
                }
            }
            curJob = bd.job;
        }
        for (int i = tid; i < nTax * (TTILE / 16); i += 512) {
            const int r = i / (TTILE / 16), q = i % (TTILE / 16);
            const int4 *src = (const int4 *)(J.codes + (size_t)r * J.nPatPad + bd.p0) + q;
            ((int4 *)(sCodes + r * TTILE))[q] = __ldg(src);
        }
        if (L.clStage) {
            for (int i = tid; i < J.nClade * (TTILE / 4); i += 512) {
                const int r = i / (TTILE / 4), q = i % (TTILE / 4);
                const int4 *src = (const int4 *)(J.cladeIdx + (size_t)r * J.nPatPad + bd.p0) + q;
                ((int4 *)(sIdx + r * TTILE))[q] = __ldg(src);
            }
        }
        __syncthreads();
        // clade k's table entry of this (pattern, category), copied into this
        // thread's own shared-memory slots while the ops before OP_CLADE k run
        // (clades are numbered in the order the program reads them)
        auto cladeCopy = [&](int k) {
            cpAsyncWaitAll();   // no earlier copy still writing the slots
            uint32_t u = sIdx[k * TTILE + row];
            if (u >= (uint32_t)J.nCladeEntries) u = 0;   // flagged where it is read
            const float *src = J.cladeTab + ((size_t)u * TNC + c) * TD;
            float *dst = sCl + (c * TTILE + row) * TD;
#pragma unroll
            for (int q = 0; q < TD / 4; q++) cpAsync16(dst + 4 * q, src + 4 * q);
            cpAsync4(sClE + c * TTILE + row, J.cladeExp + u);
            cpAsyncCommit();
            clPend = k;
        };
        clPend = -1;
        if (L.clStage) cladeCopy(0);
        const bool prefetchB = J.tcB != nullptr && L.dblB;
        if (prefetchB && row == 0 && !sAbort && sNext[nProg] >= 0) {   // the tile's first transform
            float *dst = sB0 + bufCur * B_BUF;
            tc::mbarExpectTx(&sBarB[c], 2 * B_FLOATS * 4);
            tc::bulkLoad(dst, J.tcB + ((size_t)sProg[sNext[nProg]].w * TNC + c) * 2 * B_FLOATS, 2 * B_FLOATS * 4,
                         &sBarB[c]);
            bPending = true;
        }

        float acc[TD];
        int E = 0;
        int scalePar = 0;
        int oob = 0;
#pragma unroll
        for (int i = 0; i < TD; i++) acc[i] = 1.0f;

        // rescale: the pattern's maximum over every category, through shared memory
        auto doScale = [&]() {
            float mx = 0.0f;
#pragma unroll
            for (int i = 0; i < TD; i++) mx = fmaxf(mx, acc[i]);
            float *buf = sMax + scalePar * TNC * TTILE;
            buf[c * TTILE + row] = mx;
            __syncthreads();
#pragma unroll
            for (int k = 0; k < TNC; k++) mx = fmaxf(mx, buf[k * TTILE + row]);
            scalePar ^= 1;
            if (mx < 0x1p-32f && mx > 0.0f) {
                int e2;
                (void)frexp32(mx, &e2);
                int k = -e2;
                E += k;
                while (k > 0) {
                    const int step = k > 100 ? 100 : k;
                    const float f = __uint_as_float((unsigned)(127 + step) << 23);
#pragma unroll
                    for (int i = 0; i < TD; i++) acc[i] = __fmul_rn(acc[i], f);
                    k -= step;
                }
            }
        };

        for (int ip = 0; ip < nProg; ip++) {
            const int4 I = sProg[ip];
            switch (I.x) {
            case OP_TIPSET:
            case OP_TIPMUL: {
                const int code = sCodes[I.z + row];
                float v[TD];
                if (code < TD) {
                    const float4 *col = (const float4 *)(J.decks + I.y + c * TD * TD + code * TD);
#pragma unroll
                    for (int q = 0; q < TD / 4; q++) {
                        const float4 w = __ldg(col + q);
                        v[4 * q] = w.x;
                        v[4 * q + 1] = w.y;
                        v[4 * q + 2] = w.z;
                        v[4 * q + 3] = w.w;
                    }
                } else if (code == TD) {
#pragma unroll
                    for (int i = 0; i < TD; i++) v[i] = 1.0f;
                } else {
                    const float *eq = J.eqTab + (((size_t)I.w * J.nPartial + (code - TD - 1)) * TNC + c) * TD;
#pragma unroll
                    for (int i = 0; i < TD; i++) v[i] = __ldg(eq + i);
                }
                if (I.x == OP_TIPSET) {
#pragma unroll
                    for (int i = 0; i < TD; i++) acc[i] = v[i];
                } else {
#pragma unroll
                    for (int i = 0; i < TD; i++) acc[i] = __fmul_rn(acc[i], v[i]);
                }
                break;
            }
            case OP_CHERRY: {
                if (!J.cherryTab) {   // no table for this job: run the cherry's own ops
                    ip++;
                    break;
                }
                const int K = TD + 1 + J.nPartial;
                const int ca = sCodes[I.z + row], cb = sCodes[I.w + row];
                const float4 *e = (const float4 *)(J.cherryTab + I.y + ((ca * K + cb) * TNC + c) * TD);
#pragma unroll
                for (int q = 0; q < TD / 4; q++) {
                    const float4 w = __ldg(e + q);
                    acc[4 * q] = w.x;
                    acc[4 * q + 1] = w.y;
                    acc[4 * q + 2] = w.z;
                    acc[4 * q + 3] = w.w;
                }
                ip += 4;   // the OP_ARG word and the cherry's TIPSET, TIPMUL, SCALE_XFORM
                break;
            }
            case OP_CLADE: {
                int u = L.clStage ? (int)sIdx[I.w * TTILE + row] : (int)J.cladeIdx[I.y + bd.p0 + row];
                if ((uint32_t)u >= (uint32_t)J.nCladeEntries) {   // a stale index: not read (bad bit 4)
                    oob = 1;
                    u = 0;
                }
                if (L.clStage) {
                    cpAsyncWaitAll();
                    const bool have = clPend == I.w;
                    if (have) {
                        const float4 *e = (const float4 *)(sCl + (c * TTILE + row) * TD);
#pragma unroll
                        for (int q = 0; q < TD / 4; q++) {
                            const float4 w = e[q];
                            acc[4 * q] = w.x;
                            acc[4 * q + 1] = w.y;
                            acc[4 * q + 2] = w.z;
                            acc[4 * q + 3] = w.w;
                        }
                        E += sClE[c * TTILE + row];
                    }
                    clPend = -1;
                    if (I.w + 1 < J.nClade) cladeCopy(I.w + 1);
                    if (have) break;
                }
                const float4 *e = (const float4 *)(J.cladeTab + ((size_t)u * TNC + c) * TD);
#pragma unroll
                for (int q = 0; q < TD / 4; q++) {
                    const float4 w = __ldg(e + q);
                    acc[4 * q] = w.x;
                    acc[4 * q + 1] = w.y;
                    acc[4 * q + 2] = w.z;
                    acc[4 * q + 3] = w.w;
                }
                E += J.cladeExp[u];
                break;
            }
            case OP_SCALE_XFORM:
                doScale();
                [[fallthrough]];
            case OP_XFORM: {
                // B = P of this node and category, split into TF32 hi/lo, as core matrices:
                // a copy of the image setPrams wrote, or split here from the FP32 deck
                if (prefetchB) {
                    // bulk-copied into buffer bufCur: the issuing thread waits for it below
                    sBhi = sB0 + bufCur * B_BUF;
                    sBlo = sBhi + B_FLOATS;
                } else {
                    sBhi = sB0;
                    sBlo = sBhi + B_FLOATS;
                    const float *P = J.decks + I.y + c * TD * TD;
                    for (int i = row; i < TD * TD; i += TTILE) {
                        const int s = i / TD, j = i % TD;
                        const float p = __ldg(P + i);
                        const float hi = tc::toTf32(p);
                        const float lo = tc::toTf32(p - hi);
                        const int off = (s >> 3) * (B_SBO / 4) + (j >> 2) * (B_LBO / 4) + (s & 7) * 4 + (j & 3);
                        sBhi[off] = hi;
                        sBlo[off] = lo;
                    }
                }
                // A = this pattern's vector, split the same way, into tensor memory
#pragma unroll
                for (int k = 0; k < TK / 8; k++) {
                    float h[8], l[8];
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        const float x = (8 * k + e < TD) ? acc[8 * k + e] : 0.f;
                        h[e] = tc::toTf32(x);
                        l[e] = tc::toTf32(x - h[e]);
                    }
                    tc::st8(tA + tLane + 8 * k, h);
                    tc::st8(tAlo + tLane + 8 * k, l);
                }
                tc::fenceProxyAsync();
                tc::waitSt();
                tc::fenceBeforeSync();
                namedBarrier(1 + c, 128);
                tc::fenceAfterSync();
                const bool dead = sAbort != 0;
                bool haveB = true;
                if (row == 0 && !dead && prefetchB) {   // this transform's image has arrived
                    if (tc::mbarWait(&sBarB[c], bPhase)) {
                        bPending = false;
                        bPhase ^= 1u;
                    } else {   // give up: no MMAs; complete the MMA barrier's phase for the warpgroup
                        timedOut = true;
                        sAbort = 1;
                        haveB = false;
                        tc::mbarArrive(&sBar[c]);
                    }
                }
                if (row == 0 && !dead && haveB) {
                    const uint32_t bHi = tc::smemAddr(sBhi), bLo = tc::smemAddr(sBlo);
#pragma unroll
                    for (int k = 0; k < TK / 8; k++) {
                        const uint64_t dHi = tc::sdesc(bHi + 256u * k, B_LBO, B_SBO);
                        const uint64_t dLo = tc::sdesc(bLo + 256u * k, B_LBO, B_SBO);
                        tc::mmaTf32TS(tD, tAlo + 8u * k, dHi, idesc, k > 0);
                        tc::mmaTf32TS(tD, tA + 8u * k, dLo, idesc, true);
                        tc::mmaTf32TS(tD, tA + 8u * k, dHi, idesc, true);
                    }
                    tc::commit(&sBar[c]);
                    // the next transform's image into the other buffer, whose
                    // last MMAs completed before the previous read-back
                    const int nx = prefetchB ? sNext[ip] : -1;
                    if (nx >= 0) {
                        tc::mbarExpectTx(&sBarB[c], 2 * B_FLOATS * 4);
                        tc::bulkLoad(sB0 + (bufCur ^ 1) * B_BUF,
                                     J.tcB + ((size_t)sProg[nx].w * TNC + c) * 2 * B_FLOATS, 2 * B_FLOATS * 4,
                                     &sBarB[c]);
                        bPending = true;
                    }
                }
                if (prefetchB) bufCur ^= 1;
                if (!dead) {
                    if (!tc::mbarWait(&sBar[c], phase)) {
                        timedOut = true;
                        sAbort = 1;
                    }
                    phase ^= 1u;
                }
                tc::fenceAfterSync();
                {   // the D columns: every load issued, then one wait
                    static_assert(TK / 8 == 3, "three 8-column loads");
                    float v[TK / 8][8];
#pragma unroll
                    for (int k = 0; k < TK / 8; k++) tc::ld8(tD + tLane + 8 * k, v[k]);
                    tc::waitLd24(v);
#pragma unroll
                    for (int k = 0; k < TK / 8; k++)
#pragma unroll
                        for (int e = 0; e < 8; e++)
                            if (8 * k + e < TD) acc[8 * k + e] = v[k][e];
                }
                break;
            }
            case OP_PUSH: {
                float *sl = sSlots + I.y + c * TD * TTILE + row;
#pragma unroll
                for (int i = 0; i < TD; i++) sl[i * TTILE] = acc[i];
                break;
            }
            case OP_MULSLOT: {
                const float *sl = sSlots + I.y + c * TD * TTILE + row;
#pragma unroll
                for (int i = 0; i < TD; i++) acc[i] = __fmul_rn(acc[i], sl[i * TTILE]);
                break;
            }
            default:   // OP_SCALE
                doScale();
                break;
            }
        }

        if (J.cladeOut) {   // clade-table job: the transformed product and its exponent
            const int pc = bd.p0 + row;
            if (pc < J.nPat) {
                float *o = J.cladeOut + ((size_t)pc * TNC + c) * TD;
#pragma unroll
                for (int s = 0; s < TD; s++) o[s] = sAbort ? __int_as_float(0x7fc00000) : acc[s];
                if (c == 0) J.cladeOutExp[pc] = E;
            }
            continue;
        }

        // ---- root: one fmaf chain over (category, state) in category order
        const int pp = bd.p0 + row;
        const bool valid = pp < J.nPat;
        uint32_t rmask = (1u << TD) - 1u;
        if (J.rootLeafRow >= 0) {
            const int code = sCodes[J.rootLeafRow * TTILE + row];
            if (code < TD) rmask = 1u << code;
            else if (code > TD) rmask = J.partialMask[code - TD - 1];
        }
        if (J.rootCL && valid) {   // root partials for ancestral-state draws
            float *o = J.rootCL + ((size_t)pp * TNC + c) * TD;
#pragma unroll
            for (int s = 0; s < TD; s++) o[s] = ((rmask >> s) & 1u) ? acc[s] : 0.0f;
        }
        if (J.catLikes && valid) {   // per-category sums for site rates
            float sc = 0.0f;
#pragma unroll
            for (int s = 0; s < TD; s++)
                if ((rmask >> s) & 1u) sc = __fmaf_rn(sPi[s], acc[s], sc);
            J.catLikes[(size_t)pp * TNC + c] = sc;
        }
        for (int k = 0; k < TNC; k++) {
            if (c == k) {
                float like32 = (k == 0) ? 0.0f : sChain[row];
#pragma unroll
                for (int s = 0; s < TD; s++)
                    if ((rmask >> s) & 1u) like32 = __fmaf_rn(sPi[s], acc[s], like32);
                sChain[row] = like32;
            }
            __syncthreads();
        }
        double v = 0.0;
        int bad = 0;
        if (c == TNC - 1) {
            const float like32 = sChain[row];
            const int pc = valid ? pp : J.nPat - 1;
            const double cnt = J.counts[pc];
            const uint32_t im = (J.pInvar != 0.0) ? J.invMask[pc] : 0u;
            double lnl;
            bool badk;
            if (im) {
                double lt = __dmul_rn(ldexp((double)like32, -E), J.varScale);
                for (int s = 0; s < TD; s++)
                    if ((im >> s) & 1u) lt = __dadd_rn(lt, __dmul_rn(J.rootComp[s], J.pInvar));
                badk = !(lt > 0.0);
                lnl = log(lt);
            } else {
                badk = !(like32 > 0.0f);
                int e;
                const float m = frexp32(like32, &e);
                lnl = (double)logf(m) + (double)(e - E) * LN2 + J.logScale;
            }
            if (valid && J.likeScaled) {
                J.likeScaled[pp] = like32;
                J.exps[pp] = E;
                J.lnl[pp] = lnl;
            }
            if (valid && !badk) v = cnt * lnl;
            bad = valid && badk;
            for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if ((tid & 31) == 0) sRed[warp & 3] = v;
        }
        const int anyBad = (__syncthreads_or(bad) ? 1 : 0) | (sAbort ? 2 : 0) | (__syncthreads_or(oob) ? 4 : 0);
        if (tid == 0) {
            const double s = sRed[0] + sRed[1] + sRed[2] + sRed[3];
            J.partials[bd.blk] = s;
            if (anyBad) atomicOr(J.badFlag, anyBad);
            __threadfence();
            const int t = atomicAdd(J.ticket, 1);
            sLast = (t == J.nBlocks - 1);
        }
        __syncthreads();
        if (sLast && tid < 32) {
            __threadfence();
            double s = 0.0;
            for (int i = tid; i < J.nBlocks; i += 32) s += __ldcg(J.partials + i);
            for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (tid == 0) {
                const int badAny = atomicExch(J.badFlag, 0);
                *J.out = (badAny & 6) ? __longlong_as_double(0x7ff8000000000000LL) : (badAny ? -1.0e99 : s);
                atomicExch(J.ticket, 0);
            }
        }
    }
    (void)timedOut;
    cpAsyncWaitAll();
    // a bulk copy still in flight (after an aborted tile) lands before the
    // block's shared memory is released; the wait is bounded like the others
    if (row == 0 && bPending) (void)tc::mbarWait(&sBarB[c], bPhase);
    tc::fenceBeforeSync();
    __syncthreads();
    if (warp == 0) tc::tmemDealloc(sTmem, TMEM_COLS);
}

}  // namespace

int pruneTcSmemBytes(int nProg, int nTax, int nSlots, int nClade)
{
    const int t = tcLayout(nProg, nTax, nSlots, nClade).total;
    return t <= TC_DYN_SMEM_MAX ? t : 227 * 1024 + 1;   // too large: callers take another shape
}

int launchPruneTc(const PruneJob *dJobs, const BlockDesc *dBlocks, int nTiles, int smemBytes, cudaStream_t s,
                  const int *nTilesDev, int early)
{
    (void)early;   // an ordinary launch: the stream orders it after the previous kernel
    static int configured = 0;
    if (configured < smemBytes) {
        P4G_CUDA(cudaFuncSetAttribute(k_prune_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBytes));
        configured = smemBytes;
    }
    // one block per SM: each block holds all 512 tensor-memory columns
    const int grid = nTiles < ctx().nSM ? nTiles : ctx().nSM;
    k_prune_tc<<<grid, 512, smemBytes, s>>>(dJobs, dBlocks, nTiles, nTilesDev);
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

}  // namespace p4g
