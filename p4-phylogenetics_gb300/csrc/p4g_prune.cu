// Fused FP32 Felsenstein pruning: the whole post-order tree for a tile of
// site patterns in one block, one pattern per thread, every Gamma category
// of that pattern in the thread's registers.
//
// Reference loop: p4_setConditionalLikelihoodsOfInternalNodePart
// (Pf/p4_node.c:636-857) for every internal node in post-order
// (Pf/p4_tree.c:868-922), then the root reduction p4_partLogLike /
// p4_partLogLikeLoop / p4_partLogLikeLoopRootLeaf (Pf/p4_tree.c:924-1378).
//
// The reference stores every internal node's conditional likelihoods
// (cl[part][cat][state][pattern], FP64) in memory.  Here a host-built
// program walks the tree with a small stack: a node's running product lives
// in registers, only partial products that wait for a second internal child
// are pushed to shared memory, and nothing but the per-block lnL partial
// sum is written to HBM.  HBM traffic is the tip codes (one byte per taxon
// per pattern) and the pattern weights.
//
// Numerics (the CPU mirror in the oracle follows the same steps):
//   internal child : out[s] = P[s][0]*x[0], then fmaf(P[s][j], x[j], out[s])
//   tip child      : P[s][code] for a state, 1 for gap/?/N-like, a
//                    precomputed FP32 sum over members for other equates
//   node product   : internal children first (largest stack need first,
//                    then sibling order), tips in sibling order, one fp32
//                    multiply per factor
//   rescale        : when a pattern's largest entry (over categories and
//                    states) is below 2^-32, multiply by 2^k so it lands in
//                    [0.5, 1) and add k to the pattern's integer exponent E
//   root           : like32 = fmaf over (cat, state) of pi[s]*cl, then
//                    lnl = logf(m) + (e - E) ln2 + log(scale) in FP64 with
//                    like32 = m 2^e; patterns that can be invariant under a
//                    pInvar model take an FP64 path; the pattern-weighted sum
//                    is FP64 with a fixed-order block reduction.
#include <cuda_runtime.h>
#include <algorithm>
#include "p4g_internal.h"
#include "p4g_prune_common.cuh"

namespace p4g {

bool g_pdl = true;

template <bool S>
__device__ __forceinline__ float ldP(const float *p)
{
    if (S) return *p;
    return __ldg(p);
}

template <bool S>
__device__ __forceinline__ float4 ld4(const float *p)
{
    if (S) return *(const float4 *)p;
    return __ldg((const float4 *)p);
}

// Per-pattern rescale.  A pattern's values may be spread over the G lanes of
// its lane group (G = 1, 2, 4; groups are aligned within the warp): the
// group's maximum is the maximum of the lanes' maxima, so every lane takes
// the same decision and keeps the same exponent E.
template <int N, int G>
__device__ __forceinline__ void rescale(float (&acc)[N], int &E)
{
    float mx = 0.0f;
#pragma unroll
    for (int i = 0; i < N; i++) mx = fmaxf(mx, acc[i]);
#pragma unroll
    for (int o = 1; o < G; o <<= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (mx < 0x1p-32f && mx > 0.0f) {
        int e2;
        (void)frexp32(mx, &e2);
        int k = -e2;
        E += k;
        while (k > 0) {
            int step = k > 100 ? 100 : k;
            float f = __uint_as_float((unsigned)(127 + step) << 23);
#pragma unroll
            for (int i = 0; i < N; i++) acc[i] = __fmul_rn(acc[i], f);
            k -= step;
        }
    }
}

struct SmemLayout {
    int offProg, offDecks, offCodes, offIdx, offPi, offSlots, offRed, total;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

// tile = patterns per block pass (tp / g * ppt); every smem region is sized per tile
__host__ __device__ inline SmemLayout smemLayout(int nProg, int nNodes, int nTax, int dim, int nc,
                                                 int tp, int ppt, int g, int nSlots, bool sdeck, int nClade)
{
    SmemLayout L;
    const int tile = tp / g * ppt;
    int o = 0;
    L.offProg = o;
    o += nProg * 16;
    L.offDecks = o;
    if (sdeck) o += align16(nNodes * nc * dim * dim * 4);
    L.offCodes = o;
    o += align16(nTax * tile);
    L.offIdx = o;
    o += nClade * tile * 4;
    L.offPi = o;
    o += align16(dim * 4);
    L.offSlots = o;
    o += nSlots * nc * dim * tile * 4;
    L.offRed = o;
    o += (tp / 32) * 8 + 16;
    L.total = o;
    return L;
}

// One clade-table entry per pattern of this thread: the lane's categories of
// the clade's transformed product and the entry's scale exponent.
// An entry index at or past the table's end (which a stale or unfilled index
// row could hold) is not read: entry 0 is read instead and oob set.
template <int DIM, int NC, int NL, int PPT, int TPP>
__device__ __forceinline__ void cladeFetch(const PruneJob &J, const uint32_t *idxRow, int q, int c0,
                                           float (&v)[PPT][NL], int (&e)[PPT], int &oob)
{
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        uint32_t u = idxRow[q + k * TPP];
        if (u >= (uint32_t)J.nCladeEntries) {
            oob = 1;
            u = 0;
        }
        const float *src = J.cladeTab + ((size_t)u * NC + c0) * DIM;
        if (DIM % 4 == 0) {
#pragma unroll
            for (int i4 = 0; i4 < NL / 4; i4++) {
                const float4 w = __ldg((const float4 *)src + i4);
                v[k][4 * i4] = w.x;
                v[k][4 * i4 + 1] = w.y;
                v[k][4 * i4 + 2] = w.z;
                v[k][4 * i4 + 3] = w.w;
            }
        } else {
#pragma unroll
            for (int i = 0; i < NL; i++) v[k][i] = __ldg(src + i);
        }
        e[k] = __ldg(J.cladeExp + u);
    }
}

// One block walks tiles blockIdx.x, +gridDim.x, ...; the job's program and
// P decks are staged once per job change, the tip codes once per tile.
// A pattern is handled by a group of G adjacent lanes, lane g of the group
// holding categories [g*NC/G, (g+1)*NC/G); thread t works on patterns
// p0 + t/G + k*(TP/G) for k < PPT.  The arithmetic on every (category,
// state) value is the same for every G, so every tile shape gives the same
// per-pattern results.
// MB: resident blocks per SM the compiler keeps registers for (0: its own
// choice).  Tile shapes 11 and 12 hold the DNA lane-per-pattern kernels with 3
// or 4 categories to 3 blocks of 256 threads or 4 of 128 threads x 2 patterns,
// at the price of a few spilled words: more warps for the latency-bound
// clade-table and deck loads when many tiles are resident (batches of trees).
template <int DIM, int NC, int TP, int PPT, bool SDECK, int G, int MB = 0>
__global__ void __launch_bounds__(TP, MB)
k_prune(const PruneJob *__restrict__ jobs, const BlockDesc *__restrict__ blocks, int nTiles,
        const int *__restrict__ nTilesDev, int early)
{
    static_assert(NC % G == 0 && (G == 1 || G == 2 || G == 4), "lane groups must split the categories");
    // the wait on the previous kernel comes before the first read of what it
    // may have written (PDL_EARLY_* bits: what it does not write), so the
    // staging below can run while that kernel drains
    bool waited = false;
    auto waitPrev = [&]() {
        if (!waited) {
            pdlEnter();
            waited = true;
        }
    };
    if (!(early & PDL_EARLY_JOBS)) waitPrev();
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int CPT = NC / G;          // categories per thread
    constexpr int NL = CPT * DIM;        // values per thread and pattern
    constexpr int TPP = TP / G;          // patterns per block per pass
    constexpr int TILE = TPP * PPT;
    constexpr int N = NC * DIM;
    const int tid = threadIdx.x;
    const int q = tid / G;               // pattern slot in the pass
    const int g = tid % G;               // lane in the group
    const int c0 = g * CPT;              // first category of this lane
    __shared__ int sLast;
    int curJob = -1;
    SmemLayout L;
    int4 *sProg = nullptr;
    float *sDecks = nullptr;
    uint8_t *sCodes = nullptr;
    uint32_t *sIdx = nullptr;
    float *sPi = nullptr;
    float *sSlots = nullptr;
    double *sRed = nullptr;

    if (nTilesDev) nTiles = min(nTiles, *nTilesDev);
    for (int tile = blockIdx.x; tile < nTiles; tile += gridDim.x) {
        const BlockDesc bd = blocks[tile];
        const PruneJob &J = jobs[bd.job];
        const int nProg = J.nProg, nTax = J.nTax;
        __syncthreads();   // previous tile is done with the shared buffers
        if (bd.job != curJob) {
            L = smemLayout(nProg, J.deckMap ? J.nDeck : J.nNodes, J.rowMap ? J.nRow : nTax, DIM, NC, TP, PPT, G,
                           J.nSlots, SDECK, J.nClade);
            sProg = (int4 *)(smem + L.offProg);
            sDecks = (float *)(smem + L.offDecks);
            sCodes = smem + L.offCodes;
            sIdx = (uint32_t *)(smem + L.offIdx);
            sPi = (float *)(smem + L.offPi);
            sSlots = (float *)(smem + L.offSlots);
            sRed = (double *)(smem + L.offRed);
            // decode once: op, deck (or slot) offset, code-row offset
            const int *rowOf = J.rowMap;                        // taxon -> staged code row
            const int *deckOf = SDECK ? J.deckMap : nullptr;    // node -> shared-memory deck
            for (int i = tid; i < nProg; i += TP) {
                const int ins = J.prog[i];
                const int op = ins & 15, a = (ins >> 4) & 0x3fff, b = ins >> 18;
                const bool tip = op == OP_TIPSET || op == OP_TIPMUL;
                const bool deck = tip || op == OP_XFORM || op == OP_SCALE_XFORM;
                int4 d;
                d.x = op;
                d.y = (op == OP_PUSH || op == OP_MULSLOT) ? a * N * TILE
                                                          : ((deck && deckOf) ? deckOf[a] : a) * NC * DIM * DIM;
                d.z = ((tip && rowOf) ? rowOf[b] : b) * TILE;
                d.w = a;   // node: partial-equate tables are not staged
                if (op == OP_CHERRY) {   // table offset, both code rows
                    const int K = DIM + 1 + J.nPartial;
                    const int b2 = J.prog[i + 1] >> 18;
                    d.y = a * K * K * N;
                    d.z = (rowOf ? rowOf[b] : b) * TILE;
                    d.w = (rowOf ? rowOf[b2] : b2) * TILE;
                }
                if (op == OP_CLADE) d.y = a * TILE;   // the clade's index row in sIdx
                sProg[i] = d;
            }
            if (SDECK) {
                if (!(early & PDL_EARLY_DECKS)) waitPrev();
                constexpr int PER = N * DIM / 4;   // float4s of one node's deck
                const int *node = J.deckMap ? J.deckMap + J.nNodes : nullptr;
                const int n4 = (node ? J.nDeck : J.nNodes) * PER;
                const float4 *g4 = (const float4 *)J.decks;
                float4 *s4 = (float4 *)sDecks;
                for (int i = tid; i < n4; i += TP) {
                    const int k = i / PER;
                    s4[i] = __ldg(g4 + (size_t)(node ? node[k] : k) * PER + (i - k * PER));
                }
            }
            if (tid < DIM && !J.cladeOut) sPi[tid] = (float)J.rootComp[tid];   // clade jobs have no root
            curJob = bd.job;
        }
        {
            constexpr int V = TILE / 16;   // int4 chunks per taxon row
            const int *tax = J.rowMap ? J.rowMap + nTax : nullptr;
            const int total = (tax ? J.nRow : nTax) * V;
            for (int i = tid; i < total; i += TP) {
                int row = i / V, c = i % V;
                const int4 *src = (const int4 *)(J.codes + (size_t)(tax ? tax[row] : row) * J.nPatPad + bd.p0) + c;
                ((int4 *)(sCodes + row * TILE))[c] = __ldg(src);
            }
            const int totalIdx = J.nClade * (TILE / 4);   // table entries of each clade, this tile
            for (int i = tid; i < totalIdx; i += TP) {
                int row = i / (TILE / 4), c = i % (TILE / 4);
                const int4 *src = (const int4 *)(J.cladeIdx + (size_t)row * J.nPatPad + bd.p0) + c;
                ((int4 *)(sIdx + row * TILE))[c] = __ldg(src);
            }
        }
        int pp[PPT];
        bool valid[PPT];
        double cnt[PPT];
        uint32_t im[PPT];
#pragma unroll
        for (int k = 0; k < PPT; k++) {
            pp[k] = bd.p0 + q + k * TPP;
            valid[k] = pp[k] < J.nPat;
            const int pc = valid[k] ? pp[k] : J.nPat - 1;
            cnt[k] = J.counts[pc];
            im[k] = (J.pInvar != 0.0) ? J.invMask[pc] : 0u;
        }
        __syncthreads();
        waitPrev();   // the tables (and decks read through L1) of earlier kernels

        const float *decks = SDECK ? sDecks : J.decks;
        float acc[PPT][NL];
        int E[PPT];
#pragma unroll
        for (int k = 0; k < PPT; k++) {
            E[k] = 0;
#pragma unroll
            for (int i = 0; i < NL; i++) acc[k][i] = 1.0f;
        }
        // DNA: clade k's table entries are loaded one OP_CLADE ahead (clades
        // are numbered in read order), so the loads are in flight while the
        // ops before it run
        constexpr bool PF = DIM == 4;
        float pre[PPT][NL];
        int preE[PPT];
        int oob = 0;
        if (PF && J.nClade > 0) cladeFetch<DIM, NC, NL, PPT, TPP>(J, sIdx, q, c0, pre, preE, oob);

        for (int ip = 0; ip < nProg; ip++) {
            const int4 I = sProg[ip];
            switch (I.x) {
            case OP_TIPSET:
            case OP_TIPMUL: {
                const float *deck = decks + I.y + c0 * DIM * DIM;
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    const int code = sCodes[I.z + q + k * TPP];
                    float v[NL];
                    if (code < DIM) {
                        const float *col = deck + code * DIM;
                        if (DIM % 4 == 0) {
#pragma unroll
                            for (int c = 0; c < CPT; c++)
#pragma unroll
                                for (int s4 = 0; s4 < DIM / 4; s4++) {
                                    float4 w = ld4<SDECK>(col + c * DIM * DIM + 4 * s4);
                                    v[c * DIM + 4 * s4 + 0] = w.x;
                                    v[c * DIM + 4 * s4 + 1] = w.y;
                                    v[c * DIM + 4 * s4 + 2] = w.z;
                                    v[c * DIM + 4 * s4 + 3] = w.w;
                                }
                        } else {
#pragma unroll
                            for (int c = 0; c < CPT; c++)
#pragma unroll
                                for (int s = 0; s < DIM; s++) v[c * DIM + s] = ldP<SDECK>(col + c * DIM * DIM + s);
                        }
                    } else if (code == DIM) {
#pragma unroll
                        for (int i = 0; i < NL; i++) v[i] = 1.0f;
                    } else {
                        const float *eq =
                            J.eqTab + (((size_t)I.w * J.nPartial + (code - DIM - 1)) * NC + c0) * DIM;
#pragma unroll
                        for (int i = 0; i < NL; i++) v[i] = __ldg(eq + i);
                    }
                    if (I.x == OP_TIPSET) {
#pragma unroll
                        for (int i = 0; i < NL; i++) acc[k][i] = v[i];
                    } else {
#pragma unroll
                        for (int i = 0; i < NL; i++) acc[k][i] = __fmul_rn(acc[k][i], v[i]);
                    }
                }
                break;
            }
            case OP_CHERRY: {
                if (DIM < 20 || !J.cherryTab) {   // no table for this job: run the cherry's own ops
                    ip++;
                    break;
                }
                const int K = DIM + 1 + J.nPartial;
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    const int ca = sCodes[I.z + q + k * TPP], cb = sCodes[I.w + q + k * TPP];
                    const float *e = J.cherryTab + I.y + ((ca * K + cb) * NC + c0) * DIM;
                    if (DIM % 4 == 0) {
#pragma unroll
                        for (int i4 = 0; i4 < NL / 4; i4++) {
                            const float4 w = __ldg((const float4 *)e + i4);
                            acc[k][4 * i4] = w.x;
                            acc[k][4 * i4 + 1] = w.y;
                            acc[k][4 * i4 + 2] = w.z;
                            acc[k][4 * i4 + 3] = w.w;
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < NL; i++) acc[k][i] = __ldg(e + i);
                    }
                }
                ip += 4;   // the OP_ARG word and the cherry's TIPSET, TIPMUL, SCALE_XFORM
                break;
            }
            case OP_CLADE: {
                if constexpr (PF) {
#pragma unroll
                    for (int k = 0; k < PPT; k++) {
#pragma unroll
                        for (int i = 0; i < NL; i++) acc[k][i] = pre[k][i];
                        E[k] += preE[k];
                    }
                    if (I.w + 1 < J.nClade)
                        cladeFetch<DIM, NC, NL, PPT, TPP>(J, sIdx + (I.w + 1) * TILE, q, c0, pre, preE, oob);
                } else {
                    int e[PPT];
                    cladeFetch<DIM, NC, NL, PPT, TPP>(J, sIdx + I.y, q, c0, acc, e, oob);
#pragma unroll
                    for (int k = 0; k < PPT; k++) E[k] += e[k];
                }
                break;
            }
            case OP_SCALE_XFORM:
#pragma unroll
                for (int k = 0; k < PPT; k++) rescale<NL, G>(acc[k], E[k]);
                [[fallthrough]];
            case OP_XFORM: {
                const float *P = decks + I.y + c0 * DIM * DIM;
#pragma unroll
                for (int c = 0; c < CPT; c++) {
                    float x[PPT][DIM];
#pragma unroll
                    for (int k = 0; k < PPT; k++)
#pragma unroll
                        for (int j = 0; j < DIM; j++) x[k][j] = acc[k][c * DIM + j];
                    const float *Pc = P + c * DIM * DIM;
                    if (DIM % 4 == 0) {
#pragma unroll
                        for (int s = 0; s < DIM; s++) {
                            float t[PPT];
                            float4 w = ld4<SDECK>(Pc + s * DIM);
#pragma unroll
                            for (int k = 0; k < PPT; k++) {
                                t[k] = __fmul_rn(w.x, x[k][0]);
                                t[k] = __fmaf_rn(w.y, x[k][1], t[k]);
                                t[k] = __fmaf_rn(w.z, x[k][2], t[k]);
                                t[k] = __fmaf_rn(w.w, x[k][3], t[k]);
                            }
#pragma unroll
                            for (int j4 = 1; j4 < DIM / 4; j4++) {
                                w = ld4<SDECK>(Pc + s * DIM + 4 * j4);
#pragma unroll
                                for (int k = 0; k < PPT; k++) {
                                    t[k] = __fmaf_rn(w.x, x[k][4 * j4 + 0], t[k]);
                                    t[k] = __fmaf_rn(w.y, x[k][4 * j4 + 1], t[k]);
                                    t[k] = __fmaf_rn(w.z, x[k][4 * j4 + 2], t[k]);
                                    t[k] = __fmaf_rn(w.w, x[k][4 * j4 + 3], t[k]);
                                }
                            }
#pragma unroll
                            for (int k = 0; k < PPT; k++) acc[k][c * DIM + s] = t[k];
                        }
                    } else {
#pragma unroll
                        for (int s = 0; s < DIM; s++) {
                            float t[PPT];
                            const float p0 = ldP<SDECK>(Pc + s * DIM);
#pragma unroll
                            for (int k = 0; k < PPT; k++) t[k] = __fmul_rn(p0, x[k][0]);
#pragma unroll
                            for (int j = 1; j < DIM; j++) {
                                const float pj = ldP<SDECK>(Pc + s * DIM + j);
#pragma unroll
                                for (int k = 0; k < PPT; k++) t[k] = __fmaf_rn(pj, x[k][j], t[k]);
                            }
#pragma unroll
                            for (int k = 0; k < PPT; k++) acc[k][c * DIM + s] = t[k];
                        }
                    }
                }
                break;
            }
            case OP_PUSH: {
                float *sl = sSlots + I.y + tid;
#pragma unroll
                for (int k = 0; k < PPT; k++)
#pragma unroll
                    for (int i = 0; i < NL; i++) sl[i * (TP * PPT) + k * TP] = acc[k][i];
                break;
            }
            case OP_MULSLOT: {
                const float *sl = sSlots + I.y + tid;
#pragma unroll
                for (int k = 0; k < PPT; k++)
#pragma unroll
                    for (int i = 0; i < NL; i++) acc[k][i] = __fmul_rn(acc[k][i], sl[i * (TP * PPT) + k * TP]);
                break;
            }
            default: {   // OP_SCALE
#pragma unroll
                for (int k = 0; k < PPT; k++) rescale<NL, G>(acc[k], E[k]);
                break;
            }
            }
        }

        if (J.cladeOut) {   // clade-table job: the transformed product and its exponent
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                if (!valid[k]) continue;
                float *o = J.cladeOut + ((size_t)pp[k] * NC + c0) * DIM;
#pragma unroll
                for (int i = 0; i < NL; i++) o[i] = acc[k][i];
                if (g == 0) J.cladeOutExp[pp[k]] = E[k];
            }
            continue;
        }

        // ---- root reduction: one fmaf chain over (category, state) in
        // category order, carried from lane to lane through the group
        double v = 0.0;
        int bad = 0;
        const int lane = tid & 31;
        const int base = lane & ~(G - 1);
        const int rootRow = (J.rootLeafRow >= 0 && J.rowMap) ? J.rowMap[J.rootLeafRow] : J.rootLeafRow;
#pragma unroll
        for (int k = 0; k < PPT; k++) {
            uint32_t rmask = (DIM >= 32) ? 0xffffffffu : ((1u << DIM) - 1u);
            if (rootRow >= 0) {
                const int code = sCodes[rootRow * TILE + q + k * TPP];
                if (code < DIM) rmask = 1u << code;
                else if (code > DIM) rmask = J.partialMask[code - DIM - 1];
            }
            float like32 = 0.0f;
#pragma unroll
            for (int j = 0; j < G; j++) {
                if (g == j) {
#pragma unroll
                    for (int c = 0; c < CPT; c++)
#pragma unroll
                        for (int s = 0; s < DIM; s++)
                            if ((rmask >> s) & 1u) like32 = __fmaf_rn(sPi[s], acc[k][c * DIM + s], like32);
                }
                if (G > 1 && j < G - 1) {
                    const float nxt = __shfl_sync(0xffffffffu, like32, base + j);
                    if (g == j + 1) like32 = nxt;
                }
            }
            if (G > 1) like32 = __shfl_sync(0xffffffffu, like32, base + G - 1);
            if (J.rootCL && valid[k]) {   // root partials for ancestral-state draws
                float *o = J.rootCL + ((size_t)pp[k] * NC + c0) * DIM;
#pragma unroll
                for (int i = 0; i < NL; i++) o[i] = ((rmask >> (i % DIM)) & 1u) ? acc[k][i] : 0.0f;
            }
            if (J.catLikes && valid[k]) {   // per-category sums for site rates
#pragma unroll
                for (int c = 0; c < CPT; c++) {
                    float sc = 0.0f;
#pragma unroll
                    for (int s = 0; s < DIM; s++)
                        if ((rmask >> s) & 1u) sc = __fmaf_rn(sPi[s], acc[k][c * DIM + s], sc);
                    J.catLikes[(size_t)pp[k] * NC + c0 + c] = sc;
                }
            }
            double lnl;
            bool badk;
            if (im[k]) {
                double lt = __dmul_rn(ldexp((double)like32, -E[k]), J.varScale);
                for (int s = 0; s < DIM; s++)
                    if ((im[k] >> s) & 1u) lt = __dadd_rn(lt, __dmul_rn(J.rootComp[s], J.pInvar));
                badk = !(lt > 0.0);
                lnl = log(lt);
            } else {
                badk = !(like32 > 0.0f);
                int e;
                float m = frexp32(like32, &e);
                lnl = (double)logf(m) + (double)(e - E[k]) * LN2 + J.logScale;
            }
            const bool mine = valid[k] && g == 0;
            if (mine && J.likeScaled) {
                J.likeScaled[pp[k]] = like32;
                J.exps[pp[k]] = E[k];
                J.lnl[pp[k]] = lnl;
            }
            if (mine && !badk) v += cnt[k] * lnl;
            bad |= (mine && badk);
        }
        const int anyBad = (__syncthreads_or(bad) ? 1 : 0) | (__syncthreads_or(oob) ? 4 : 0);

        // ---- tile reduction (fixed order) and last-tile-done finish per job
        for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) sRed[tid >> 5] = v;
        __syncthreads();
        if (tid == 0) {
            double s = 0.0;
            for (int w = 0; w < TP / 32; w++) s += sRed[w];
            J.partials[bd.blk] = s;
            if (anyBad) atomicOr(J.badFlag, anyBad);
            __threadfence();
            int t = atomicAdd(J.ticket, 1);
            sLast = (t == J.nBlocks - 1);
        }
        __syncthreads();
        if (sLast && tid < 32) {
            __threadfence();
            double s = 0.0;
            for (int i = tid; i < J.nBlocks; i += 32) s += __ldcg(J.partials + i);
            for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (tid == 0) {
                int badAny = atomicExch(J.badFlag, 0);
                *J.out = (badAny & 4) ? __longlong_as_double(0x7ff8000000000000LL) : (badAny ? -1.0e99 : s);
                atomicExch(J.ticket, 0);
            }
        }
    }
}

// Cherry tables of one evaluation: for every job, cherry (node v with leaf
// children a, b), code pair (ca, cb) and category, the transformed product
// XFORM_v(TIPSET(a, ca) * TIPMUL(b, cb)) with exactly the FP32 operations
// the program would run (no rescale in between: the values are products of
// two probabilities, far from FP32's range limits, and a later rescale point
// scales them by the same exact power of two).
__device__ __forceinline__ void tipColumn(const PruneJob &J, int leaf, int code, int cat, float *v)
{
    const int D = J.dim, NC = J.nCat;
    if (code < D) {
        const float *col = J.decks + ((size_t)leaf * NC + cat) * D * D + code * D;
        for (int i = 0; i < D; i++) v[i] = col[i];
    } else if (code == D) {
        for (int i = 0; i < D; i++) v[i] = 1.0f;
    } else {
        const float *eq = J.eqTab + (((size_t)leaf * J.nPartial + (code - D - 1)) * NC + cat) * D;
        for (int i = 0; i < D; i++) v[i] = eq[i];
    }
}

// A tip column with the state count known at compile time (float4 reads; the
// column stays in registers).
template <int D>
__device__ __forceinline__ void tipColumnT(const PruneJob &J, int leaf, int code, int cat, float (&v)[D])
{
    const int NC = J.nCat;
    if (code < D) {
        const float4 *col = (const float4 *)(J.decks + ((size_t)leaf * NC + cat) * D * D + code * D);
#pragma unroll
        for (int i = 0; i < D / 4; i++) {
            const float4 q = __ldg(col + i);
            v[4 * i] = q.x;
            v[4 * i + 1] = q.y;
            v[4 * i + 2] = q.z;
            v[4 * i + 3] = q.w;
        }
    } else if (code == D) {
#pragma unroll
        for (int i = 0; i < D; i++) v[i] = 1.0f;
    } else {
        const float4 *eq = (const float4 *)(J.eqTab + (((size_t)leaf * J.nPartial + (code - D - 1)) * NC + cat) * D);
#pragma unroll
        for (int i = 0; i < D / 4; i++) {
            const float4 q = __ldg(eq + i);
            v[4 * i] = q.x;
            v[4 * i + 1] = q.y;
            v[4 * i + 2] = q.z;
            v[4 * i + 3] = q.w;
        }
    }
}

// One block per (job, cherry, category): the node's P deck of that category is
// staged in shared memory (every thread's rows are the same, so they are read
// as broadcasts), and the threads take the K x K code pairs.
template <int D>
__device__ __forceinline__ void cherryBlockT(const PruneJob &J, int c, int cat, float *sP)
{
    static_assert(D % 4 == 0, "float4 rows");
    const int NC = J.nCat, K = D + 1 + J.nPartial;
    const int4 ch = J.cherries[c];
    const float4 *P = (const float4 *)(J.decks + ((size_t)ch.x * NC + cat) * D * D);
    float4 *sP4 = (float4 *)sP;
    for (int k = threadIdx.x; k < D * D / 4; k += blockDim.x) sP4[k] = __ldg(P + k);
    __syncthreads();
    for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
        const int ca = e / K, cb = e - ca * K;
        float x[D], y[D];
        tipColumnT<D>(J, ch.y, ca, cat, x);
        tipColumnT<D>(J, ch.z, cb, cat, y);
#pragma unroll
        for (int i = 0; i < D; i++) x[i] = __fmul_rn(x[i], y[i]);
        float4 *out = (float4 *)(J.cherryTab + ((((size_t)c * K + ca) * K + cb) * NC + cat) * D);
#pragma unroll
        for (int s4 = 0; s4 < D / 4; s4++) {
            float o[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int s = 4 * s4 + u;
                float t = 0.f;
#pragma unroll
                for (int j4 = 0; j4 < D / 4; j4++) {
                    const float4 q = sP4[(s * D) / 4 + j4];
                    if (j4 == 0) t = __fmul_rn(q.x, x[0]);
                    else t = __fmaf_rn(q.x, x[4 * j4], t);
                    t = __fmaf_rn(q.y, x[4 * j4 + 1], t);
                    t = __fmaf_rn(q.z, x[4 * j4 + 2], t);
                    t = __fmaf_rn(q.w, x[4 * j4 + 3], t);
                }
                o[u] = t;
            }
            out[s4] = make_float4(o[0], o[1], o[2], o[3]);
        }
    }
}

// The same for a state count known only at run time.
__device__ void cherryBlock(const PruneJob &J, int c, int cat, float *sP)
{
    const int D = J.dim, NC = J.nCat, K = D + 1 + J.nPartial;
    const int4 ch = J.cherries[c];
    const float *P = J.decks + ((size_t)ch.x * NC + cat) * D * D;
    for (int k = threadIdx.x; k < D * D; k += blockDim.x) sP[k] = P[k];
    __syncthreads();
    for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
        const int ca = e / K, cb = e - ca * K;
        float x[MAX_DIM], y[MAX_DIM];
        tipColumn(J, ch.y, ca, cat, x);
        tipColumn(J, ch.z, cb, cat, y);
        for (int i = 0; i < D; i++) x[i] = __fmul_rn(x[i], y[i]);
        float *out = J.cherryTab + ((((size_t)c * K + ca) * K + cb) * NC + cat) * D;
        for (int s = 0; s < D; s++) {
            float t = __fmul_rn(sP[s * D], x[0]);
            for (int j = 1; j < D; j++) t = __fmaf_rn(sP[s * D + j], x[j], t);
            out[s] = t;
        }
    }
}

// grid: (cherry-list capacity x the largest nCat, jobs)
__global__ void __launch_bounds__(256) k_cherry(const PruneJob *__restrict__ jobs)
{
    __shared__ __align__(16) float sP[MAX_DIM * MAX_DIM];
    const PruneJob &J = jobs[blockIdx.y];
    if (J.nCherry == 0 || !J.cherryTab) return;
    const int c = blockIdx.x / J.nCat, cat = blockIdx.x - c * J.nCat;
    if (c >= J.nCherry) return;   // block-uniform, before any barrier
    if (J.dim == 20) cherryBlockT<20>(J, c, cat, sP);
    else cherryBlock(J, c, cat, sP);
}

int launchCherry(const PruneJob *dJobs, int nJobs, long long cherryBlocks, cudaStream_t s)
{
    if (nJobs <= 0 || cherryBlocks <= 0) return P4G_OK;
    dim3 grid((unsigned)cherryBlocks, (unsigned)nJobs);
    k_cherry<<<grid, 256, 0, s>>>(dJobs);
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

// Tile shapes the autotuner chooses from, per state count: threads per
// block, patterns per thread, P decks staged in shared memory (else read
// through L1, which leaves shared memory to the codes and the stack and so
// raises the number of resident warps), and lanes per pattern (categories
// spread over 1, 2 or 4 lanes: more threads for the same patterns, which is
// what fills the GPU when the alignment has few patterns).  Every shape
// holds at least 64 patterns per tile.
struct PruneShape {
    int tp, ppt;
    bool sdeck;
    int g;
    bool tc;   // tensor-core kernel (k_prune_tc, p4g_prune_tc.cu)
    int mb;    // resident blocks per SM the registers are held to (0: free)
};
static const PruneShape kShapes4[] = {{128, 1, true, 1, false},  {128, 2, true, 1, false},
                                      {256, 1, true, 1, false},  {256, 1, false, 1, false},
                                      {128, 2, false, 1, false}, {512, 1, false, 1, false},
                                      {256, 1, false, 4, false}, {256, 1, false, 2, false},
                                      {128, 1, false, 2, false}, {256, 1, true, 4, false},
                                      {512, 1, false, 4, false}, {256, 1, true, 1, false, 3},
                                      {128, 2, true, 1, false, 4}};
// protein: shape 3 is the tensor-core kernel (4 categories only): 512
// threads, 4 lanes (one per category) per pattern, 128 patterns per tile
static const PruneShape kShapes20[] = {{64, 1, false, 1, false}, {256, 1, false, 4, false},
                                       {128, 1, false, 2, false}, {512, 1, false, 4, true}};
static const PruneShape kShapes2[] = {{128, 2, true, 1, false}};

int pruneNumShapes(int dim)
{
    return dim == 4 ? 13 : dim == 20 ? 4 : 1;
}

static PruneShape shapeOf(int dim, int shape)
{
    if (dim == 4) return kShapes4[shape];
    if (dim == 20) return kShapes20[shape];
    return kShapes2[0];
}

int pruneShapeValid(int dim, int nCat, int shape)
{
    if (shape < 0 || shape >= pruneNumShapes(dim)) return 0;
    if (shapeOf(dim, shape).mb && (nCat < 3 || nCat > 4)) return 0;   // register-held: 3 or 4 categories
    return nCat % shapeOf(dim, shape).g == 0;
}

int pruneTile(int dim, int shape)
{
    PruneShape s = shapeOf(dim, shape);
    return s.tp / s.g * s.ppt;
}

int pruneSmemBytes(int dim, int nCat, int nProg, int nNodes, int nTax, int nSlots, int shape, int nClade,
                   int nDeck, int nRow)
{
    PruneShape s = shapeOf(dim, shape);
    // the tensor-core kernel asks for at least 120 KB so that one block fits
    // per SM (each block allocates all 512 tensor-memory columns)
    if (s.tc) return std::max(pruneTcSmemBytes(nProg, nTax, nSlots, nClade), 120 * 1024);
    // the staging maps (nDeck decks, nRow code rows) apply to this kernel only
    return smemLayout(nProg, nDeck >= 0 ? nDeck : nNodes, nRow >= 0 ? nRow : nTax, dim, nCat, s.tp, s.ppt, s.g,
                      nSlots, s.sdeck, nClade)
        .total;
}

template <int DIM, int NC, int TP, int PPT, bool SDECK, int G, int MB = 0>
static int launchT(const PruneJob *dJobs, const BlockDesc *dBlocks, int nTiles, int smemBytes,
                   cudaStream_t s, const int *nTilesDev, int early)
{
    auto k = k_prune<DIM, NC, TP, PPT, SDECK, G, MB>;
    static int configured = 0;
    static int perSM = 0, perSMsmem = -1;
    if (smemBytes > 48 * 1024 && configured < smemBytes) {
        P4G_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBytes));
        configured = smemBytes;
    }
    if (perSMsmem != smemBytes) {
        P4G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k, TP, smemBytes));
        perSMsmem = smemBytes;
    }
    if (perSM < 1) return setError(P4G_EUNSUPPORTED, "pruning kernel does not fit on an SM (%d B smem)", smemBytes);
    int grid = std::min(nTiles, perSM * ctx().nSM);
    P4G_CUDA(launchPdl(k, dim3(grid), dim3(TP), smemBytes, s, dJobs, dBlocks, nTiles, nTilesDev, early));
    return P4G_OK;
}

#define P4G_L(D, C, TP, PPT, SD, G) \
    return launchT<D, C, TP, PPT, SD, G>(dJobs, dBlocks, nTiles, smemBytes, s, nTilesDev, early)
// shapes 0-5 (one lane per pattern) exist for every category count
#define P4G_CASE4_G1(C)                                  \
    case 0: P4G_L(4, C, 128, 1, true, 1);                \
    case 1: P4G_L(4, C, 128, 2, true, 1);                \
    case 2: P4G_L(4, C, 256, 1, true, 1);                \
    case 3: P4G_L(4, C, 256, 1, false, 1);               \
    case 4: P4G_L(4, C, 128, 2, false, 1);               \
    case 5: P4G_L(4, C, 512, 1, false, 1);
#define P4G_CASE4_G2(C)                                  \
    case 7: P4G_L(4, C, 256, 1, false, 2);               \
    case 8: P4G_L(4, C, 128, 1, false, 2);
#define P4G_LM(D, C, TP, PPT, SD, G, MB) \
    return launchT<D, C, TP, PPT, SD, G, MB>(dJobs, dBlocks, nTiles, smemBytes, s, nTilesDev, early)
#define P4G_CASE4_MB(C)                                  \
    case 11: P4G_LM(4, C, 256, 1, true, 1, 3);           \
    case 12: P4G_LM(4, C, 128, 2, true, 1, 4);
#define P4G_CASE4_G4(C)                                  \
    case 6: P4G_L(4, C, 256, 1, false, 4);               \
    case 9: P4G_L(4, C, 256, 1, true, 4);                \
    case 10: P4G_L(4, C, 512, 1, false, 4);

// 1 when launchPrune has a compiled kernel for (dim, nCat, shape): the same
// table as the switch below, for callers that must know before they queue
// any work.
int pruneKernelExists(int dim, int nCat, int shape)
{
    if (!pruneShapeValid(dim, nCat, shape)) return 0;
    if (dim == 4) {
        const bool g1 = shape <= 5, g2 = shape == 7 || shape == 8;
        const bool g4 = shape == 6 || shape == 9 || shape == 10, mb = shape == 11 || shape == 12;
        switch (nCat) {
        case 1: case 5: return g1;
        case 2: case 6: return g1 || g2;
        case 3: return g1 || mb;
        case 4: return g1 || g2 || g4 || mb;
        case 8: return g1 || g2 || g4;
        default: return 0;
        }
    }
    if (dim == 20) return (nCat == 1 && shape == 0) || (nCat == 4 && shape >= 0 && shape <= 3);
    if (dim == 2) return shape == 0 && (nCat == 1 || nCat == 4);
    return 0;
}

int launchPrune(const PruneJob *dJobs, const BlockDesc *dBlocks, int nTiles, int dim, int nCat,
                int smemBytes, int shape, cudaStream_t s, const int *nTilesDev, int early)
{
    if (nTiles <= 0) return P4G_OK;
    if (!pruneShapeValid(dim, nCat, shape))
        return setError(P4G_EUNSUPPORTED, "pruning tile shape %d does not apply to dim=%d nCat=%d", shape, dim,
                        nCat);
    if (dim == 4) {
        switch (nCat) {
        case 1: switch (shape) { P4G_CASE4_G1(1) } break;
        case 2: switch (shape) { P4G_CASE4_G1(2) P4G_CASE4_G2(2) } break;
        case 3: switch (shape) { P4G_CASE4_G1(3) P4G_CASE4_MB(3) } break;
        case 4: switch (shape) { P4G_CASE4_G1(4) P4G_CASE4_G2(4) P4G_CASE4_G4(4) P4G_CASE4_MB(4) } break;
        case 5: switch (shape) { P4G_CASE4_G1(5) } break;
        case 6: switch (shape) { P4G_CASE4_G1(6) P4G_CASE4_G2(6) } break;
        case 8: switch (shape) { P4G_CASE4_G1(8) P4G_CASE4_G2(8) P4G_CASE4_G4(8) } break;
        default: break;
        }
    } else if (dim == 20) {
        if (nCat == 1 && shape == 0) P4G_L(20, 1, 64, 1, false, 1);
        if (nCat == 4) {
            switch (shape) {
            case 0: P4G_L(20, 4, 64, 1, false, 1);
            case 1: P4G_L(20, 4, 256, 1, false, 4);
            case 2: P4G_L(20, 4, 128, 1, false, 2);
            case 3: return launchPruneTc(dJobs, dBlocks, nTiles, smemBytes, s, nTilesDev, early);
            default: break;
            }
        }
    } else if (dim == 2 && shape == 0) {
        if (nCat == 1) P4G_L(2, 1, 128, 2, true, 1);
        if (nCat == 4) P4G_L(2, 4, 128, 2, true, 1);
    }
    return setError(P4G_EUNSUPPORTED, "no fused pruning kernel for dim=%d nCat=%d shape %d", dim, nCat, shape);
}

}  // namespace p4g
