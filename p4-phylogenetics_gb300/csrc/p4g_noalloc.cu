// Log likelihood of a tree without allocating device memory.
//
// Who needs this: code that runs inside a host program whose device memory
// belongs to another allocator -- a framework's caching pool, or an arena
// that a service with a fixed memory budget reserves up front.  Such code
// may not call cudaMalloc itself: the pool can already hold nearly all of the
// device's memory, so a fresh cudaMalloc fails, and cudaMalloc / cudaFree
// synchronise the whole device, stalling everything else the program runs.
//
// p4g_treeLogLikeNoAlloc does the evaluation of p4g_setPrams(t, -1) followed
// by p4g_treeLogLike(t, 0, lnL) -- parameter values, eigensystems, gamma
// rates, P decks, compact tip codes, and the fused pruning kernel's per-tile
// partial sums, completion tickets and failure flags -- inside one fixed
// array declared below, `g_scratch`.  The array is part of the library's
// device image: it exists once the library's code is loaded on a device, and
// no call allocates or frees device memory, pinned memory or a memory pool.
// The inputs are staged in a fixed host array of the same size; that array is
// pageable, so the driver copies it through its own pinned buffers and the
// copy blocks the calling thread.
//
// The kernels are the library's own (k_gammaEig, k_pdeck, k_prune); only the
// memory they are pointed at differs.  The tree's own device state (the one
// p4g_treeLogLike uses) is neither read nor written.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <mutex>
#include <vector>
#include "p4g_internal.h"
#include "p4g_pmat.cuh"

using namespace p4g;

namespace {

constexpr size_t kScratchBytes = P4G_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// Every call on a device uses this array; see the race note at the entry point.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host staging of everything the kernels read (the first part of g_scratch).
alignas(256) static unsigned char g_stage[kScratchBytes];

// Device address of g_scratch, looked up once per device.
static void *g_scratchPtr[kMaxDevices];
static std::mutex g_lock;

inline size_t up256(size_t x) { return (x + 255) / 256 * 256; }

// Offsets of one call's regions inside the array.  Regions [0, imgBytes) are
// copied from g_stage; [imgBytes, total) are written by the kernels and
// cleared first.
struct Layout {
    size_t desc, jobs, prefix, eigTasks, gammaTasks, brLen, nodeIdx, isLeaf, prog, blocks;
    size_t out, ticket, bad, status;   // must start at zero: part of the staged image
    std::vector<size_t> comps, R, gval, codes, counts, invMask, partialMask;
    size_t imgBytes;
    std::vector<size_t> rates, eig, decks32, decks64, eqTab, partials;
    size_t total;
};

int scratchAddress(void **ptr)
{
    int dev = -1;
    P4G_CUDA(cudaGetDevice(&dev));
    if (dev != ctx().device)
        return setError(P4G_ESTATE, "treeLogLikeNoAlloc: current device %d is not the library's device %d", dev,
                        ctx().device);
    if (dev < 0 || dev >= kMaxDevices)
        return setError(P4G_EUNSUPPORTED, "treeLogLikeNoAlloc: device index %d beyond %d", dev, kMaxDevices);
    if (!g_scratchPtr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p)
            return setError(P4G_ECUDA, "treeLogLikeNoAlloc: cudaGetSymbolAddress of the scratch array: %s",
                            cudaGetErrorString(e));
        g_scratchPtr[dev] = p;
    }
    *ptr = g_scratchPtr[dev];
    return P4G_OK;
}

}  // namespace

#define RET(call)                      \
    do {                               \
        int rc_ = (call);              \
        if (rc_ != P4G_OK) return rc_; \
    } while (0)

extern "C" int p4g_treeLogLikeNoAlloc(p4g_tree *tt, double *lnL)
{
    Tree *t = reinterpret_cast<Tree *>(tt);
    if (!t || !lnL) return setError(P4G_EINVAL, "treeLogLikeNoAlloc: null argument");
    RET(ensureCtx());
    RET(validateModel(t, -1));
    Model *m = t->model;
    Data *d = t->data;
    const int nP = t->nParts, nn = t->nNodes, nTax = d->nTax;
    for (int p = 0; p < nP; p++) {
        Part *dp = d->parts[p];
        if (!dp) return setError(P4G_ESTATE, "data part %d missing", p);
        if (!dp->patternsMade) return setError(P4G_ESTATE, "part %d has no patterns (makePatterns not called)", p);
        if (m->parts[p].dim != dp->dim)
            return setError(P4G_EINVAL, "part %d: model dim %d != data dim %d", p, m->parts[p].dim, dp->dim);
        if (dp->nTax != nTax) return setError(P4G_EINVAL, "part %d: nTax mismatch", p);
    }

    std::lock_guard<std::mutex> hold(g_lock);
    void *scratch = nullptr;
    RET(scratchAddress(&scratch));

    for (int p = 0; p < nP; p++) {
        Part *dp = d->parts[p];
        if (!dp->invarMade) RET(p4g_setGlobalInvarSitesVec(reinterpret_cast<p4g_part *>(dp)));
        buildCompact(dp);
        if (dp->dim + 1 + dp->nPartial > 255)
            return setError(P4G_EUNSUPPORTED, "too many equates for 8-bit codes");
    }
    std::vector<int> prog;
    int nSlots = 0;
    RET(buildProgram(t, prog, nSlots));

    // ---------------------------------------------------------- layout
    Layout L;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o = up256(o + std::max<size_t>(bytes, 1));
        return at;
    };
    size_t nPairs = 0, nGd = 0;
    for (int p = 0; p < nP; p++) {
        nPairs += (size_t)m->parts[p].nComps * m->parts[p].nRMatrices;
        nGd += m->parts[p].nGdasrvs;
    }
    std::vector<int> shape(nP), tile(nP), nPatPad(nP), nBlk(nP);
    int totalBlocks = 0;
    for (int p = 0; p < nP; p++) {
        shape[p] = defaultShape(m->parts[p].dim);
        tile[p] = pruneTile(m->parts[p].dim, shape[p]);
        nPatPad[p] = (d->parts[p]->nPatterns + 511) / 512 * 512;   // the largest tile is 512 patterns
        nBlk[p] = (d->parts[p]->nPatterns + tile[p] - 1) / tile[p];
        totalBlocks += nBlk[p];
    }
    L.desc = take(sizeof(PmatPart) * nP);
    L.jobs = take(sizeof(PruneJob) * nP);
    L.prefix = take(sizeof(int) * nP);
    L.eigTasks = take(sizeof(int2) * nPairs);
    L.gammaTasks = take(sizeof(int2) * nGd);
    L.brLen = take(sizeof(double) * nn);
    L.nodeIdx = take(sizeof(int) * (size_t)nn * nP * 3);
    L.isLeaf = take(sizeof(int) * nn);
    L.prog = take(sizeof(int) * prog.size());
    L.blocks = take(sizeof(BlockDesc) * totalBlocks);
    L.out = take(sizeof(double) * nP);
    L.ticket = take(sizeof(int) * nP);
    L.bad = take(sizeof(int) * nP);
    L.status = take(sizeof(int));
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        const Part *dp = d->parts[p];
        L.comps.push_back(take(sizeof(double) * mp.nComps * mp.dim));
        L.R.push_back(take(sizeof(double) * (size_t)mp.nRMatrices * mp.dim * mp.dim));
        L.gval.push_back(take(sizeof(double) * std::max(mp.nGdasrvs, 1)));
        L.codes.push_back(take((size_t)nTax * nPatPad[p]));
        L.counts.push_back(take(sizeof(double) * dp->nPatterns));
        L.invMask.push_back(take(sizeof(uint32_t) * dp->nPatterns));
        L.partialMask.push_back(take(sizeof(uint32_t) * (dp->nPartial + 1)));
    }
    L.imgBytes = o;
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        const int dim = mp.dim;
        const size_t nDeck = ((size_t)nn * mp.nCat * dim * dim + 3) / 4 * 4;
        L.rates.push_back(take(sizeof(double) * std::max(mp.nGdasrvs, 1) * mp.nCat));
        L.eig.push_back(take(sizeof(double) * mp.nComps * mp.nRMatrices * eigRecDoubles(dim)));
        L.decks32.push_back(take(sizeof(float) * nDeck));
        L.decks64.push_back(take(sizeof(double) * nDeck));
        L.eqTab.push_back(take(sizeof(float) * (size_t)nn * std::max(d->parts[p]->nPartial, 1) * mp.nCat * dim));
        L.partials.push_back(take(sizeof(double) * nBlk[p]));
    }
    L.total = o;
    if (L.total > kScratchBytes)
        return setError(P4G_EUNSUPPORTED,
                        "treeLogLikeNoAlloc: this tree and data need %zu bytes of scratch; the fixed array "
                        "holds %zu (P4G_NOALLOC_SCRATCH_BYTES).  Use p4g_treeLogLike instead",
                        L.total, kScratchBytes);
    // Everything that can reject the call is checked here, before any work is
    // queued on the stream.
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        if (!pruneKernelExists(mp.dim, mp.nCat, shape[p]))
            return setError(P4G_EUNSUPPORTED, "treeLogLikeNoAlloc: no fused pruning kernel for dim=%d nCat=%d",
                            mp.dim, mp.nCat);
        const int smem = pruneSmemBytes(mp.dim, mp.nCat, (int)prog.size(), nn, nTax, nSlots, shape[p]);
        if (smem > 227 * 1024)
            return setError(P4G_EUNSUPPORTED, "tree too large for the fused kernel's shared memory (%d bytes)",
                            smem);
    }

    // ---------------------------------------------------------- host staging
    unsigned char *h = g_stage;
    char *g = (char *)scratch;
    memset(h, 0, L.imgBytes);   // also zeroes out, ticket, bad and status
    double *brLen = (double *)(h + L.brLen);
    int *nodeIdx = (int *)(h + L.nodeIdx);
    int *isLeaf = (int *)(h + L.isLeaf);
    for (int v = 0; v < nn; v++) {
        Node *n = t->nodes[v];
        brLen[v] = n ? n->brLen : 0.0;
        isLeaf[v] = n ? n->isLeaf : 0;
        for (int p = 0; p < nP; p++) {
            int *x = nodeIdx + ((size_t)v * nP + p) * 3;
            x[0] = n ? n->compNums[p] : 0;
            x[1] = n ? n->rMatrixNums[p] : 0;
            x[2] = n ? n->gdasrvNums[p] : 0;
        }
    }
    memcpy(h + L.prog, prog.data(), sizeof(int) * prog.size());
    PmatPart *desc = (PmatPart *)(h + L.desc);
    PruneJob *jobs = (PruneJob *)(h + L.jobs);
    int *prefix = (int *)(h + L.prefix);
    int2 *eigTasks = (int2 *)(h + L.eigTasks);
    int2 *gammaTasks = (int2 *)(h + L.gammaTasks);
    BlockDesc *blocks = (BlockDesc *)(h + L.blocks);
    int nE = 0, nG = 0, nD = 0, maxDim = 0, nb = 0;
    Node *rootNode = t->nodes[t->root];
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        const Part *dp = d->parts[p];
        const int dim = mp.dim;
        double *comps = (double *)(h + L.comps[p]);
        for (int c = 0; c < mp.nComps; c++) memcpy(comps + c * dim, mp.comps[c].val, sizeof(double) * dim);
        double *R = (double *)(h + L.R[p]);
        for (int r = 0; r < mp.nRMatrices; r++)
            memcpy(R + (size_t)r * dim * dim, mp.rMatrices[r].bigR.data(), sizeof(double) * dim * dim);
        double *gv = (double *)(h + L.gval[p]);
        for (int k = 0; k < mp.nGdasrvs; k++) gv[k] = mp.gdasrvs[k]->val[0];
        // tip codes, weights, invariant masks, partial-equate masks
        uint8_t *codes = h + L.codes[p];
        for (int x = 0; x < nTax; x++)
            for (int k = 0; k < dp->nPatterns; k++)
                codes[(size_t)x * nPatPad[p] + k] =
                    (uint8_t)compactCode(dp, dp->patterns[(size_t)x * dp->nPatterns + k]);
        double *cnt = (double *)(h + L.counts[p]);
        uint32_t *inv = (uint32_t *)(h + L.invMask[p]);
        for (int k = 0; k < dp->nPatterns; k++) {
            cnt[k] = (double)dp->counts[k];
            uint32_t msk = 0;
            for (int j = 0; j < dim; j++)
                if (dp->invArr[(size_t)j * dp->nPatterns + k]) msk |= 1u << j;
            inv[k] = msk;
        }
        if (dp->nPartial) memcpy(h + L.partialMask[p], dp->partialMask.data(), sizeof(uint32_t) * dp->nPartial);
        // setPrams descriptor: every eigensystem and every gamma rate set
        PmatPart &P = desc[p];
        P.comps = (const double *)(g + L.comps[p]);
        P.R = (const double *)(g + L.R[p]);
        P.gval = (const double *)(g + L.gval[p]);
        P.brLen = (const double *)(g + L.brLen);
        P.nodeIdx = (const int *)(g + L.nodeIdx);
        P.isLeaf = (const int *)(g + L.isLeaf);
        P.rates = (double *)(g + L.rates[p]);
        P.eig = (double *)(g + L.eig[p]);
        P.decks32 = (float *)(g + L.decks32[p]);
        P.eqTab = (float *)(g + L.eqTab[p]);
        P.decks64 = (double *)(g + L.decks64[p]);
        P.partialMask = (const uint32_t *)(g + L.partialMask[p]);
        P.pInvar = mp.pInvar;
        P.relRate = mp.relRate;
        P.dim = dim;
        P.nCat = mp.nCat;
        P.nComps = mp.nComps;
        P.nR = mp.nRMatrices;
        P.nG = mp.nGdasrvs;
        P.nNodes = nn;
        P.root = t->root;
        P.nPartial = dp->nPartial;
        P.partIdx = p;
        P.nParts = nP;
        for (int c = 0; c < mp.nComps; c++)
            for (int r = 0; r < mp.nRMatrices; r++) eigTasks[nE++] = make_int2(p, c * mp.nRMatrices + r);
        for (int k = 0; k < mp.nGdasrvs; k++) gammaTasks[nG++] = make_int2(p, k);
        prefix[p] = nD;
        nD += pdeckTasks(dim, nn, mp.nCat);
        maxDim = std::max(maxDim, dim);
        // pruning job
        PruneJob &J = jobs[p];
        J.decks = P.decks32;
        J.eqTab = P.eqTab;
        J.codes = (const uint8_t *)(g + L.codes[p]);
        J.counts = (const double *)(g + L.counts[p]);
        J.invMask = (const uint32_t *)(g + L.invMask[p]);
        J.partialMask = P.partialMask;
        J.prog = (const int *)(g + L.prog);
        J.rootComp = P.comps + (size_t)rootNode->compNums[p] * dim;
        J.partials = (double *)(g + L.partials[p]);
        J.out = (double *)(g + L.out) + p;
        J.ticket = (int *)(g + L.ticket) + p;
        J.badFlag = (int *)(g + L.bad) + p;
        J.pInvar = mp.pInvar;
        J.varScale = (1.0 - mp.pInvar) / (double)mp.nCat;
        J.logScale = (mp.pInvar != 0.0) ? log(J.varScale) : (mp.nCat > 1 ? log(1.0 / mp.nCat) : 0.0);
        J.nPat = dp->nPatterns;
        J.nPatPad = nPatPad[p];
        J.nPartial = dp->nPartial;
        J.nProg = (int)prog.size();
        J.nNodes = nn;
        J.nTax = nTax;
        J.nBlocks = nBlk[p];
        J.nSlots = nSlots;
        J.rootLeafRow = rootNode->isLeaf ? rootNode->seqNum : -1;
        J.dim = dim;
        J.nCat = mp.nCat;
        J.deckMap = nullptr;   // every deck and code row staged
        J.rowMap = nullptr;
        J.nDeck = nn;
        J.nRow = nTax;
        for (int b = 0; b < nBlk[p]; b++) blocks[nb + b] = BlockDesc{p, b * tile[p], b, 0};
        nb += nBlk[p];
    }

    // ---------------------------------------------------------- device work
    // From the first enqueue on, an error return first waits for the work
    // already queued, so that no kernel of this call still uses the shared
    // array once the lock is released.
    cudaStream_t s = ctx().stream;
    auto drain = [&](int rc) {
        cudaStreamSynchronize(s);
        return rc;
    };
#define RET_Q(call)                              \
    do {                                         \
        int rc_ = (call);                        \
        if (rc_ != P4G_OK) return drain(rc_);    \
    } while (0)
#define CUDA_Q(call)                                                                                  \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return drain(setError(P4G_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,               \
                                  cudaGetErrorString(e_)));                                           \
    } while (0)
    CUDA_Q(cudaMemcpyAsync(g, h, L.imgBytes, cudaMemcpyHostToDevice, s));
    CUDA_Q(cudaMemsetAsync(g + L.imgBytes, 0, L.total - L.imgBytes, s));
    RET_Q(launchPmat((const PmatPart *)(g + L.desc), (const int2 *)(g + L.eigTasks), nE,
                     (const int2 *)(g + L.gammaTasks), nG, (const int *)(g + L.prefix), nP, nD, maxDim,
                     (int *)(g + L.status), s));
    const PruneJob *dJobs = (const PruneJob *)(g + L.jobs);
    const BlockDesc *dBlocks = (const BlockDesc *)(g + L.blocks);
    nb = 0;
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        const int smem = pruneSmemBytes(mp.dim, mp.nCat, (int)prog.size(), nn, nTax, nSlots, shape[p]);
        RET_Q(launchPrune(dJobs, dBlocks + nb, nBlk[p], mp.dim, mp.nCat, smem, shape[p], s));
        nb += nBlk[p];
    }
    // results come back into the unused tail of the staging array (L.total
    // <= kScratchBytes leaves at least 256 bytes per part past the image)
    int status = 0;
    double *outp = (double *)(h + L.imgBytes);
    CUDA_Q(cudaMemcpyAsync(outp, g + L.out, sizeof(double) * nP, cudaMemcpyDeviceToHost, s));
    CUDA_Q(cudaMemcpyAsync(&status, g + L.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_Q(cudaStreamSynchronize(s));
#undef RET_Q
#undef CUDA_Q
    if (status)
        return setError(P4G_ENUMERIC, "setPrams: %s did not converge", (status & 1) ? "discrete gamma" : "eigensystem");
    for (int p = 0; p < nP; p++)
        if (outp[p] != outp[p]) return setError(P4G_ETIMEOUT, "pruning: a device-side check failed (a tensor-core completion wait gave up, or a clade-table index was out of range)");
    double sum = 0.0;
    for (int p = 0; p < nP; p++) {
        t->partLikes[p] = outp[p];
        sum += outp[p];
    }
    t->logLike = sum;
    *lnL = sum;
    return P4G_OK;
}
