// Clade tables ("site repeats"): every maximal subtree with at most
// cladeSize leaves is evaluated once per distinct combination of its leaves'
// codes, not once per pattern.
//
// A pattern's value at a subtree's root depends only on the codes of the
// subtree's leaves, and a subtree of L leaves sees far fewer distinct code
// combinations than the alignment has patterns (at most min(nPatterns, K^L)
// with K codes).  For the current topology the host picks the maximal
// clades (non-root nodes with <= cladeSize leaves whose parent has more),
// emits each clade's own program (the same ops, in the same order, that the
// whole-tree program would run for that subtree, ending with the clade
// root's rescale + parent-edge transform), and per data part numbers the
// distinct leaf-code combinations of each clade in first-occurrence order.
// Each evaluation first runs the clade programs over those combinations
// (k_prune with the clade-table output), writing the transformed product and
// the scale exponent of every combination; the whole-tree program then reads
// one table entry per clade (OP_CLADE) instead of running its subtree.  The
// arithmetic of every pattern is unchanged, so per-pattern results are
// bit-identical with and without clade tables.
#include <cuda_runtime.h>
#include <string.h>
#include <algorithm>
#include <vector>
#include "p4g_internal.h"

using namespace p4g;

#define RET(call)                      \
    do {                               \
        int rc_ = (call);              \
        if (rc_ != P4G_OK) return rc_; \
    } while (0)

namespace {

inline size_t roundUp(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr int kMaxClades = 32;
constexpr unsigned long long kEmpty = ~0ull;   // no key: codes are below 0xff

// One (part, clade): where its combinations are numbered and its table job.
struct CladeTask {
    const uint8_t *codes;       // the part's tip codes [nTax][nPatPad]
    unsigned long long *keys;   // open-addressing table [hashSize], kEmpty-filled
    int *vals;                  // combination number of each occupied slot
    int *count;                 // combinations numbered so far (zeroed)
    int *nTiles;                // tiles listed so far in the group's list (zeroed)
    uint8_t *outCodes;          // the clade job's codes [nLeaf][nPatPad]
    uint32_t *idx;              // the whole-tree job's row [nPatPad]: table entry of each pattern
    PruneJob *job;              // the clade job (device); its nPat is written here
    BlockDesc *blocks;          // the group's tile list
    int nPat, nPatPad, hashSize, nLeaf, entry0, jobIndex, tile, pad_;
    int rows[8];                // the leaves' code rows
};

__device__ __forceinline__ unsigned long long cladeKey(const CladeTask &T, int k)
{
    unsigned long long key = 0;
    for (int i = 0; i < T.nLeaf; i++)
        key |= (unsigned long long)T.codes[(size_t)T.rows[i] * T.nPatPad + k] << (8 * i);
    return key;
}

__device__ __forceinline__ uint32_t cladeSlot(unsigned long long key, int hashSize)
{
    unsigned long long x = key * 0x9E3779B97F4A7C15ull;
    x ^= x >> 31;
    return (uint32_t)(((x >> 32) * (unsigned long long)hashSize) >> 32);
}

// One thread per pattern: insert the pattern's leaf-code combination; the
// thread that inserts a new key numbers it (atomic counter) and writes its
// codes as that column of the clade job.  idx[k] receives the slot.  Lanes
// of a warp holding the same key let one of them probe (clades of few
// leaves repeat their few combinations across every warp), and a slot is
// read before it is claimed, so a present key costs no atomic.  The table
// holds at most nPat < hashSize keys, so every probe sequence ends at the
// key or at an empty slot within hashSize steps.
__global__ void k_cladeInsert(const CladeTask *__restrict__ tasks)
{
    const CladeTask &T = tasks[blockIdx.y];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= T.nPat) return;
    const unsigned long long key = cladeKey(T, k);
    const unsigned same = __match_any_sync(__activemask(), key);
    const int leader = __ffs(same) - 1;
    uint32_t h = cladeSlot(key, T.hashSize);
    if ((int)(threadIdx.x & 31) == leader) {
        for (int probe = 0; probe < T.hashSize; probe++) {
            const unsigned long long cur = __ldcg(&T.keys[h]);
            if (cur == key) break;
            if (cur == kEmpty) {
                const unsigned long long prev = atomicCAS(&T.keys[h], kEmpty, key);
                if (prev == kEmpty) {
                    const int u = atomicAdd(T.count, 1);
                    T.vals[h] = u;
                    for (int i = 0; i < T.nLeaf; i++)
                        T.outCodes[(size_t)i * T.nPatPad + u] = (uint8_t)(key >> (8 * i));
                    break;
                }
                if (prev == key) break;
            }
            h = (h + 1 == (uint32_t)T.hashSize) ? 0u : h + 1;
        }
    }
    T.idx[k] = __shfl_sync(same, h, leader);
}

// One thread per padded pattern position: slot -> table entry; zero codes
// past the combination count (tiles read whole columns); list the clade
// job's tiles; publish the count as the job's pattern count.
__global__ void k_cladeIndex(const CladeTask *__restrict__ tasks)
{
    const CladeTask &T = tasks[blockIdx.y];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= T.nPatPad) return;
    const int n = *T.count;
    T.idx[k] = (uint32_t)(T.entry0 + (k < T.nPat ? T.vals[T.idx[k]] : 0));
    if (k >= n)
        for (int i = 0; i < T.nLeaf; i++) T.outCodes[(size_t)i * T.nPatPad + k] = 0;
    if (k == 0) T.job->nPat = n;
    if (k < n && k % T.tile == 0) {
        const int s = atomicAdd(T.nTiles, 1);
        T.blocks[s] = BlockDesc{T.jobIndex, k, k / T.tile, 0};
    }
}

// One tree's tile list of a clade group, for the batch merge.
struct CladeMergeSrc {
    const BlockDesc *blocks;
    const int *count;   // tiles the index kernel listed
    int jobBase;        // the tree's first job in the merged job array
    int pad_;
};

// One block: the trees' lists one after another, job indices shifted to the
// merged job array; the total goes to *outCount.  Each list holds at most
// its tree's capacity, and the merged list has room for the sum.
__global__ void k_cladeMerge(const CladeMergeSrc *__restrict__ src, int nSrc, BlockDesc *__restrict__ out,
                             int *__restrict__ outCount)
{
    int off = 0;
    for (int i = 0; i < nSrc; i++) {
        const int n = *src[i].count;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            BlockDesc d = src[i].blocks[k];
            d.job += src[i].jobBase;
            out[off + k] = d;
        }
        off += n;
    }
    if (threadIdx.x == 0) *outCount = off;
}

}  // namespace

// Pick the clades, build their programs and combination tables, upload
// everything and point the tree's jobs (host image) at it.  cladeOf receives,
// per node, the clade index whose table replaces its subtree (-1: none).
// Pick the clades: cladeOf receives, per node, a clade index (any order)
// for the root of every clade, -1 elsewhere.  Returns the clade count.
int cladeSelect(Tree *t, const std::vector<int> &order, std::vector<int> &cladeOf)
{
    TreeDev &dv = t->dev;
    const int nn = t->nNodes;
    const int L = dv.cladeSize;
    cladeOf.assign(nn, -1);
    if (L < 2 || dv.inBatch || dv.cladeOff) return 0;
    // leaves under every node (post-order)
    std::vector<int> leaves(nn, 0);
    for (int v : order) {
        Node *nv = t->nodes[v];
        if (nv->isLeaf && v != t->root) {
            leaves[v] = 1;
            continue;
        }
        for (int c = nv->leftChild; c >= 0; c = t->nodes[c]->sibling) leaves[v] += leaves[c];
    }
    std::vector<int> roots;
    for (int v : order) {
        Node *nv = t->nodes[v];
        if (v == t->root || nv->isLeaf || leaves[v] > L) continue;
        const int par = nv->parent;
        if (par < 0) continue;
        if (par == t->root || leaves[par] > L) roots.push_back(v);
    }
    // every tile stages one index row per clade in shared memory: keep the
    // kMaxClades largest clades (ties in post-order)
    if ((int)roots.size() > kMaxClades) {
        std::stable_sort(roots.begin(), roots.end(), [&](int a, int b) { return leaves[a] > leaves[b]; });
        roots.resize(kMaxClades);
        std::vector<int> keep(nn, 0);
        for (int v : roots) keep[v] = 1;
        roots.clear();
        for (int v : order)
            if (keep[v]) roots.push_back(v);
    }
    for (int c = 0; c < (int)roots.size(); c++) cladeOf[roots[c]] = c;
    return (int)roots.size();
}

// Build the clades' programs and combination tables, upload everything and
// point the tree's jobs (host image) at it.  cladeOf: per node, the clade
// index whose table replaces its subtree (-1: none); the whole-tree program
// reads the clades in index order.
int cladeBuild(Tree *t, const std::vector<int> &need, const std::vector<int> &cladeOf)
{
    TreeDev &dv = t->dev;
    const int nn = t->nNodes, nP = t->nParts;
    const int L = dv.cladeSize;
    dv.cladeVersion++;
    dv.nClade = 0;
    dv.cladeGroups.clear();
    dv.cladeTileCount.clear();
    int nC = 0;
    for (int v = 0; v < nn; v++) nC = std::max(nC, cladeOf[v] + 1);
    if (nC == 0) return P4G_OK;
    std::vector<int> roots(nC, -1);
    for (int v = 0; v < nn; v++)
        if (cladeOf[v] >= 0) roots[cladeOf[v]] = v;
    // programs: each clade's subtree, leaf rows renumbered 0..Lc-1
    std::vector<int> rowOf(nn, -1), progAll, progOff(nC), progLen(nC), nLeaf(nC), slots(nC);
    std::vector<std::vector<int>> seqRows(nC);
    for (int c = 0; c < nC; c++) {
        std::vector<int> st{roots[c]};
        while (!st.empty()) {   // leaves in depth-first child order
            const int v = st.back();
            st.pop_back();
            Node *nv = t->nodes[v];
            if (nv->isLeaf) {
                rowOf[v] = (int)seqRows[c].size();
                seqRows[c].push_back(nv->seqNum);
                continue;
            }
            std::vector<int> kids;
            for (int k = nv->leftChild; k >= 0; k = t->nodes[k]->sibling) kids.push_back(k);
            for (auto it = kids.rbegin(); it != kids.rend(); ++it) st.push_back(*it);
        }
        std::vector<int> prog;
        RET(emitProgram(t, roots[c], need, prog, nullptr, nullptr, &rowOf));
        progOff[c] = (int)progAll.size();
        progLen[c] = (int)prog.size();
        progAll.insert(progAll.end(), prog.begin(), prog.end());
        nLeaf[c] = (int)seqRows[c].size();
        slots[c] = need[roots[c]];
    }
    // per (part, clade) task: hash table, combination rows and clade job,
    // laid out in the tree's clade buffers (offsets in elements)
    std::vector<std::pair<int, int>> keys;   // (dim, nCat) groups
    for (int p = 0; p < nP; p++) {
        std::pair<int, int> k(t->model->parts[p].dim, t->model->parts[p].nCat);
        if (std::find(keys.begin(), keys.end(), k) == keys.end()) keys.push_back(k);
    }
    std::vector<int> shapeOfGroup(keys.size()), tileOfGroup(keys.size());
    for (size_t gi = 0; gi < keys.size(); gi++) {
        // the combination counts are small: lane groups of 4 (or 2) split the
        // categories so that the tables spread over more blocks; P decks are
        // read through L1 (a clade touches few of them)
        int shape = defaultShape(keys[gi].first);
        if (keys[gi].first == 4) shape = keys[gi].second % 4 == 0 ? 6 : keys[gi].second % 2 == 0 ? 8 : 3;
        auto it = dv.cladeShape.find(keys[gi].first * 64 + keys[gi].second);   // chosen by the timing
        if (it != dv.cladeShape.end()) shape = it->second;
        shapeOfGroup[gi] = shape;
        tileOfGroup[gi] = pruneTile(keys[gi].first, shape);
    }
    const int nTask = nP * nC;
    std::vector<size_t> keyOff(nP), idxOff(nP), codeOff(nP), tabOff(nP), expOff(nP);
    std::vector<int> hashSize(nP), groupOf(nP);
    size_t nKey = 0, nIdx = 0, nCode = 0, nTab = 0, nExp = 0;
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = t->model->parts[p];
        const int pad = t->data->parts[p]->nPatPad;
        groupOf[p] = (int)(std::find(keys.begin(), keys.end(), std::make_pair(mp.dim, mp.nCat)) - keys.begin());
        hashSize[p] = 2 * pad;   // load <= 1/2
        keyOff[p] = nKey;
        nKey += (size_t)nC * hashSize[p];
        idxOff[p] = nIdx;
        nIdx += (size_t)nC * pad;
        codeOff[p] = nCode;
        nCode += (size_t)nC * L * pad;
        tabOff[p] = nTab;
        nTab += (size_t)nC * pad * mp.nCat * mp.dim;
        expOff[p] = nExp;
        nExp += (size_t)nC * pad;
    }
    // tile lists: one region per group, sized for every pattern of every
    // clade; the index kernel fills them with the tiles actually needed
    std::vector<int> blk0(keys.size(), 0), blkCap(keys.size(), 0);
    {
        int nb = 0;
        for (size_t gi = 0; gi < keys.size(); gi++) {
            blk0[gi] = nb;
            for (int p = 0; p < nP; p++)
                if (groupOf[p] == (int)gi) blkCap[gi] += nC * (t->data->parts[p]->nPatPad / tileOfGroup[gi]);
            nb += blkCap[gi];
        }
        RET(dv.dCladeBlocks.ensure(sizeof(BlockDesc) * std::max(nb, 1)));
    }
    RET(dv.dCladeKeys.ensure(sizeof(unsigned long long) * nKey));
    RET(dv.dCladeVals.ensure(sizeof(int) * nKey));
    RET(dv.dCladeIdx.ensure(sizeof(uint32_t) * nIdx));
    RET(dv.dCladeCodes.ensure(nCode));
    RET(dv.dCladeTab.ensure(sizeof(float) * nTab));
    RET(dv.dCladeExp.ensure(sizeof(int) * nExp));
    const int nMisc = nTask + (int)keys.size();   // combination counts, then tile counts per group
    RET(dv.dCladeMisc.ensure(sizeof(int) * nMisc));
    // one upload: clade jobs, tasks, programs
    const size_t oJob = 0, oTask = roundUp(sizeof(PruneJob) * nTask, 256),
                 oProg = oTask + roundUp(sizeof(CladeTask) * nTask, 256),
                 metaBytes = oProg + sizeof(int) * progAll.size();
    RET(dv.dCladeMeta.ensure(metaBytes));
    if (!dv.cladeUp) P4G_CUDA(cudaEventCreateWithFlags(&dv.cladeUp, cudaEventDisableTiming));
    P4G_CUDA(cudaEventSynchronize(dv.cladeUp));   // the previous upload has left the staging buffer
    RET(dv.hClade.ensure(metaBytes));
    char *h = (char *)dv.hClade.ptr;
    char *dm = (char *)dv.dCladeMeta.ptr;
    PruneJob *jobs = (PruneJob *)(h + oJob);
    CladeTask *tasks = (CladeTask *)(h + oTask);
    memcpy(h + oProg, progAll.data(), sizeof(int) * progAll.size());
    const PruneJob *mainJobs = (const PruneJob *)((const char *)dv.hImg.ptr + dv.oJobs);
    int *misc = dv.dCladeMisc.as<int>();
    int maxPad = 0;
    std::vector<int> maxProg(keys.size(), 0), maxSlots(keys.size(), 0);
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = t->model->parts[p];
        const Part *dp = t->data->parts[p];
        const int pad = dp->nPatPad, gi = groupOf[p];
        for (int c = 0; c < nC; c++) {
            const int j = p * nC + c;
            PruneJob J = mainJobs[p];
            J.codes = dv.dCladeCodes.as<uint8_t>() + codeOff[p] + (size_t)c * L * pad;
            J.nPat = 0;   // written by k_cladeIndex
            J.nPatPad = pad;
            J.nTax = nLeaf[c];
            J.prog = (const int *)(dm + oProg) + progOff[c];
            J.nProg = progLen[c];
            J.nSlots = slots[c];
            J.rootLeafRow = -1;
            J.rootComp = nullptr;   // no root reduction; setPrams has not filled it yet either
            J.deckMap = nullptr;    // every deck and code row of the clade staged
            J.rowMap = nullptr;
            J.nDeck = nn;
            J.nRow = nLeaf[c];
            J.pInvar = 0.0;
            J.likeScaled = nullptr;
            J.exps = nullptr;
            J.lnl = nullptr;
            J.catLikes = nullptr;
            J.rootCL = nullptr;
            J.tcB = nullptr;
            J.cherryTab = nullptr;
            J.cherries = nullptr;
            J.nCherry = 0;
            J.cladeIdx = nullptr;
            J.cladeTab = nullptr;
            J.cladeExp = nullptr;
            J.nClade = 0;
            J.cladeOut = dv.dCladeTab.as<float>() + tabOff[p] + (size_t)c * pad * mp.nCat * mp.dim;
            J.cladeOutExp = dv.dCladeExp.as<int>() + expOff[p] + (size_t)c * pad;
            J.nBlocks = 0;
            jobs[j] = J;
            CladeTask &T = tasks[j];
            memset(&T, 0, sizeof(T));
            T.codes = dp->dCodes.as<uint8_t>();
            T.keys = dv.dCladeKeys.as<unsigned long long>() + keyOff[p] + (size_t)c * hashSize[p];
            T.vals = dv.dCladeVals.as<int>() + keyOff[p] + (size_t)c * hashSize[p];
            T.count = misc + j;
            T.nTiles = misc + nTask + gi;
            T.outCodes = (uint8_t *)J.codes;
            T.idx = dv.dCladeIdx.as<uint32_t>() + idxOff[p] + (size_t)c * pad;
            T.job = (PruneJob *)(dm + oJob) + j;
            T.blocks = dv.dCladeBlocks.as<BlockDesc>() + blk0[gi];
            T.nPat = dp->nPatterns;
            T.nPatPad = pad;
            T.hashSize = hashSize[p];
            T.nLeaf = nLeaf[c];
            T.entry0 = c * pad;
            T.jobIndex = j;
            T.tile = tileOfGroup[gi];
            for (int i = 0; i < nLeaf[c]; i++) T.rows[i] = seqRows[c][i];
            maxPad = std::max(maxPad, pad);
            maxProg[gi] = std::max(maxProg[gi], progLen[c]);
            maxSlots[gi] = std::max(maxSlots[gi], slots[c]);
        }
    }
    cudaStream_t s = ctx().stream;
    P4G_CUDA(cudaMemcpyAsync(dm, h, metaBytes, cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaEventRecord(dv.cladeUp, s));
    P4G_CUDA(cudaMemsetAsync(dv.dCladeKeys.ptr, 0xff, sizeof(unsigned long long) * nKey, s));
    P4G_CUDA(cudaMemsetAsync(misc, 0, sizeof(int) * nMisc, s));
    const dim3 grid((maxPad + 255) / 256, nTask);
    const CladeTask *dTasks = (const CladeTask *)(dm + oTask);
    k_cladeInsert<<<grid, 256, 0, s>>>(dTasks);
    P4G_CUDA(cudaGetLastError());
    k_cladeIndex<<<grid, 256, 0, s>>>(dTasks);
    P4G_CUDA(cudaGetLastError());
    dv.cladeFresh = true;   // the stream's last kernel wrote the clade jobs, tiles and codes
    for (size_t gi = 0; gi < keys.size(); gi++) {
        PruneGroup g{keys[gi].first, keys[gi].second, blk0[gi], blkCap[gi], 0, shapeOfGroup[gi]};
        g.smem = pruneSmemBytes(g.dim, g.nCat, maxProg[gi], nn, L, maxSlots[gi], g.shape);
        if (g.smem > 227 * 1024) return setError(P4G_EUNSUPPORTED, "clade program too large (%d bytes)", g.smem);
        dv.cladeGroups.push_back(g);
        dv.cladeTileCount.push_back(misc + nTask + (int)gi);
    }
    // the whole-tree jobs read the tables
    PruneJob *hJobs = (PruneJob *)((char *)dv.hImg.ptr + dv.oJobs);
    for (int p = 0; p < nP; p++) {
        hJobs[p].cladeIdx = dv.dCladeIdx.as<uint32_t>() + idxOff[p];
        hJobs[p].cladeTab = dv.dCladeTab.as<float>() + tabOff[p];
        hJobs[p].cladeExp = dv.dCladeExp.as<int>() + expOff[p];
        hJobs[p].nCladeEntries = nC * t->data->parts[p]->nPatPad;
    }
    dv.nClade = nC;
    return P4G_OK;
}

// Fill the clade tables of the current parameters (before the whole-tree launch).
int cladeLaunch(Tree *t, cudaStream_t s, int early)
{
    TreeDev &dv = t->dev;
    if (!dv.nClade) return P4G_OK;
    const PruneJob *dJobs = (const PruneJob *)dv.dCladeMeta.ptr;
    const BlockDesc *dBlocks = dv.dCladeBlocks.as<BlockDesc>();
    for (size_t gi = 0; gi < dv.cladeGroups.size(); gi++) {
        const PruneGroup &g = dv.cladeGroups[gi];
        RET(launchPrune(dJobs, dBlocks + g.blk0, g.nBlk, g.dim, g.nCat, g.smem, g.shape, s, dv.cladeTileCount[gi],
                        early));
        // a later group follows a clade launch, which writes only its tables
        if (g.nBlk > 0) early = PDL_EARLY_JOBS | PDL_EARLY_DECKS;
    }
    return P4G_OK;
}

int cladeMerge(const std::vector<Tree *> &trees, DevBuf &dJobs, DevBuf &dBlocks, DevBuf &dCounts, DevBuf &dSrc,
               std::vector<PruneGroup> &groups, cudaStream_t s)
{
    groups.clear();
    const TreeDev &d0 = trees[0]->dev;
    if (d0.cladeGroups.empty()) return P4G_OK;
    int nJobs = 0;
    std::vector<int> jobBase;
    for (Tree *t : trees) {
        const TreeDev &dv = t->dev;
        if (dv.cladeGroups.size() != d0.cladeGroups.size()) return P4G_OK;
        for (size_t gi = 0; gi < dv.cladeGroups.size(); gi++) {
            const PruneGroup &a = dv.cladeGroups[gi], &b = d0.cladeGroups[gi];
            if (a.dim != b.dim || a.nCat != b.nCat || a.shape != b.shape) return P4G_OK;
        }
        jobBase.push_back(nJobs);
        nJobs += t->nParts * dv.nClade;
    }
    const size_t nG = d0.cladeGroups.size();
    std::vector<PruneGroup> out(nG);
    int nb = 0;
    for (size_t gi = 0; gi < nG; gi++) {
        PruneGroup g = d0.cladeGroups[gi];
        g.blk0 = nb;
        g.nBlk = 0;
        g.smem = 0;
        for (Tree *t : trees) {
            g.nBlk += t->dev.cladeGroups[gi].nBlk;
            g.smem = std::max(g.smem, t->dev.cladeGroups[gi].smem);
        }
        nb += g.nBlk;
        out[gi] = g;
    }
    RET(dJobs.ensure(sizeof(PruneJob) * std::max(nJobs, 1)));
    RET(dBlocks.ensure(sizeof(BlockDesc) * std::max(nb, 1)));
    RET(dCounts.ensure(sizeof(int) * nG));
    RET(dSrc.ensure(sizeof(CladeMergeSrc) * trees.size() * nG));
    std::vector<CladeMergeSrc> src(trees.size() * nG);
    for (size_t ti = 0; ti < trees.size(); ti++) {
        const TreeDev &dv = trees[ti]->dev;
        // the tree's clade jobs lead its clade metadata block
        P4G_CUDA(cudaMemcpyAsync(dJobs.as<PruneJob>() + jobBase[ti], dv.dCladeMeta.ptr,
                                 sizeof(PruneJob) * trees[ti]->nParts * dv.nClade, cudaMemcpyDeviceToDevice, s));
        for (size_t gi = 0; gi < nG; gi++)
            src[gi * trees.size() + ti] = CladeMergeSrc{dv.dCladeBlocks.as<BlockDesc>() + dv.cladeGroups[gi].blk0,
                                                        dv.cladeTileCount[gi], jobBase[ti], 0};
    }
    P4G_CUDA(cudaMemcpyAsync(dSrc.ptr, src.data(), sizeof(CladeMergeSrc) * src.size(), cudaMemcpyHostToDevice, s));
    for (size_t gi = 0; gi < nG; gi++) {
        k_cladeMerge<<<1, 256, 0, s>>>(dSrc.as<CladeMergeSrc>() + gi * trees.size(), (int)trees.size(),
                                        dBlocks.as<BlockDesc>() + out[gi].blk0, dCounts.as<int>() + gi);
        P4G_CUDA(cudaGetLastError());
    }
    groups = out;
    return P4G_OK;
}
