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
#include <unordered_map>
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

}  // namespace

// Pick the clades, build their programs and combination tables, upload
// everything and point the tree's jobs (host image) at it.  cladeOf receives,
// per node, the clade index whose table replaces its subtree (-1: none).
int cladeBuild(Tree *t, const std::vector<int> &need, const std::vector<int> &order, std::vector<int> &cladeOf)
{
    TreeDev &dv = t->dev;
    const int nn = t->nNodes, nP = t->nParts;
    const int L = dv.cladeSize;
    cladeOf.assign(nn, -1);
    dv.nClade = 0;
    dv.cladeGroups.clear();
    if (L < 2 || dv.inBatch) return P4G_OK;
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
    const int nC = (int)roots.size();
    if (nC == 0) return P4G_OK;
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
    // per part: distinct combinations of each clade's leaf codes
    struct PartTabs {
        std::vector<uint32_t> idx;     // [nC][nPatPad]
        std::vector<int> off;          // [nC] first entry of each clade
        std::vector<int> nU;           // [nC]
        std::vector<size_t> codeOff;   // [nC] byte offset into the codes blob
        int entries = 0;
    };
    std::vector<PartTabs> pt(nP);
    std::vector<uint8_t> codesAll;
    for (int p = 0; p < nP; p++) {
        const Part *dp = t->data->parts[p];
        const int nPat = dp->nPatterns, pad = dp->nPatPad;
        PartTabs &T = pt[p];
        T.idx.assign((size_t)nC * pad, 0u);
        T.off.resize(nC);
        T.nU.resize(nC);
        T.codeOff.resize(nC);
        std::unordered_map<uint64_t, int> ids;
        for (int c = 0; c < nC; c++) {
            const int Lc = nLeaf[c];
            T.off[c] = T.entries;
            ids.clear();
            ids.reserve(2 * std::min(nPat, 4096));
            std::vector<int> firstPat;
            for (int k = 0; k < nPat; k++) {
                uint64_t key = 0;
                for (int i = 0; i < Lc; i++)
                    key |= (uint64_t)dp->hCodes[(size_t)seqRows[c][i] * pad + k] << (8 * i);
                auto it = ids.find(key);
                int u;
                if (it == ids.end()) {
                    u = (int)firstPat.size();
                    ids.emplace(key, u);
                    firstPat.push_back(k);
                } else {
                    u = it->second;
                }
                T.idx[(size_t)c * pad + k] = (uint32_t)(T.off[c] + u);
            }
            for (int k = nPat; k < pad; k++) T.idx[(size_t)c * pad + k] = (uint32_t)T.off[c];   // padding: any valid entry
            const int nU = (int)firstPat.size();
            const size_t uPad = roundUp((size_t)nU, 512);   // the largest tile is 512 patterns
            T.nU[c] = nU;
            T.entries += nU;
            T.codeOff[c] = codesAll.size();
            codesAll.resize(codesAll.size() + (size_t)Lc * uPad, 0);
            uint8_t *cc = codesAll.data() + T.codeOff[c];
            for (int i = 0; i < Lc; i++)
                for (int u = 0; u < nU; u++)
                    cc[(size_t)i * uPad + u] = dp->hCodes[(size_t)seqRows[c][i] * pad + firstPat[u]];
        }
    }
    // device buffers (offsets in elements)
    std::vector<size_t> idxOff(nP), tabOff(nP), expOff(nP);
    size_t nIdx = 0, nTab = 0, nExp = 0;
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = t->model->parts[p];
        idxOff[p] = nIdx;
        nIdx += pt[p].idx.size();
        tabOff[p] = nTab;
        nTab += roundUp((size_t)pt[p].entries * mp.nCat * mp.dim, 4);
        expOff[p] = nExp;
        nExp += pt[p].entries;
    }
    RET(dv.dCladeProg.ensure(sizeof(int) * progAll.size()));
    RET(dv.dCladeIdx.ensure(sizeof(uint32_t) * nIdx));
    RET(dv.dCladeTab.ensure(sizeof(float) * nTab));
    RET(dv.dCladeExp.ensure(sizeof(int) * nExp));
    RET(dv.dCladeCodes.ensure(std::max<size_t>(codesAll.size(), 16)));
    cudaStream_t s = ctx().stream;
    P4G_CUDA(cudaMemcpyAsync(dv.dCladeProg.ptr, progAll.data(), sizeof(int) * progAll.size(),
                             cudaMemcpyHostToDevice, s));
    for (int p = 0; p < nP; p++) {
        P4G_CUDA(cudaMemcpyAsync(dv.dCladeIdx.as<uint32_t>() + idxOff[p], pt[p].idx.data(),
                                 sizeof(uint32_t) * pt[p].idx.size(), cudaMemcpyHostToDevice, s));
    }
    if (!codesAll.empty())
        P4G_CUDA(cudaMemcpyAsync(dv.dCladeCodes.ptr, codesAll.data(), codesAll.size(), cudaMemcpyHostToDevice, s));
    // the clade-table jobs (one per part and clade) and their tiles, grouped
    // like the whole-tree groups by (dim, nCat)
    const PruneJob *mainJobs = (const PruneJob *)((const char *)dv.hImg.ptr + dv.oJobs);
    std::vector<PruneJob> jobs((size_t)nP * nC);
    std::vector<BlockDesc> blocks;
    int maxProg = 0, maxSlots = 0;
    for (int c = 0; c < nC; c++) {
        maxProg = std::max(maxProg, progLen[c]);
        maxSlots = std::max(maxSlots, slots[c]);
    }
    std::vector<std::pair<int, int>> keys;
    for (int p = 0; p < nP; p++) {
        std::pair<int, int> k(t->model->parts[p].dim, t->model->parts[p].nCat);
        if (std::find(keys.begin(), keys.end(), k) == keys.end()) keys.push_back(k);
    }
    for (auto &k : keys) {
        // the combination counts are small: lane groups of 4 (or 2) split the
        // categories so that the tables spread over more blocks
        int shape = defaultShape(k.first);
        if (k.first == 4) shape = k.second % 4 == 0 ? 6 : k.second % 2 == 0 ? 8 : 3;
        PruneGroup g{k.first, k.second, (int)blocks.size(), 0, 0, shape};
        const int tile = pruneTile(g.dim, g.shape);
        for (int p = 0; p < nP; p++) {
            const ModelPart &mp = t->model->parts[p];
            if (mp.dim != g.dim || mp.nCat != g.nCat) continue;
            for (int c = 0; c < nC; c++) {
                const int j = p * nC + c;
                PruneJob J = mainJobs[p];
                const int nU = pt[p].nU[c];
                J.codes = dv.dCladeCodes.as<uint8_t>() + pt[p].codeOff[c];
                J.nPat = nU;
                J.nPatPad = (int)roundUp((size_t)nU, 512);
                J.nTax = nLeaf[c];
                J.prog = dv.dCladeProg.as<int>() + progOff[c];
                J.nProg = progLen[c];
                J.nSlots = slots[c];
                J.rootLeafRow = -1;
                J.rootComp = nullptr;   // no root reduction; setPrams has not filled it yet either
                J.pInvar = 0.0;
                J.likeScaled = nullptr;
                J.exps = nullptr;
                J.lnl = nullptr;
                J.catLikes = nullptr;
                J.tcB = nullptr;
                J.cherryTab = nullptr;
                J.cherries = nullptr;
                J.nCherry = 0;
                J.cladeIdx = nullptr;
                J.nClade = 0;
                J.firstClade = 0;
                J.cladeTab = nullptr;
                J.cladeExp = nullptr;
                J.cladeOut = dv.dCladeTab.as<float>() + tabOff[p] + (size_t)pt[p].off[c] * mp.nCat * mp.dim;
                J.cladeOutExp = dv.dCladeExp.as<int>() + expOff[p] + pt[p].off[c];
                const int nb = (nU + tile - 1) / tile;
                for (int b = 0; b < nb; b++) blocks.push_back(BlockDesc{j, b * tile, b, 0});
                J.nBlocks = nb;
                jobs[j] = J;
            }
        }
        g.nBlk = (int)blocks.size() - g.blk0;
        g.smem = pruneSmemBytes(g.dim, g.nCat, maxProg, nn, L, maxSlots, g.shape);
        if (g.smem > 227 * 1024) return setError(P4G_EUNSUPPORTED, "clade program too large (%d bytes)", g.smem);
        dv.cladeGroups.push_back(g);
    }
    RET(dv.dCladeJobs.ensure(sizeof(PruneJob) * jobs.size()));
    RET(dv.dCladeBlocks.ensure(sizeof(BlockDesc) * std::max<size_t>(blocks.size(), 1)));
    P4G_CUDA(cudaMemcpyAsync(dv.dCladeJobs.ptr, jobs.data(), sizeof(PruneJob) * jobs.size(), cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaMemcpyAsync(dv.dCladeBlocks.ptr, blocks.data(), sizeof(BlockDesc) * blocks.size(),
                             cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaStreamSynchronize(s));   // host vectors go out of scope
    // the whole-tree jobs read the tables
    PruneJob *hJobs = (PruneJob *)((char *)dv.hImg.ptr + dv.oJobs);
    for (int p = 0; p < nP; p++) {
        hJobs[p].cladeIdx = dv.dCladeIdx.as<uint32_t>() + idxOff[p];
        hJobs[p].cladeTab = dv.dCladeTab.as<float>() + tabOff[p];
        hJobs[p].cladeExp = dv.dCladeExp.as<int>() + expOff[p];
    }
    dv.nClade = nC;
    return P4G_OK;
}

// Fill the clade tables of the current parameters (before the whole-tree launch).
int cladeLaunch(Tree *t, cudaStream_t s)
{
    TreeDev &dv = t->dev;
    if (!dv.nClade) return P4G_OK;
    const PruneJob *dJobs = dv.dCladeJobs.as<PruneJob>();
    const BlockDesc *dBlocks = dv.dCladeBlocks.as<BlockDesc>();
    for (auto &g : dv.cladeGroups)
        RET(launchPrune(dJobs, dBlocks + g.blk0, g.nBlk, g.dim, g.nCat, g.smem, g.shape, s));
    return P4G_OK;
}
