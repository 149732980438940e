// Draws from the tree's distributions, on the GPU:
//
//   p4g_drawAncStates  a draw of every site's root state (or invariant
//                      state) and Gamma category from its posterior given
//                      the data: p4_drawAncState (Pf/p4_treeSim.c:591-845),
//                      once per site, as Tree.ancestralStateDraw
//                      (p4/tree.py:9640-9670) calls it;
//   p4g_simulate       a new alignment down the tree: p4_simulate without a
//                      reference tree (Pf/p4_treeSim.c:14-590).
//
// Random numbers.  Both functions take their uniforms either from the caller
// (one per decision, in the order the reference's sequential loops draw
// them) or from a Philox4x32-10 stream (p4g_philox.h), whose n-th value is a
// pure function of (seed, n).  Every GPU thread computes the index n of the
// number the reference's loop would draw for its decision, so the draws are
// those of the sequential algorithm fed the same stream.
//
// p4_simulate draws, in this order: per part with nCat > 1, one Gamma
// category per site (floor(nCat * u)); per part, the root state of every
// site from the running sum of the root composition (last entry 1.0); per
// part with pInvar > 0, an invariant flag per site (u < pInvar); then per
// part, per non-root node in pre-order, per site that is not invariant, the
// child state from the running sum of the parent state's row of P(t) for the
// site's category (last entry 1.0).  Invariant sites copy the parent's state
// and draw nothing, so a node's draws are indexed by the site's rank among
// the part's variable sites (a prefix sum on the GPU).
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <algorithm>
#include <new>
#include <vector>
#include "p4g_internal.h"
#include "p4g_philox.h"

using namespace p4g;

#define RET(call)                      \
    do {                               \
        int rc_ = (call);              \
        if (rc_ != P4G_OK) return rc_; \
    } while (0)

namespace {

// ---------------------------------------------------------- ancestral draws

struct AncPart {
    const float *rootCL;     // [nPat][nCat][dim], scaled by 2^E (exps)
    const int *exps;         // [nPat]
    const uint32_t *invMask; // [nPat] states for which the pattern is constant
    const int *seqPosIdx;    // [nChar] site -> pattern
    const double *rootComp;  // [dim]
    const double *uniforms;  // [nChar] or null: Philox(seed, site)
    int *draws;              // [nChar][4] (chState, cat, isInvar, invarState)
    int *failed;             // set when a site's picker finds nothing
    unsigned long long seed, offset;   // Philox: site i takes value offset + i
    double pInvar, freq;     // freq = (1 - pInvar) / nCat, the category weight
    int nChar, nCat, dim, pInvarFree;
};

// One thread per site.  The running sum follows p4_drawAncState: categories
// outer, states inner, each term pi_s * cl[c][s] * freq, then pi_s * pInvar
// for every state the pattern may be constant in; the site's uniform times
// the total picks the first entry whose running sum exceeds it.  With
// pInvar the partials are unscaled (2^-E) so that both kinds of term share
// one scale; without it the common factor 2^-E cancels and is left out.
__global__ void k_drawAnc(AncPart A)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.nChar) return;
    const int k = A.seqPosIdx[i];
    const float *cl = A.rootCL + (size_t)k * A.nCat * A.dim;
    const double unscale = (A.pInvar != 0.0) ? ldexp(1.0, -A.exps[k]) : 1.0;
    const uint32_t im = (A.pInvar != 0.0) ? A.invMask[k] : 0u;
    double sLike = 0.0;
    for (int c = 0; c < A.nCat; c++)
        for (int s = 0; s < A.dim; s++) sLike += A.rootComp[s] * ((double)cl[c * A.dim + s] * unscale) * A.freq;
    for (int s = 0; s < A.dim; s++)
        if ((im >> s) & 1u) sLike += A.rootComp[s] * A.pInvar;
    const double u = A.uniforms ? A.uniforms[i] : philoxUniform(A.seed, A.offset + (unsigned long long)i);
    const double x = u * sLike;
    int *d = A.draws + (size_t)i * 4;
    double run = 0.0;
    for (int c = 0; c < A.nCat; c++)
        for (int s = 0; s < A.dim; s++) {
            run += A.rootComp[s] * ((double)cl[c * A.dim + s] * unscale) * A.freq;
            if (x < run) {
                d[0] = s;
                d[1] = c;
                d[2] = 0;
                d[3] = -1;
                return;
            }
        }
    if (A.pInvarFree)
        for (int s = 0; s < A.dim; s++)
            if ((im >> s) & 1u) {
                run += A.rootComp[s] * A.pInvar;
                if (x < run) {
                    d[0] = -1;
                    d[1] = -1;
                    d[2] = 1;
                    d[3] = s;
                    return;
                }
            }
    d[0] = d[1] = d[3] = -1;
    d[2] = 0;
    atomicOr(A.failed, 1);
}

// ---------------------------------------------------------- simulation

struct SimPart {
    const double *decks64;    // [nNodes][nCat][dim][dim], row = parent state
    const double *rootComp;   // [dim]
    int8_t *states;           // [nNodes][nChar]
    uint8_t *cat;             // [nChar]
    uint8_t *inv;             // [nChar]
    int *varRank;             // [nChar] rank of the site among the variable ones
    int *nVar;                // variable sites of the part
    const double *uniforms;   // caller's stream or null (Philox)
    unsigned long long seed;
    unsigned long long n1, n2, n3;   // first uniform of the category, root and invariant loops
    double pInvar;
    int nChar, nCat, dim, part;
};

struct SimTree {
    const int *preNodes;      // non-root nodes in pre-order
    const int *parentOf;      // [nNodes]
    int nPre, root, nParts;
    unsigned long long n4;    // first uniform of the mutation loop
};

__device__ __forceinline__ double simUniform(const SimPart &P, unsigned long long n)
{
    return P.uniforms ? P.uniforms[n] : philoxUniform(P.seed, n);
}

// One thread per (site, part): Gamma category, root state, invariant flag.
__global__ void k_simRoot(const SimPart *__restrict__ parts, SimTree T)
{
    const SimPart &P = parts[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nChar) return;
    P.cat[i] = (P.nCat > 1) ? (uint8_t)(int)floor((double)P.nCat * simUniform(P, P.n1 + i)) : 0;
    const double u = simUniform(P, P.n2 + i);
    double run = P.rootComp[0];
    int s = 0;
    for (; s < P.dim - 1; s++) {
        if (u < run) break;
        run += P.rootComp[s + 1];
    }
    // the last entry of the picker is 1.0: u < 1 always lands there
    P.states[(size_t)T.root * P.nChar + i] = (int8_t)s;
    P.inv[i] = (P.pInvar > 0.0) ? (simUniform(P, P.n3 + i) < P.pInvar) : 0;
}

// One block per part: exclusive prefix sum of the variable-site flags.
__global__ void __launch_bounds__(1024) k_simRank(const SimPart *__restrict__ parts)
{
    const SimPart &P = parts[blockIdx.x];
    __shared__ int part[1024];
    const int t = threadIdx.x, n = P.nChar;
    const int chunk = (n + 1023) / 1024;
    const int b = min(n, t * chunk), e = min(n, b + chunk);
    int s = 0;
    for (int i = b; i < e; i++) s += !P.inv[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;
    for (int i = b; i < e; i++) {
        P.varRank[i] = run;
        run += !P.inv[i];
    }
    if (t == 1023) *P.nVar = part[1023];
}

// One thread per (site, part): the site's states down the tree, node by
// node in pre-order, each from its parent's state.
__global__ void k_simMutate(const SimPart *__restrict__ parts, SimTree T)
{
    const SimPart &P = parts[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nChar) return;
    unsigned long long base = T.n4;
    for (int q = 0; q < P.part; q++) base += (unsigned long long)T.nPre * (unsigned long long)*parts[q].nVar;
    const unsigned long long nVar = (unsigned long long)*P.nVar;
    const bool invariant = P.inv[i] != 0;
    const int c = P.cat[i];
    const unsigned long long rank = (unsigned long long)P.varRank[i];
    const int dd = P.dim * P.dim;
    for (int r = 0; r < T.nPre; r++) {
        const int v = T.preNodes[r];
        const int ps = P.states[(size_t)T.parentOf[v] * P.nChar + i];
        int s = ps;
        if (!invariant) {
            const double u = simUniform(P, base + (unsigned long long)r * nVar + rank);
            const double *row = P.decks64 + ((size_t)v * P.nCat + c) * dd + (size_t)ps * P.dim;
            double run = row[0];
            for (s = 0; s < P.dim - 1; s++) {
                if (u < run) break;
                run += row[s + 1];
            }
        }
        P.states[(size_t)v * P.nChar + i] = (int8_t)s;
    }
}

}  // namespace

extern "C" int p4g_drawAncStates(p4g_tree *tt, int pNum, const double *uniforms, unsigned long long seed,
                                 int *draws)
{
    Tree *t = reinterpret_cast<Tree *>(tt);
    if (!t || !draws || pNum < 0 || pNum >= t->nParts) return setError(P4G_EINVAL, "drawAncStates: bad arguments");
    if (t->dev.precision != 0) return setError(P4G_EUNSUPPORTED, "drawAncStates: needs the FP32 path (precision 0)");
    if (t->root < 0 || !t->nodes[t->root] || t->nodes[t->root]->isLeaf)
        return setError(P4G_EUNSUPPORTED, "drawAncStates: the root must be an internal node");
    TreeDev &dv = t->dev;
    dv.rootCLOn = true;
    double lnL = 0.0;
    int rc = treeLogLikeSites(t, &lnL);
    dv.rootCLOn = false;
    RET(rc);
    const ModelPart &mp = t->model->parts[pNum];
    Part *dp = t->data->parts[pNum];
    const int nChar = dp->nChar;
    DevBuf dSeqPos, dU, dDraws, dFail;
    RET(dSeqPos.ensure(sizeof(int) * nChar));
    RET(dDraws.ensure(sizeof(int) * 4 * (size_t)nChar));
    RET(dFail.ensure(sizeof(int)));
    if (uniforms) RET(dU.ensure(sizeof(double) * nChar));
    cudaStream_t s = ctx().stream;
    P4G_CUDA(cudaMemcpyAsync(dSeqPos.ptr, dp->seqPosIdx.data(), sizeof(int) * nChar, cudaMemcpyHostToDevice, s));
    if (uniforms) P4G_CUDA(cudaMemcpyAsync(dU.ptr, uniforms, sizeof(double) * nChar, cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaMemsetAsync(dFail.ptr, 0, sizeof(int), s));
    const PruneJob *hj = (const PruneJob *)((const char *)dv.hImg.ptr + dv.oJobs);
    AncPart A;
    A.rootCL = dv.dRootCL.as<float>() + dv.oRootCL[pNum];
    A.exps = dv.dExp.as<int>() + dv.oPat[pNum];
    A.invMask = dp->dInvMask.as<uint32_t>();
    A.seqPosIdx = dSeqPos.as<int>();
    A.rootComp = hj[pNum].rootComp;
    A.uniforms = uniforms ? dU.as<double>() : nullptr;
    A.draws = dDraws.as<int>();
    A.failed = dFail.as<int>();
    A.seed = seed;
    A.offset = 0;   // the parts' sites form one stream, in part order
    for (int q = 0; q < pNum; q++) A.offset += (unsigned long long)t->data->parts[q]->nChar;
    A.pInvar = mp.pInvar;
    A.freq = (1.0 / mp.nCat) * (1.0 - mp.pInvar);
    A.nChar = nChar;
    A.nCat = mp.nCat;
    A.dim = mp.dim;
    A.pInvarFree = mp.pInvarFree;
    k_drawAnc<<<(nChar + 255) / 256, 256, 0, s>>>(A);
    P4G_CUDA(cudaGetLastError());
    int failed = 0;
    P4G_CUDA(cudaMemcpyAsync(draws, dDraws.ptr, sizeof(int) * 4 * (size_t)nChar, cudaMemcpyDeviceToHost, s));
    P4G_CUDA(cudaMemcpyAsync(&failed, dFail.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    P4G_CUDA(cudaStreamSynchronize(s));
    if (failed)
        return setError(P4G_ENUMERIC, "drawAncStates: the ancestral state picker found no state for some site");
    return P4G_OK;
}

// The simulation of p4_simulate (Pf/p4_treeSim.c:14-590).  rootDraws null:
// every site's Gamma category, root state and invariant flag from the
// uniform stream, then the mutation loop; rootDraws (per part nChar x 4
// ints, p4_drawAncState's (chState, cat, isInvar, invarState) on the
// reference tree): those fixed, and the mutation loop takes the stream from
// its first value, as the reference-tree mode does (Pf/p4_treeSim.c:223-284).
static int simulateCore(Tree *t, const double *uniforms, long long nUniforms, unsigned long long seed,
                        signed char *allStates, const std::vector<std::vector<int>> *rootDraws)
{
    if (!t || (uniforms && nUniforms <= 0)) return setError(P4G_EINVAL, "simulate: bad arguments");
    if (t->root < 0 || !t->nodes[t->root]) return setError(P4G_ESTATE, "simulate: the tree has no root");
    const int nP = t->nParts, nn = t->nNodes;
    Data *d = t->data;
    Model *m = t->model;
    for (int p = 0; p < nP; p++)
        if (m->parts[p].nCat > 255) return setError(P4G_EUNSUPPORTED, "simulate: more than 255 categories");
    // P(t) of every node for the current parameters (the reference recomputes
    // the decks before its mutation loop)
    RET(setPramsForDraws(t));
    // pre-order over the tree's relations (p4's order: a node, then its
    // children from leftChild along the siblings)
    std::vector<int> pre, parentOf(nn, -1), st{t->root};
    while (!st.empty()) {
        const int v = st.back();
        st.pop_back();
        if (v != t->root) pre.push_back(v);
        std::vector<int> kids;
        for (int c = t->nodes[v]->leftChild; c >= 0; c = t->nodes[c]->sibling) {
            kids.push_back(c);
            parentOf[c] = v;
        }
        for (auto it = kids.rbegin(); it != kids.rend(); ++it) st.push_back(*it);
    }
    // uniform offsets of the three per-site loops (none with root draws)
    unsigned long long n1 = 0, n2 = 0, n3 = 0;
    std::vector<unsigned long long> o1(nP), o2(nP), o3(nP);
    for (int p = 0; p < nP; p++) {
        o1[p] = n1;
        if (m->parts[p].nCat > 1 && !rootDraws) n1 += d->parts[p]->nChar;
    }
    n2 = n1;
    for (int p = 0; p < nP; p++) {
        o2[p] = n2;
        if (!rootDraws) n2 += d->parts[p]->nChar;
    }
    n3 = n2;
    for (int p = 0; p < nP; p++) {
        o3[p] = n3;
        if (m->parts[p].pInvar > 0.0 && !rootDraws) n3 += d->parts[p]->nChar;
    }
    // the mutation loop draws at most nPre uniforms per site
    unsigned long long maxDraws = n3;
    for (int p = 0; p < nP; p++) maxDraws += (unsigned long long)pre.size() * d->parts[p]->nChar;
    if (uniforms && (unsigned long long)nUniforms < maxDraws)
        return setError(P4G_EINVAL, "simulate: %lld uniforms given, up to %llu may be drawn", nUniforms, maxDraws);
    size_t nStates = 0, nSites = 0;
    std::vector<size_t> oStates(nP), oSites(nP);
    int maxChar = 0;
    for (int p = 0; p < nP; p++) {
        oStates[p] = nStates;
        nStates += (size_t)nn * d->parts[p]->nChar;
        oSites[p] = nSites;
        nSites += d->parts[p]->nChar;
        maxChar = std::max(maxChar, d->parts[p]->nChar);
    }
    DevBuf dStates, dCat, dInv, dRank, dNVar, dParts, dPre, dParent, dU;
    RET(dStates.ensure(std::max<size_t>(nStates, 1)));
    RET(dCat.ensure(nSites));
    RET(dInv.ensure(nSites));
    RET(dRank.ensure(sizeof(int) * nSites));
    RET(dNVar.ensure(sizeof(int) * nP));
    RET(dParts.ensure(sizeof(SimPart) * nP));
    RET(dPre.ensure(sizeof(int) * std::max<size_t>(pre.size(), 1)));
    RET(dParent.ensure(sizeof(int) * nn));
    if (uniforms) RET(dU.ensure(sizeof(double) * (size_t)nUniforms));
    TreeDev &dv = t->dev;
    const PruneJob *hj = (const PruneJob *)((const char *)dv.hImg.ptr + dv.oJobs);
    std::vector<SimPart> parts(nP);
    for (int p = 0; p < nP; p++) {
        SimPart &P = parts[p];
        P.decks64 = dv.dDecks64.as<double>() + dv.oDecks[p];
        P.rootComp = hj[p].rootComp;
        P.states = dStates.as<int8_t>() + oStates[p];
        P.cat = dCat.as<uint8_t>() + oSites[p];
        P.inv = dInv.as<uint8_t>() + oSites[p];
        P.varRank = dRank.as<int>() + oSites[p];
        P.nVar = dNVar.as<int>() + p;
        P.uniforms = uniforms ? dU.as<double>() : nullptr;
        P.seed = seed;
        P.n1 = o1[p];
        P.n2 = o2[p];
        P.n3 = o3[p];
        P.pInvar = m->parts[p].pInvar;
        P.nChar = d->parts[p]->nChar;
        P.nCat = m->parts[p].nCat;
        P.dim = m->parts[p].dim;
        P.part = p;
    }
    SimTree T;
    T.preNodes = dPre.as<int>();
    T.parentOf = dParent.as<int>();
    T.nPre = (int)pre.size();
    T.root = t->root;
    T.nParts = nP;
    T.n4 = n3;
    cudaStream_t s = ctx().stream;
    P4G_CUDA(cudaMemcpyAsync(dParts.ptr, parts.data(), sizeof(SimPart) * nP, cudaMemcpyHostToDevice, s));
    if (!pre.empty())
        P4G_CUDA(cudaMemcpyAsync(dPre.ptr, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaMemcpyAsync(dParent.ptr, parentOf.data(), sizeof(int) * nn, cudaMemcpyHostToDevice, s));
    if (uniforms)
        P4G_CUDA(cudaMemcpyAsync(dU.ptr, uniforms, sizeof(double) * (size_t)nUniforms, cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaMemsetAsync(dStates.ptr, 0, std::max<size_t>(nStates, 1), s));
    const dim3 grid((maxChar + 255) / 256, nP);
    const SimPart *dp = dParts.as<SimPart>();
    std::vector<int8_t> hRoot;
    std::vector<uint8_t> hCat, hInv;
    if (rootDraws) {   // the root states, categories and invariant flags the reference tree drew
        hCat.assign(nSites, 0);
        hInv.assign(nSites, 0);
        for (int p = 0; p < nP; p++) {
            const std::vector<int> &dr = (*rootDraws)[p];
            const int nChar = d->parts[p]->nChar;
            hRoot.assign(nChar, 0);
            for (int i = 0; i < nChar; i++) {
                const int *x = dr.data() + 4 * (size_t)i;
                const bool inv = x[2] != 0;
                hRoot[i] = (int8_t)(inv ? x[3] : x[0]);
                hCat[oSites[p] + i] = (uint8_t)(inv ? 0 : x[1]);   // unused at an invariant site
                hInv[oSites[p] + i] = (uint8_t)inv;
            }
            P4G_CUDA(cudaMemcpyAsync(dStates.as<int8_t>() + oStates[p] + (size_t)t->root * nChar, hRoot.data(),
                                     nChar, cudaMemcpyHostToDevice, s));
            P4G_CUDA(cudaStreamSynchronize(s));   // hRoot is reused for the next part
        }
        P4G_CUDA(cudaMemcpyAsync(dCat.ptr, hCat.data(), nSites, cudaMemcpyHostToDevice, s));
        P4G_CUDA(cudaMemcpyAsync(dInv.ptr, hInv.data(), nSites, cudaMemcpyHostToDevice, s));
    } else {
        k_simRoot<<<grid, 256, 0, s>>>(dp, T);
    }
    k_simRank<<<nP, 1024, 0, s>>>(dp);
    k_simMutate<<<grid, 256, 0, s>>>(dp, T);
    P4G_CUDA(cudaGetLastError());
    std::vector<int8_t> hs(nStates);
    P4G_CUDA(cudaMemcpyAsync(hs.data(), dStates.ptr, nStates, cudaMemcpyDeviceToHost, s));
    P4G_CUDA(cudaStreamSynchronize(s));
    if (allStates) memcpy(allStates, hs.data(), nStates);
    // the leaves' states become the parts' sequences; their patterns are
    // stale until makePatterns, as p4_simulate leaves them (nPatterns = 0)
    for (int p = 0; p < nP; p++) {
        Part *dpart = d->parts[p];
        const int nChar = dpart->nChar;
        dpart->sequences.assign((size_t)dpart->nTax * nChar, 0);
        for (int v = 0; v < nn; v++) {
            const Node *nv = t->nodes[v];
            if (!nv->isLeaf || nv->seqNum < 0 || nv->seqNum >= dpart->nTax) continue;
            const int8_t *row = hs.data() + oStates[p] + (size_t)v * nChar;
            for (int k = 0; k < nChar; k++) dpart->sequences[(size_t)nv->seqNum * nChar + k] = row[k];
        }
        dpart->nPatterns = 0;
        dpart->patternsMade = false;
        dpart->invarMade = false;
        dpart->devValid = false;
        dpart->dev64Valid = false;
    }
    return resetTreeDev(t);   // pattern counts change: the tree's device state is rebuilt on next use
}

extern "C" int p4g_simulate(p4g_tree *tt, const double *uniforms, long long nUniforms, unsigned long long seed,
                            signed char *allStates)
{
    return simulateCore(reinterpret_cast<Tree *>(tt), uniforms, nUniforms, seed, allStates, nullptr);
}

extern "C" int p4g_simulateRef(p4g_tree *tt, p4g_tree *rr, const double *refUniforms, unsigned long long refSeed,
                               const double *uniforms, long long nUniforms, unsigned long long seed,
                               signed char *allStates)
{
    Tree *t = reinterpret_cast<Tree *>(tt), *r = reinterpret_cast<Tree *>(rr);
    if (!t || !r) return setError(P4G_EINVAL, "simulateRef: null tree");
    if (t == r) return setError(P4G_EINVAL, "simulateRef: the simulation tree is the reference tree");
    if (t->nParts != r->nParts) return setError(P4G_EINVAL, "simulateRef: the trees' part counts differ");
    for (int p = 0; p < t->nParts; p++)
        if (t->data->parts[p]->nChar != r->data->parts[p]->nChar ||
            t->model->parts[p].dim != r->model->parts[p].dim || t->model->parts[p].nCat != r->model->parts[p].nCat)
            return setError(P4G_EINVAL, "simulateRef: part %d differs between the trees", p);
    // every site's root state and category from the reference tree's root
    // posterior, parts in order, one uniform per site (p4_drawAncState)
    std::vector<std::vector<int>> draws(t->nParts);
    size_t off = 0;
    for (int p = 0; p < t->nParts; p++) {
        const int nChar = r->data->parts[p]->nChar;
        draws[p].assign(4 * (size_t)nChar, 0);
        RET(p4g_drawAncStates(rr, p, refUniforms ? refUniforms + off : nullptr, refSeed, draws[p].data()));
        off += nChar;
    }
    return simulateCore(t, uniforms, nUniforms, seed, allStates, &draws);
}
