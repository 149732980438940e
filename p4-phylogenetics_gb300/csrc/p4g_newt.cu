// Newton optimisation of branch lengths (Pf/p4_treeNewt.c), FP64 on the GPU.
//
// The reference's p4_newtAround visits the non-root nodes in post-order and
// runs Newton-Raphson on each node's branch length, using the node's
// conditional likelihoods from below (cl, the FP64 pruning) and from above
// (cl2: at the parent's end of the branch, the likelihood of everything
// outside the node's subtree, Pf/p4_node.c:860-1018).  The control flow is
// the reference's, on the host: the same flags (a node's cl is recomputed
// when a branch below it moved, cl2 once per round along the path from the
// first stale ancestor), the same Newton update, bounds and stopping rules.
// Each step's arithmetic runs on the GPU over all patterns at once:
//
//   k_newtDecks  P, dP/dt, d2P/dt2 of the moved node for every category, from
//                the eigensystems setPrams left in HBM (the formula k_pdeck
//                uses for P, so P is what setPrams would compute);
//   k_cl2        one node's cl2, one thread per (pattern, category);
//   k_newtSum    per pattern the site likelihood and its first and second
//                derivatives in the branch length, the pattern-weighted
//                lnL, d lnL/dt, d2 lnL/dt2 terms, summed per block (FP64);
//   k_node64     (the plain FP64 path's kernel) one node's cl.
//
// cl2 is stored for every node as [nNodes][nCat][dim][nPatPad] FP64 beside
// the FP64 path's cl of the internal nodes.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <algorithm>
#include <vector>
#include "p4g_internal.h"
#include "p4g_pmat.cuh"

using namespace p4g;

#define RET(call)                      \
    do {                               \
        int rc_ = (call);              \
        if (rc_ != P4G_OK) return rc_; \
    } while (0)

namespace {

constexpr int kMaxDim = 20;
constexpr int kMaxSibs = 16;
constexpr int kSumThreads = 128;

// One data part: where its decks, CLs and sums live.
struct NewtPart {
    double *decks64;         // [nNodes][nCat][dim][dim], row = parent state
    double *dP, *d2P;        // [nCat][dim][dim] of the moved node
    const double *eig;       // eigensystems [(c * nR + r)][n*n + 2n]: U, lambda, sqrt(pi)
    const double *rates;     // [nGdasrvs][nCat]
    const int *patterns;     // raw codes [nTax][nPat]
    const int *equates;      // [nEquates][dim]
    const double *cl;        // internal nodes' CLs [nInternal][nCat][dim][nPatPad]
    double *cl2;             // [nNodes][nCat][dim][nPatPad]
    const double *rootComp;  // [dim]
    const double *counts;    // [nPat]
    const uint32_t *invMask; // [nPat]
    double *sums;            // [nSumBlocks][3]
    double pInvar, relRate;
    int nPat, nPatPad, nCat, dim, nR;
    int cNum, rNum, gNum;    // the moved node's model components in this part (-1: no gdasrv)
};

// A node: its deck index and where its CL is (leaf: code row).
struct NodeRef {
    int node, internal, seqNum, pad_;
};

// The node whose cl2 is computed (k_cl2) or whose branch moves (k_newtSum).
struct NewtStep {
    NodeRef self;
    int parent, parentIsRoot, nSibs, pad_;
    NodeRef sibs[kMaxSibs];
};

// The tip factor of a leaf child, as p4_setCL2Down and the pruning treat
// codes (Pf/p4_node.c:948-990): P[s][code] for a state, nothing (1) for a
// gap, '?' or an all-states equate, the sum over members for other equates.
__device__ __forceinline__ double tipFactor(const double *P, int dim, int code, const int *equates, int s)
{
    if (code >= 0) return P[s * dim + code];
    if (code == GAP_CODE || code == QMARK_CODE || code == N_LIKE) return 1.0;
    const int *eq = equates + (code - EQUATES_BASE) * dim;
    bool isN = true;
    for (int j = 0; j < dim; j++)
        if (!eq[j]) isN = false;
    if (isN) return 1.0;
    double sum = 0.0;
    for (int j = 0; j < dim; j++)
        if (eq[j]) sum += P[s * dim + j];
    return sum;
}

// One block per part, one thread per (category, row): P(t), dP/dt, d2P/dt2
// of node v at branch length brLen.  t = brLen * r, r = rate * relRate
// (/(1 - pInvar)) as p4_calculateBigPDecks_1stD/2ndD form it
// (Pf/p4_node.c:442-540); dP = V diag(lambda r e^(lambda t)) V^-1,
// d2P = V diag((lambda r)^2 e^(lambda t)) V^-1 (Pf/eig.c:294-395), in the
// symmetric form of the eigensystem: P_ij = (sq_j / sq_i) sum_k U_ik e_k U_jk.
__global__ void k_newtDecks(NewtPart *parts, int v, double brLen, int derivs)
{
    NewtPart &A = parts[blockIdx.x];
    const int n = A.dim, cat = threadIdx.x / n, i = threadIdx.x % n;
    if (cat >= A.nCat) return;
    // t exactly as k_pdeck forms it (so P is what setPrams computes); the
    // derivative factor r as the reference's `temp`
    double t, r;
    if (A.gNum >= 0) {
        const double rate = A.rates[A.gNum * A.nCat + cat];
        t = brLen * rate * A.relRate;
        r = rate * A.relRate;
    } else {
        t = brLen * A.relRate;
        r = A.relRate;
    }
    if (A.pInvar != 0.0) {
        t = t / (1.0 - A.pInvar);
        r = r / (1.0 - A.pInvar);
    }
    const double *E = A.eig + (size_t)(A.cNum * A.nR + A.rNum) * eigRecDoubles(n);
    const double *lam = E + n * n, *sq = lam + n;
    double e0[kMaxDim], e1[kMaxDim], e2[kMaxDim];
    for (int k = 0; k < n; k++) {
        const double ek = exp(lam[k] * t);
        e0[k] = E[i * n + k] * ek;
        e1[k] = E[i * n + k] * (lam[k] * r * ek);
        e2[k] = E[i * n + k] * (lam[k] * r * lam[k] * r * ek);
    }
    const double ri = 1.0 / sq[i];
    double *P = A.decks64 + ((size_t)v * A.nCat + cat) * n * n + i * n;
    double *P1 = A.dP + (size_t)cat * n * n + i * n, *P2 = A.d2P + (size_t)cat * n * n + i * n;
    for (int j = 0; j < n; j++) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int k = 0; k < n; k++) {
            a0 += e0[k] * E[j * n + k];
            a1 += e1[k] * E[j * n + k];
            a2 += e2[k] * E[j * n + k];
        }
        const double f = sq[j] * ri;
        P[j] = a0 * f;
        if (derivs) {
            P1[j] = a1 * f;
            P2[j] = a2 * f;
        }
    }
}

// cl2 of node S.self (Pf/p4_treeNewt.c:597-619 with p4_initializeCL2ToRootComp,
// p4_setCL2Up, p4_setCL2Down): from the root composition when the parent is
// the root, else the parent's cl2 carried down the parent's branch
// (sum_from P_par[from][s] cl2_par[from]); times each sibling's transformed
// CL or tip factor, siblings in order.
__global__ void k_cl2(NewtPart *parts, NewtStep S)
{
    const NewtPart &A = parts[blockIdx.y];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.nPat * A.nCat) return;
    const int cat = q / A.nPat, pat = q % A.nPat, n = A.dim;
    const size_t plane = (size_t)A.nPatPad;
    double w[kMaxDim];
    if (S.parentIsRoot) {
        for (int s = 0; s < n; s++) w[s] = A.rootComp[s];
    } else {
        const double *P = A.decks64 + ((size_t)S.parent * A.nCat + cat) * n * n;
        const double *up = A.cl2 + ((size_t)S.parent * A.nCat + cat) * n * plane + pat;
        double u[kMaxDim];
        for (int f = 0; f < n; f++) u[f] = up[f * plane];
        for (int s = 0; s < n; s++) {
            double sum = 0.0;
            for (int f = 0; f < n; f++) sum += P[f * n + s] * u[f];
            w[s] = sum;
        }
    }
    for (int k = 0; k < S.nSibs; k++) {
        const NodeRef &b = S.sibs[k];
        const double *P = A.decks64 + ((size_t)b.node * A.nCat + cat) * n * n;
        if (b.internal < 0) {
            const int code = A.patterns[(size_t)b.seqNum * A.nPat + pat];
            for (int s = 0; s < n; s++) w[s] *= tipFactor(P, n, code, A.equates, s);
        } else {
            const double *x = A.cl + ((size_t)b.internal * A.nCat + cat) * n * plane + pat;
            double xv[kMaxDim];
            for (int j = 0; j < n; j++) xv[j] = x[j * plane];
            for (int s = 0; s < n; s++) {
                double sum = 0.0;
                for (int j = 0; j < n; j++) sum += P[s * n + j] * xv[j];
                w[s] *= sum;
            }
        }
    }
    double *out = A.cl2 + ((size_t)S.self.node * A.nCat + cat) * n * plane + pat;
    for (int s = 0; s < n; s++) out[s * plane] = w[s];
}

// Per pattern (p4_newtNode, Pf/p4_treeNewt.c:240-520): like, first and
// second over categories from cl2 of the moved node and its CL (internal)
// or its code (leaf), weighted and combined as the reference does; the
// block sums (lnL, d lnL, d2 lnL) go to sums[block].
__global__ void __launch_bounds__(kSumThreads) k_newtSum(NewtPart *parts, NewtStep S)
{
    const NewtPart &A = parts[blockIdx.y];
    if (blockIdx.x * kSumThreads >= A.nPat) return;   // the grid covers the largest part
    const int pat = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = A.dim;
    const size_t plane = (size_t)A.nPatPad;
    double lnL = 0.0, d1 = 0.0, d2 = 0.0;
    if (pat < A.nPat) {
        double likeS = 0.0, firstS = 0.0, secondS = 0.0;
        const bool leaf = S.self.internal < 0;
        const int code = leaf ? A.patterns[(size_t)S.self.seqNum * A.nPat + pat] : 0;
        bool isN = false;
        const int *eq = nullptr;
        if (leaf && code < 0 && code != GAP_CODE && code != QMARK_CODE) {
            if (code == N_LIKE) {
                isN = true;
            } else {
                eq = A.equates + (code - EQUATES_BASE) * n;
                isN = true;
                for (int j = 0; j < n; j++)
                    if (!eq[j]) isN = false;
            }
        }
        for (int cat = 0; cat < A.nCat; cat++) {
            const double *P = A.decks64 + ((size_t)S.self.node * A.nCat + cat) * n * n;
            const double *P1 = A.dP + (size_t)cat * n * n, *P2 = A.d2P + (size_t)cat * n * n;
            const double *c2 = A.cl2 + ((size_t)S.self.node * A.nCat + cat) * n * plane + pat;
            double like = 0.0, first = 0.0, second = 0.0;
            if (!leaf) {
                const double *x = A.cl + ((size_t)S.self.internal * A.nCat + cat) * n * plane + pat;
                for (int f = 0; f < n; f++) {
                    const double a = c2[f * plane];
                    for (int to = 0; to < n; to++) {
                        const double tmp = a * x[to * plane];
                        like += tmp * P[f * n + to];
                        first += tmp * P1[f * n + to];
                        second += tmp * P2[f * n + to];
                    }
                }
            } else if (code >= 0) {
                for (int f = 0; f < n; f++) {
                    const double a = c2[f * plane];
                    like += a * P[f * n + code];
                    first += a * P1[f * n + code];
                    second += a * P2[f * n + code];
                }
            } else if (code == GAP_CODE || code == QMARK_CODE) {
                for (int f = 0; f < n; f++) {
                    const double a = c2[f * plane];
                    like += a;
                    for (int to = 0; to < n; to++) {
                        first += a * P1[f * n + to];
                        second += a * P2[f * n + to];
                    }
                }
            } else {
                for (int f = 0; f < n; f++) {
                    const double a = c2[f * plane];
                    for (int to = 0; to < n; to++) {
                        if (isN || eq[to]) {
                            like += a * P[f * n + to];
                            first += a * P1[f * n + to];
                            second += a * P2[f * n + to];
                        }
                    }
                }
            }
            likeS += like;
            firstS += first;
            secondS += second;
        }
        if (A.pInvar != 0.0) {
            const double fr = (1.0 - A.pInvar) / (double)A.nCat;
            likeS *= fr;
            firstS *= fr;
            secondS *= fr;
            const uint32_t im = A.invMask[pat];
            for (int f = 0; f < n; f++)
                if ((im >> f) & 1u) likeS += A.rootComp[f] * A.pInvar;
        } else if (A.nCat > 1) {
            likeS /= (double)A.nCat;
            firstS /= (double)A.nCat;
            secondS /= (double)A.nCat;
        }
        const double w = A.counts[pat];
        if (likeS < 1.0e-300) {
            lnL = w * -100000.0;
            d1 = w * 1000000.0;
            d2 = w * 10000000.0;
        } else {
            lnL = w * log(likeS);
            d1 = w * (firstS / likeS);
            d2 = w * ((secondS * likeS - firstS * firstS) / (likeS * likeS));
        }
    }
    __shared__ double red[3][kSumThreads / 32];
    for (int o = 16; o; o >>= 1) {
        lnL += __shfl_down_sync(0xffffffffu, lnL, o);
        d1 += __shfl_down_sync(0xffffffffu, d1, o);
        d2 += __shfl_down_sync(0xffffffffu, d2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = lnL;
        red[1][threadIdx.x >> 5] = d1;
        red[2][threadIdx.x >> 5] = d2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int w = 0; w < kSumThreads / 32; w++) s += red[threadIdx.x][w];
        A.sums[(size_t)blockIdx.x * 3 + threadIdx.x] = s;
    }
}

// ------------------------------------------------------------------ host

struct Newt {
    Tree *t;
    std::vector<NewtPart> parts;
    DevBuf dParts;
    std::vector<int> internalOf;   // node -> internal index of the FP64 path (-1: leaf)
    std::vector<char> clStale, cl2Stale;
    std::vector<size_t> oSums;
    int sumBlocks = 0, maxPatCat = 0, maxPat = 0;
    double brMin = 1e-8, brMax = 3.0;
};

int uploadParts(Newt &N)
{
    P4G_CUDA(cudaMemcpyAsync(N.dParts.ptr, N.parts.data(), sizeof(NewtPart) * N.parts.size(),
                             cudaMemcpyHostToDevice, ctx().stream));
    return P4G_OK;
}

NodeRef refOf(const Newt &N, int v)
{
    NodeRef r;
    r.node = v;
    r.internal = N.internalOf[v];
    r.seqNum = N.t->nodes[v]->seqNum;
    r.pad_ = 0;
    return r;
}

int stepOf(const Newt &N, int v, NewtStep &S)
{
    Tree *t = N.t;
    const int par = t->nodes[v]->parent;
    memset(&S, 0, sizeof(S));
    S.self = refOf(N, v);
    S.parent = par;
    S.parentIsRoot = (par == t->root);
    for (int c = t->nodes[par]->leftChild; c >= 0; c = t->nodes[c]->sibling) {
        if (c == v) continue;
        if (S.nSibs == kMaxSibs) return setError(P4G_EUNSUPPORTED, "newtAround: more than %d siblings", kMaxSibs);
        S.sibs[S.nSibs++] = refOf(N, c);
    }
    return P4G_OK;
}

int launchCl2(Newt &N, int v)
{
    NewtStep S;
    RET(stepOf(N, v, S));
    const dim3 grid((N.maxPatCat + 127) / 128, (unsigned)N.parts.size());
    k_cl2<<<grid, 128, 0, ctx().stream>>>(N.dParts.as<NewtPart>(), S);
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

// One node's FP64 CL from its children (the plain path's kernel, one launch
// per part).
int launchCl(Newt &N, int v)
{
    TreeDev &dv = N.t->dev;
    for (size_t p = 0; p < N.parts.size(); p++)
        RET(launchNode64(dv.dJobs64.as<Node64Job>() + p, dv.jobs64[p], N.internalOf[v], ctx().stream));
    return P4G_OK;
}

int setModelOfNode(Newt &N, int v)
{
    Tree *t = N.t;
    for (size_t p = 0; p < N.parts.size(); p++) {
        const Node *nv = t->nodes[v];
        N.parts[p].cNum = nv->compNums[p];
        N.parts[p].rNum = nv->rMatrixNums[p];
        N.parts[p].gNum = t->model->parts[p].nGdasrvs ? nv->gdasrvNums[p] : -1;
    }
    return uploadParts(N);
}

// p4_newtNode (Pf/p4_treeNewt.c:210-590): Newton-Raphson on node v's branch.
int newtNode(Newt &N, int v, double epsilon)
{
    Tree *t = N.t;
    Node *nv = t->nodes[v];
    RET(setModelOfNode(N, v));
    NewtStep S;
    RET(stepOf(N, v, S));
    cudaStream_t s = ctx().stream;
    const double oldBrLen = nv->brLen;
    double currentGuess = oldBrLen;
    int iter = 0;
    std::vector<double> hs((size_t)N.sumBlocks * 3);
    const dim3 grid((N.maxPat + kSumThreads - 1) / kSumThreads, (unsigned)N.parts.size());
    while (true) {
        k_newtDecks<<<(unsigned)N.parts.size(), kMaxDim * 16, 0, s>>>(N.dParts.as<NewtPart>(), v, currentGuess, 1);
        k_newtSum<<<grid, kSumThreads, 0, s>>>(N.dParts.as<NewtPart>(), S);
        P4G_CUDA(cudaGetLastError());
        P4G_CUDA(cudaMemcpyAsync(hs.data(), N.t->dev.dNewtSums.ptr, sizeof(double) * hs.size(),
                                 cudaMemcpyDeviceToHost, s));
        P4G_CUDA(cudaStreamSynchronize(s));
        double firstD = 0.0, secondD = 0.0;
        for (size_t p = 0; p < N.parts.size(); p++) {
            const int nb = (N.parts[p].nPat + kSumThreads - 1) / kSumThreads;
            for (int b = 0; b < nb; b++) {
                firstD += hs[N.oSums[p] + (size_t)b * 3 + 1];
                secondD += hs[N.oSums[p] + (size_t)b * 3 + 2];
            }
        }
        double nextGuess = currentGuess - (firstD / secondD);
        if (secondD >= 0.0) nextGuess = currentGuess / 5.0;
        if (nextGuess < N.brMin) {
            nv->brLen = N.brMin;
            break;
        }
        if (nextGuess >= 5.0 * oldBrLen) {
            nv->brLen = 5.0 * oldBrLen;
            break;
        }
        if (nextGuess > N.brMax) {
            nv->brLen = N.brMax;
            break;
        }
        if (iter > 20) {
            nv->brLen = currentGuess;
            break;
        }
        iter++;
        if (fabs(firstD) < epsilon) {
            nv->brLen = currentGuess;
            break;
        }
        currentGuess = nextGuess;
        nv->brLen = nextGuess;
    }
    // P of the final branch length, for the CLs that follow
    k_newtDecks<<<(unsigned)N.parts.size(), kMaxDim * 16, 0, s>>>(N.dParts.as<NewtPart>(), v, nv->brLen, 0);
    P4G_CUDA(cudaGetLastError());
    return P4G_OK;
}

int newtSetup(Tree *t, Newt &N, double *lnL)
{
    if (t->root < 0 || !t->nodes[t->root] || t->nodes[t->root]->isLeaf)
        return setError(P4G_EUNSUPPORTED, "newtAround: the root must be an internal node");
    for (int p = 0; p < t->nParts; p++) {
        if (t->model->parts[p].dim > kMaxDim) return setError(P4G_EUNSUPPORTED, "newtAround: dim > %d", kMaxDim);
        if (t->model->parts[p].nCat > 16) return setError(P4G_EUNSUPPORTED, "newtAround: more than 16 categories");
    }
    N.t = t;
    // setPrams and every internal CL (p4_treeLogLike at the start of p4_newtAround)
    RET(fp64Evaluate(t, true, lnL));
    TreeDev &dv = t->dev;
    const int nn = t->nNodes;
    N.internalOf.assign(nn, -1);
    for (size_t k = 0; k < dv.nodeStart64.size(); k++) N.internalOf[dv.table64[dv.nodeStart64[k]]] = (int)k;
    size_t nCl2 = 0, nSums = 0;
    N.oSums.assign(t->nParts, 0);
    std::vector<size_t> oCl2(t->nParts), oP(t->nParts);
    size_t nP = 0;
    for (int p = 0; p < t->nParts; p++) {
        const ModelPart &mp = t->model->parts[p];
        const Part *dp = t->data->parts[p];
        oCl2[p] = nCl2;
        nCl2 += (size_t)nn * mp.nCat * mp.dim * dp->nPatPad;
        N.oSums[p] = nSums;
        nSums += (size_t)((dp->nPatterns + kSumThreads - 1) / kSumThreads) * 3;
        oP[p] = nP;
        nP += (size_t)2 * mp.nCat * mp.dim * mp.dim;
        N.maxPat = std::max(N.maxPat, dp->nPatterns);
        N.maxPatCat = std::max(N.maxPatCat, dp->nPatterns * mp.nCat);
    }
    N.sumBlocks = (int)(nSums / 3);
    RET(dv.dCl2.ensure(sizeof(double) * nCl2));
    RET(dv.dNewtP.ensure(sizeof(double) * nP));
    RET(dv.dNewtSums.ensure(sizeof(double) * nSums));
    P4G_CUDA(cudaMemsetAsync(dv.dNewtSums.ptr, 0, sizeof(double) * nSums, ctx().stream));
    N.parts.resize(t->nParts);
    for (int p = 0; p < t->nParts; p++) {
        const ModelPart &mp = t->model->parts[p];
        const Node64Job &J = dv.jobs64[p];
        NewtPart &A = N.parts[p];
        A.decks64 = dv.dDecks64.as<double>() + dv.oDecks[p];
        A.dP = dv.dNewtP.as<double>() + oP[p];
        A.d2P = A.dP + (size_t)mp.nCat * mp.dim * mp.dim;
        A.eig = dv.dEig.as<double>() + dv.oEig[p];
        A.rates = dv.dRates.as<double>() + dv.oRates[p];
        A.patterns = J.patterns;
        A.equates = J.equates;
        A.cl = J.cl;
        A.cl2 = dv.dCl2.as<double>() + oCl2[p];
        A.rootComp = J.rootComp;
        A.counts = J.counts;
        A.invMask = J.invMask;
        A.sums = dv.dNewtSums.as<double>() + N.oSums[p];
        A.pInvar = mp.pInvar;
        A.relRate = mp.relRate;
        A.nPat = J.nPat;
        A.nPatPad = J.nPatPad;
        A.nCat = mp.nCat;
        A.dim = mp.dim;
        A.nR = mp.nRMatrices;
        A.cNum = A.rNum = 0;
        A.gNum = -1;
    }
    RET(N.dParts.ensure(sizeof(NewtPart) * N.parts.size()));
    RET(uploadParts(N));
    if (t->model->bounds[12]) N.brMin = *t->model->bounds[12];
    if (t->model->bounds[13]) N.brMax = *t->model->bounds[13];
    N.clStale.assign(nn, 0);
    N.cl2Stale.assign(nn, 0);
    return P4G_OK;
}

// The p4 post-order of the tree (the aliased postOrder array, entries < 0
// not in the tree).
std::vector<int> postOrderOf(Tree *t)
{
    std::vector<int> out;
    for (int k = 0; k < t->nNodes; k++) {
        const int v = t->postOrder ? t->postOrder[k] : -1;
        if (v >= 0 && v < t->nNodes) out.push_back(v);
    }
    if ((int)out.size() == 0) {   // no order given: children before parents from the relations
        std::vector<int> st{t->root};
        std::vector<char> seen(t->nNodes, 0);
        while (!st.empty()) {
            const int v = st.back();
            if (!seen[v]) {
                seen[v] = 1;
                std::vector<int> kids;
                for (int c = t->nodes[v]->leftChild; c >= 0; c = t->nodes[c]->sibling) kids.push_back(c);
                for (auto it = kids.rbegin(); it != kids.rend(); ++it) st.push_back(*it);
            } else {
                st.pop_back();
                out.push_back(v);
            }
        }
    }
    return out;
}

// p4_newtAround (Pf/p4_treeNewt.c:79-208).
int newtAround(Tree *t, double epsilon, double likeDelta, double *lnLOut)
{
    Newt N;
    double previousLogLike = 0.0;
    RET(newtSetup(t, N, &previousLogLike));
    const std::vector<int> post = postOrderOf(t);
    double thisLogLike = previousLogLike;
    for (int round = 0; round < 20; round++) {
        for (int v : post)
            if (v != t->root) N.cl2Stale[v] = 1;
        for (int v : post) {
            if (v == t->root) continue;
            Node *nv = t->nodes[v];
            if (!nv->isLeaf && N.clStale[v]) {
                RET(launchCl(N, v));
                N.clStale[v] = 0;
            }
            if (N.cl2Stale[v]) {
                std::vector<int> path;
                for (int p = v; t->nodes[p]->parent >= 0 && N.cl2Stale[p]; p = t->nodes[p]->parent) path.push_back(p);
                for (int j = (int)path.size() - 1; j >= 0; j--) {
                    RET(launchCl2(N, path[j]));
                    N.cl2Stale[path[j]] = 0;
                }
            }
            RET(newtNode(N, v, epsilon));
            for (int p = nv->parent; p >= 0; p = t->nodes[p]->parent) N.clStale[p] = 1;
        }
        // p4_treeLogLike on the new branch lengths (every CL recomputed)
        RET(fp64Evaluate(t, false, &thisLogLike));
        std::fill(N.clStale.begin(), N.clStale.end(), 0);
        const double diff = thisLogLike - previousLogLike;
        if (fabs(diff) < likeDelta) break;
        previousLogLike = thisLogLike;
    }
    if (lnLOut) *lnLOut = thisLogLike;
    return P4G_OK;
}

// ------------------------------------------------------------ model-parameter optimisation
// Tree.optLogLike(method="newtAndBrentPowell") (p4/tree.py:9467-9470 ->
// p4_newtAndBrentPowellOpt, Pf/p4_treeOpt.c:1182-1392): Newton passes over
// the branch lengths alternating with a derivative-free search over the free
// model parameters, until a pass changes lnL by less than 1e-6 (or the
// tree's pass limit is reached).  The reference searches with praxis
// (Brent's principal-axis method, Pf/brent.c); the search here is Powell's
// conjugate-direction method (M. J. D. Powell, Comput. J. 7:155, 1964) with
// Brent's line minimisation by golden section and parabolic interpolation
// (R. P. Brent, Algorithms for Minimization without Derivatives, 1973, ch. 5),
// written for this library, over an unconstrained reparameterisation:
//   a composition (dim values summing to 1) -> dim-1 logs of ratios to its last value;
//   an R matrix's dim(dim-1)/2 rates        -> logs of ratios to its last rate
//                                              (rates normalised to sum 1), or
//                                              logs of all but the last (last fixed);
//   a gamma shape                           -> its log;
//   pInvar                                  -> itself;
//   the relative rates of parts 0..n-2      -> logs; the last part's rate keeps
//                                              the site-weighted mean rate at 1;
//   (trees of fewer than 15 nodes, after the alternation, as the reference's
//   p4_allBrentPowellOptimize: also every branch length, by its log).
// Values are clamped to p4's bounds (the model's PIVEC_MIN, RATE_MIN, ...)
// when written back.  Each function value is an FP64 evaluation (setPrams +
// the plain FP64 pruning) on the GPU.
enum OptKind { O_COMP, O_RMAT, O_GAMMA, O_PINVAR, O_RELRATE, O_BRLEN };
struct OptBlock {
    int kind, part, idx, n, x0;
};

struct Opt {
    Tree *t = nullptr;
    std::vector<OptBlock> blocks;
    std::vector<double> step;   // first step of each coordinate's line search
    std::vector<double> rLast;  // per R-matrix block: the fixed last rate (not normalised to 1)
    int nX = 0, nEvals = 0;
    double fail = 0.0;          // first evaluation error (as a code), 0 if none

    double bnd(int k, double def) const { return t->model->bounds[k] ? *t->model->bounds[k] : def; }
    bool normR() const { return t->model->rMatrixNormalizeTo1 && t->model->rMatrixNormalizeTo1[0]; }
};

static void rUpper(const RMatrix &r, int dim, std::vector<double> &u)
{
    u.clear();
    for (int i = 0; i < dim - 1; i++)
        for (int j = i + 1; j < dim; j++) u.push_back(r.bigR[(size_t)i * dim + j]);
}

// The free parameters, as p4_windUpParameters counts them (Pf/p4_treeOpt.c:19-115).
static int optSpace(Opt &O, bool withBrLens)
{
    Tree *t = O.t;
    Model *m = t->model;
    O.blocks.clear();
    O.step.clear();
    O.rLast.clear();
    int n = 0, nModel = 0;
    auto add = [&](int kind, int part, int idx, int k, double st) {
        O.blocks.push_back(OptBlock{kind, part, idx, k, n});
        for (int i = 0; i < k; i++) O.step.push_back(st);
        n += k;
    };
    for (int p = 0; p < t->nParts; p++) {
        const ModelPart &mp = m->parts[p];
        for (int c = 0; c < mp.nComps; c++)
            if (mp.comps[c].free) add(O_COMP, p, c, mp.dim - 1, 0.3);
        for (int r = 0; r < mp.nRMatrices; r++)
            if (mp.rMatrices[r].free) {
                add(O_RMAT, p, r, mp.dim * (mp.dim - 1) / 2 - 1, 0.3);
                std::vector<double> u;
                rUpper(mp.rMatrices[r], mp.dim, u);
                O.rLast.push_back(u.back());
            }
        for (int g = 0; g < mp.nGdasrvs; g++)
            if (mp.gdasrvs[g]->free) add(O_GAMMA, p, g, 1, 0.3);
        if (mp.pInvarFree) add(O_PINVAR, p, 0, 1, 0.05);
    }
    if (m->relRatesAreFree)
        for (int p = 0; p < t->nParts - 1; p++) add(O_RELRATE, p, 0, 1, 0.2);
    nModel = n;
    if (withBrLens)
        for (int v = 0; v < t->nNodes; v++)
            if (v != t->root && t->nodes[v]) add(O_BRLEN, v, 0, 1, 0.3);
    O.nX = n;
    return nModel;
}

static void windUp(const Opt &O, std::vector<double> &x)
{
    Tree *t = O.t;
    Model *m = t->model;
    x.assign(O.nX, 0.0);
    int ri = 0;
    for (const OptBlock &B : O.blocks) {
        double *y = x.data() + B.x0;
        switch (B.kind) {
        case O_COMP: {
            const double *v = m->parts[B.part].comps[B.idx].val;
            const int d = m->parts[B.part].dim;
            for (int i = 0; i < d - 1; i++) y[i] = log(v[i]) - log(v[d - 1]);
            break;
        }
        case O_RMAT: {
            std::vector<double> u;
            rUpper(m->parts[B.part].rMatrices[B.idx], m->parts[B.part].dim, u);
            const size_t K = u.size();
            for (size_t k = 0; k + 1 < K; k++) y[k] = O.normR() ? log(u[k]) - log(u[K - 1]) : log(u[k]);
            ri++;
            break;
        }
        case O_GAMMA: y[0] = log(m->parts[B.part].gdasrvs[B.idx]->val[0]); break;
        case O_PINVAR: y[0] = m->parts[B.part].pInvar; break;
        case O_RELRATE: y[0] = log(m->parts[B.part].relRate); break;
        case O_BRLEN: y[0] = log(t->nodes[B.part]->brLen); break;
        }
    }
}

static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Positive values normalised to sum 1 with every value >= lo (and the last
// rounding put on the largest value).
static void normalise(std::vector<double> &v, double lo)
{
    for (int pass = 0; pass < 2; pass++) {
        double s = 0.0;
        for (double &a : v) {
            a = std::max(a, lo);
            s += a;
        }
        for (double &a : v) a /= s;
    }
    double s = 0.0;
    size_t big = 0;
    for (size_t i = 0; i < v.size(); i++) {
        s += v[i];
        if (v[i] > v[big]) big = i;
    }
    v[big] += 1.0 - s;
}

static void unWind(const Opt &O, const std::vector<double> &x)
{
    Tree *t = O.t;
    Model *m = t->model;
    int ri = 0;
    for (const OptBlock &B : O.blocks) {
        const double *y = x.data() + B.x0;
        switch (B.kind) {
        case O_COMP: {
            ModelPart &mp = m->parts[B.part];
            std::vector<double> v(mp.dim);
            for (int i = 0; i < mp.dim - 1; i++) v[i] = exp(clampd(y[i], -60.0, 60.0));
            v[mp.dim - 1] = 1.0;
            normalise(v, O.bnd(6, 1e-13));
            for (int i = 0; i < mp.dim; i++) mp.comps[B.idx].val[i] = v[i];
            break;
        }
        case O_RMAT: {
            ModelPart &mp = m->parts[B.part];
            const int d = mp.dim, K = d * (d - 1) / 2;
            std::vector<double> u(K);
            for (int k = 0; k < K - 1; k++) u[k] = exp(clampd(y[k], -60.0, 60.0));
            if (O.normR()) {
                u[K - 1] = 1.0;
                normalise(u, O.bnd(8, 1e-13));
            } else {
                u[K - 1] = O.rLast[ri];
            }
            int k = 0;
            for (int i = 0; i < d - 1; i++)
                for (int j = i + 1; j < d; j++) {
                    mp.rMatrices[B.idx].bigR[(size_t)i * d + j] = u[k];
                    mp.rMatrices[B.idx].bigR[(size_t)j * d + i] = u[k];
                    k++;
                }
            ri++;
            break;
        }
        case O_GAMMA:
            m->parts[B.part].gdasrvs[B.idx]->val[0] = clampd(exp(clampd(y[0], -60.0, 60.0)), O.bnd(4, 0.1), O.bnd(5, 300.0));
            break;
        case O_PINVAR: m->parts[B.part].pInvar = clampd(y[0], O.bnd(0, 0.0), O.bnd(1, 0.99)); break;
        case O_RELRATE:
            m->parts[B.part].relRate = clampd(exp(clampd(y[0], -60.0, 60.0)), O.bnd(10, 1e-8), O.bnd(11, 1e8));
            break;
        case O_BRLEN:
            t->nodes[B.part]->brLen = clampd(exp(clampd(y[0], -60.0, 60.0)), O.bnd(12, 1e-8), O.bnd(13, 3.0));
            break;
        }
    }
    if (m->relRatesAreFree && t->nParts > 1) {   // the last part keeps the site-weighted mean at 1
        double tot = 0.0, rest = 0.0;
        for (int p = 0; p < t->nParts; p++) tot += t->data->parts[p]->nChar;
        for (int p = 0; p < t->nParts - 1; p++) rest += m->parts[p].relRate * t->data->parts[p]->nChar;
        const int last = t->nParts - 1;
        m->parts[last].relRate = std::max((tot - rest) / t->data->parts[last]->nChar, O.bnd(10, 1e-8));
    }
}

// -lnL at x (FP64 setPrams + pruning); a failed or non-positive evaluation
// counts as +infinity, the first error code is kept.
static double optF(Opt &O, const std::vector<double> &x)
{
    unWind(O, x);
    O.nEvals++;
    double lnL = 0.0;
    const int rc = fp64Evaluate(O.t, true, &lnL);
    if (rc != P4G_OK) {
        if (O.fail == 0.0) O.fail = rc;
        return INFINITY;
    }
    if (!(lnL > -1.0e98)) return INFINITY;
    return -lnL;
}

// Minimise f(x + a d) over a (Brent 1973, ch. 5): bracket from a = 0 and
// a = 1 by golden-ratio expansion, then golden-section steps and parabolic
// interpolation.  x and fx move to the minimum found.
static void lineMin(Opt &O, std::vector<double> &x, const std::vector<double> &d, double &fx)
{
    const double G = 1.618033988749895, CG = 0.3819660112501051;
    const size_t n = x.size();
    std::vector<double> xt(n);
    auto g = [&](double a) {
        for (size_t i = 0; i < n; i++) xt[i] = x[i] + a * d[i];
        return optF(O, xt);
    };
    double a = 0.0, fa = fx, b = 1.0, fb = g(b);
    if (fb > fa) {
        std::swap(a, b);
        std::swap(fa, fb);
    }
    double c = b + G * (b - a), fc = g(c);
    for (int k = 0; k < 60 && fc < fb; k++) {
        a = b;
        fa = fb;
        b = c;
        fb = fc;
        c = b + G * (b - a);
        fc = g(c);
    }
    // Brent's minimiser on [lo, hi] starting from the bracket's middle point
    double lo = std::min(a, c), hi = std::max(a, c);
    double xm = b, w = b, v = b, fxm = fb, fw = fb, fv = fb, e = 0.0, dd = 0.0;
    for (int it = 0; it < 100; it++) {
        const double mid = 0.5 * (lo + hi);
        const double tol1 = 1.0e-5 * fabs(xm) + 1.0e-8, tol2 = 2.0 * tol1;
        if (fabs(xm - mid) <= tol2 - 0.5 * (hi - lo)) break;
        bool golden = true;
        if (fabs(e) > tol1) {   // try a parabola through x, w, v
            double r = (xm - w) * (fxm - fv), q = (xm - v) * (fxm - fw), p = (xm - v) * q - (xm - w) * r;
            q = 2.0 * (q - r);
            if (q > 0.0) p = -p;
            q = fabs(q);
            const double eOld = e;
            e = dd;
            if (fabs(p) < fabs(0.5 * q * eOld) && p > q * (lo - xm) && p < q * (hi - xm)) {
                dd = p / q;
                const double u = xm + dd;
                if (u - lo < tol2 || hi - u < tol2) dd = (mid >= xm) ? tol1 : -tol1;
                golden = false;
            }
        }
        if (golden) {
            e = (xm >= mid) ? lo - xm : hi - xm;
            dd = CG * e;
        }
        const double u = (fabs(dd) >= tol1) ? xm + dd : xm + (dd > 0.0 ? tol1 : -tol1);
        const double fu = g(u);
        if (fu <= fxm) {
            if (u >= xm) lo = xm;
            else hi = xm;
            v = w;
            fv = fw;
            w = xm;
            fw = fxm;
            xm = u;
            fxm = fu;
        } else {
            if (u < xm) lo = u;
            else hi = u;
            if (fu <= fw || w == xm) {
                v = w;
                fv = fw;
                w = u;
                fw = fu;
            } else if (fu <= fv || v == xm || v == w) {
                v = u;
                fv = fu;
            }
        }
    }
    if (fxm < fx) {
        for (size_t i = 0; i < n; i++) x[i] += xm * d[i];
        fx = fxm;
    }
    unWind(O, x);
}

// Powell's method from x (f(x) = fx): line searches along n directions,
// then along the pass's net displacement, which replaces the direction of
// largest decrease when Powell's test accepts it.  Returns f at the result.
static double powell(Opt &O, std::vector<double> &x, double fx)
{
    const size_t n = x.size();
    std::vector<std::vector<double>> dirs(n, std::vector<double>(n, 0.0));
    for (size_t i = 0; i < n; i++) dirs[i][i] = O.step[i];
    std::vector<double> xs(n), xe(n), dn(n);
    for (int it = 0; it < 200; it++) {
        const double fs = fx;
        xs = x;
        double big = 0.0;
        size_t ibig = 0;
        for (size_t i = 0; i < n; i++) {
            const double fp = fx;
            lineMin(O, x, dirs[i], fx);
            if (fp - fx > big) {
                big = fp - fx;
                ibig = i;
            }
        }
        if (2.0 * (fs - fx) <= 1.0e-10 * (fabs(fs) + fabs(fx)) + 1.0e-12) break;
        for (size_t i = 0; i < n; i++) {
            xe[i] = 2.0 * x[i] - xs[i];
            dn[i] = x[i] - xs[i];
        }
        const double fe = optF(O, xe);
        unWind(O, x);
        if (fe < fs) {
            const double tt = 2.0 * (fs - 2.0 * fx + fe) * (fs - fx - big) * (fs - fx - big) - big * (fs - fe) * (fs - fe);
            if (tt < 0.0) {
                lineMin(O, x, dn, fx);
                dirs[ibig] = dirs[n - 1];
                dirs[n - 1] = dn;
            }
        }
    }
    return fx;
}

int newtAndBrentPowellOpt(Tree *t)
{
    Opt O;
    O.t = t;
    double lnL = 0.0;
    // the model's nFreePrams decides, as in the reference: with none, branch
    // lengths only, whatever the free flags say
    const int nModel = t->model->nFreePrams == 0 ? 0 : optSpace(O, false);
    if (nModel != t->model->nFreePrams)
        return setError(P4G_EINVAL, "newtAndBrentPowellOpt: the model says %d free parameters, the free flags give %d",
                        t->model->nFreePrams, nModel);
    if (nModel == 0) {   // Pf/p4_treeOpt.c:1215-1224
        const double eps[4] = {1.0, 1.0e-1, 1.0e-2, 1.0e-5}, delta[4] = {10.0, 1.0, 0.1, 1.0e-7};
        for (int k = 0; k < 4; k++) RET(newtAround(t, eps[k], delta[k], &lnL));
        return P4G_OK;
    }
    const double eps[3] = {1.0, 1.0e-1, 1.0e-5}, delta[3] = {10.0, 1.0, 1.0e-7};
    for (int k = 0; k < 3; k++) RET(newtAround(t, eps[k], delta[k], &lnL));
    std::vector<double> x;
    windUp(O, x);
    double prev = -optF(O, x);
    const int limit = t->passLimit ? t->passLimit[0] : 50;
    for (int pass = 0;; pass++) {
        RET(newtAround(t, 1.0e-5, 1.0e-7, &lnL));
        windUp(O, x);
        const double cur = -powell(O, x, -lnL);
        if (O.fail != 0.0) return setError((int)O.fail, "newtAndBrentPowellOpt: an evaluation failed");
        unWind(O, x);
        if (fabs(cur - prev) < 1.0e-6 || pass >= limit) break;
        prev = cur;
    }
    if (t->nNodes < 15) {   // small trees: every branch length as well (Pf/p4_treeOpt.c:1384-1388)
        Opt A;
        A.t = t;
        optSpace(A, true);
        std::vector<double> y;
        windUp(A, y);
        double f = optF(A, y);
        for (int pass = 0; pass < 50; pass++) {
            const double f0 = f;
            f = powell(A, y, f);
            if (fabs(f - f0) < 1.0e-6) break;
        }
        unWind(A, y);
        if (A.fail != 0.0) return setError((int)A.fail, "newtAndBrentPowellOpt: an evaluation failed");
    }
    RET(fp64Evaluate(t, true, &lnL));
    return P4G_OK;
}

}  // namespace

extern "C" int p4g_newtSetup(p4g_tree *tt)
{
    Tree *t = reinterpret_cast<Tree *>(tt);
    if (!t) return setError(P4G_EINVAL, "newtSetup: null tree");
    return P4G_OK;   // the buffers are sized by each p4g_newtAround call
}

extern "C" int p4g_newtAround(p4g_tree *tt, double epsilon, double likeDelta)
{
    Tree *t = reinterpret_cast<Tree *>(tt);
    if (!t) return setError(P4G_EINVAL, "newtAround: null tree");
    double lnL = 0.0;
    RET(newtAround(t, epsilon, likeDelta, &lnL));
    t->dev.cacheValid = false;   // branch lengths moved: the next setPrams recomputes every deck
    return P4G_OK;
}

extern "C" int p4g_newtAndBrentPowellOpt(p4g_tree *tt)
{
    Tree *t = reinterpret_cast<Tree *>(tt);
    if (!t) return setError(P4G_EINVAL, "newtAndBrentPowellOpt: null tree");
    const int rc = newtAndBrentPowellOpt(t);
    t->dev.cacheValid = false;   // branch lengths and model values moved
    return rc;
}

extern "C" int p4g_getFreePrams(p4g_tree *tt, double *out, int cap, int *n)
{
    Tree *t = reinterpret_cast<Tree *>(tt);
    if (!t || !n || (cap > 0 && !out)) return setError(P4G_EINVAL, "getFreePrams: bad arguments");
    std::vector<double> v;
    const Model *m = t->model;
    for (int p = 0; p < t->nParts; p++) {   // p4_windUpParameters order (Pf/p4_treeOpt.c:19-115)
        const ModelPart &mp = m->parts[p];
        for (int c = 0; c < mp.nComps; c++)
            if (mp.comps[c].free)
                for (int i = 0; i < mp.dim - 1; i++) v.push_back(mp.comps[c].val[i]);
        for (int r = 0; r < mp.nRMatrices; r++)
            if (mp.rMatrices[r].free)
                for (int i = 0; i < mp.dim - 2; i++)
                    for (int j = i + 1; j < mp.dim; j++) v.push_back(mp.rMatrices[r].bigR[(size_t)i * mp.dim + j]);
        for (int g = 0; g < mp.nGdasrvs; g++)
            if (mp.gdasrvs[g]->free) v.push_back(mp.gdasrvs[g]->val[0]);
        if (mp.pInvarFree) v.push_back(mp.pInvar);
    }
    if (m->relRatesAreFree)
        for (int p = 0; p < t->nParts - 1; p++) v.push_back(m->parts[p].relRate);
    *n = (int)v.size();
    if ((int)v.size() > cap) return setError(P4G_EINVAL, "getFreePrams: %d values, room for %d", (int)v.size(), cap);
    for (size_t i = 0; i < v.size(); i++) out[i] = v[i];
    return P4G_OK;
}

extern "C" int p4g_getBrLens(p4g_tree *tt, double *out)
{
    Tree *t = reinterpret_cast<Tree *>(tt);
    if (!t || !out) return setError(P4G_EINVAL, "getBrLens: bad arguments");
    for (int v = 0; v < t->nNodes; v++) out[v] = t->nodes[v] ? t->nodes[v]->brLen : 0.0;
    if (t->root >= 0 && t->root < t->nNodes) out[t->root] = -1.0;   // the reference's placeholder
    return P4G_OK;
}
