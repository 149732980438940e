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
    const double *E = A.eig + (size_t)(A.cNum * A.nR + A.rNum) * (n * n + 2 * n);
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
    if (t->model->nFreePrams != 0)
        return setError(P4G_EUNSUPPORTED,
                        "newtAndBrentPowellOpt: %d free model parameters; only branch lengths are optimised here",
                        t->model->nFreePrams);
    // Pf/p4_treeOpt.c:1207-1212: no free model parameters
    const double eps[4] = {1.0, 1.0e-1, 1.0e-2, 1.0e-5}, delta[4] = {10.0, 1.0, 0.1, 1.0e-7};
    for (int k = 0; k < 4; k++) RET(p4g_newtAround(tt, eps[k], delta[k]));
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
