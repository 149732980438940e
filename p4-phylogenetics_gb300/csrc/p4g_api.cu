// C ABI of libp4gpu: data, model and tree objects with the call shapes of
// p4's CPython extension (Pf/pfmodule.c), plus the host side of setPrams and
// of the fused pruning launch.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <functional>
#include <map>
#include <new>
#include <unordered_map>
#include "p4g_internal.h"
#include "p4g_math.cuh"
#include "p4g_pmat.cuh"
#include "p4g_prune64.cuh"

using namespace p4g;

// ===================================================================== status
namespace p4g {
static thread_local char g_err[1024] = "";

int setError(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int DevBuf::ensure(size_t n)
{
    if (n <= bytes && ptr) return P4G_OK;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return setError(P4G_ENOMEM, "cudaMalloc(%zu): %s", n, cudaGetErrorString(e));
    }
    bytes = n;
    return P4G_OK;
}
void DevBuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}
int PinnedBuf::ensure(size_t n)
{
    if (n <= bytes && ptr) return P4G_OK;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMallocHost(&ptr, n);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return setError(P4G_ENOMEM, "cudaMallocHost(%zu): %s", n, cudaGetErrorString(e));
    }
    bytes = n;
    return P4G_OK;
}
void PinnedBuf::release()
{
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
}

static Ctx g_ctx;
Ctx &ctx() { return g_ctx; }

int ensureCtx()
{
    if (g_ctx.device >= 0) return P4G_OK;
    int dev = 0;
    P4G_CUDA(cudaGetDevice(&dev));
    P4G_CUDA(cudaSetDevice(dev));
    cudaDeviceProp prop;
    P4G_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (!g_ctx.stream) {
        P4G_CUDA(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
        g_ctx.ownStream = true;
    }
    g_ctx.nSM = prop.multiProcessorCount;
    g_ctx.device = dev;
    return P4G_OK;
}

int discreteGammaHost(double alpha, int K, double *rates)
{
    double cut[MAX_CAT];
    if (K > MAX_CAT) return -1;
    return gm_discreteGamma(alpha, K, rates, cut);
}
}  // namespace p4g

#define RET(call)                      \
    do {                               \
        int rc_ = (call);              \
        if (rc_ != P4G_OK) return rc_; \
    } while (0)

static inline Part *P_(p4g_part *p) { return reinterpret_cast<Part *>(p); }
static inline Data *D_(p4g_data *d) { return reinterpret_cast<Data *>(d); }
static inline Model *M_(p4g_model *m) { return reinterpret_cast<Model *>(m); }
static inline Tree *T_(p4g_tree *t) { return reinterpret_cast<Tree *>(t); }
static inline Node *N_(p4g_node *n) { return reinterpret_cast<Node *>(n); }
static inline Gdasrv *G_(p4g_gdasrv *g) { return reinterpret_cast<Gdasrv *>(g); }
namespace p4g {
struct Batch;
}

extern "C" const char *p4g_lastError(void) { return g_err; }

extern "C" const char *p4g_version(void)
{
    return "libp4gpu sm_103a: fused FP32 pruning (dim 2/4/20), FP64 setPrams";
}

extern "C" int p4g_init(int device)
{
    if (g_ctx.device >= 0 && g_ctx.device != device)
        return setError(P4G_ESTATE, "p4g_init: already bound to device %d", g_ctx.device);
    P4G_CUDA(cudaSetDevice(device));
    return ensureCtx();
}

extern "C" int p4g_setStream(void *stream)
{
    RET(ensureCtx());
    if (stream) {
        g_ctx.stream = (cudaStream_t)stream;
    } else {
        P4G_CUDA(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
        g_ctx.ownStream = true;
    }
    return P4G_OK;
}

extern "C" void *p4g_getStream(void)
{
    if (ensureCtx() != P4G_OK) return nullptr;
    return (void *)g_ctx.stream;
}

// ======================================================================= data
extern "C" p4g_data *p4g_newData(int nTax, int nParts)
{
    if (nTax < 1 || nParts < 1) {
        setError(P4G_EINVAL, "newData: nTax=%d nParts=%d", nTax, nParts);
        return nullptr;
    }
    Data *d = new Data;
    d->nTax = nTax;
    d->nParts = nParts;
    d->parts.assign(nParts, nullptr);
    return reinterpret_cast<p4g_data *>(d);
}

extern "C" int p4g_freeData(p4g_data *d)
{
    delete D_(d);
    return P4G_OK;
}

extern "C" int p4g_pokePartInData(p4g_part *p, p4g_data *d, int pNum)
{
    if (!p || !d || pNum < 0 || pNum >= D_(d)->nParts)
        return setError(P4G_EINVAL, "pokePartInData: bad part number %d", pNum);
    D_(d)->parts[pNum] = P_(p);
    return P4G_OK;
}

extern "C" p4g_part *p4g_newPart(int nTax, int nChar, const char *equateSymbols, int nEquates,
                                 const char *symbols, int dim)
{
    if (nTax < 1 || nChar < 1 || dim < 2 || dim > MAX_DIM || nEquates < 0) {
        setError(P4G_EINVAL, "newPart: nTax=%d nChar=%d dim=%d (2..%d) nEquates=%d", nTax, nChar,
                 dim, MAX_DIM, nEquates);
        return nullptr;
    }
    Part *p = new Part;
    p->nTax = nTax;
    p->nChar = nChar;
    p->dim = dim;
    p->nEquates = nEquates;
    p->symbols.assign(symbols, dim);
    p->equateSymbols.assign(equateSymbols ? equateSymbols : "", nEquates);
    p->equates.assign((size_t)nEquates * dim, 0);
    p->sequences.assign((size_t)nTax * nChar, 0);
    return reinterpret_cast<p4g_part *>(p);
}

extern "C" int p4g_freePart(p4g_part *p)
{
    delete P_(p);
    return P4G_OK;
}

// Pf/part.c:279-313: row-major nEquates x dim of '0'/'1'.
extern "C" int p4g_pokeEquatesTable(p4g_part *pp, const char *table)
{
    Part *p = P_(pp);
    if (!p || !table) return setError(P4G_EINVAL, "pokeEquatesTable: null argument");
    size_t n = (size_t)p->nEquates * p->dim;
    if (strlen(table) < n) return setError(P4G_EINVAL, "pokeEquatesTable: table too short");
    for (size_t k = 0; k < n; k++) p->equates[k] = (table[k] == '1') ? 1 : 0;
    p->devValid = false;
    return P4G_OK;
}

// Pf/part.c:127-277: symbols -> 0..dim-1, '-' -> -1, '?' -> -2,
// equate m -> -64+m (N-like equates keep their equate code).
extern "C" int p4g_symbolSequences(p4g_part *pp, char *out)
{
    const Part *p = P_(pp);
    if (!p || !out) return setError(P4G_EINVAL, "symbolSequences: null argument");
    if (p->nChar <= 0 || (long long)p->sequences.size() != (long long)p->nTax * p->nChar)
        return setError(P4G_ESTATE, "symbolSequences: no sequences");
    size_t spot = 0;
    for (int c : p->sequences) {
        char ch;
        if (c >= 0 && c < (int)p->symbols.size()) ch = p->symbols[c];
        else if (c == GAP_CODE) ch = '-';
        else if (c == QMARK_CODE) ch = '?';
        else if (c >= EQUATES_BASE && c < EQUATES_BASE + p->nEquates) ch = p->equateSymbols[c - EQUATES_BASE];
        else return setError(P4G_EINVAL, "symbolSequences: character number %d is not recognized", c);
        out[spot++] = ch;
    }
    out[spot] = '\0';
    return P4G_OK;
}

extern "C" int p4g_pokeSequences(p4g_part *pp, const char *seqs)
{
    Part *p = P_(pp);
    if (!p || !seqs) return setError(P4G_EINVAL, "pokeSequences: null argument");
    int lut[256];
    for (int c = 0; c < 256; c++) lut[c] = 9999;
    for (int m = p->nEquates - 1; m >= 0; m--) lut[(unsigned char)p->equateSymbols[m]] = EQUATES_BASE + m;
    lut[(unsigned char)'?'] = QMARK_CODE;
    lut[(unsigned char)'-'] = GAP_CODE;
    for (int m = p->dim - 1; m >= 0; m--) lut[(unsigned char)p->symbols[m]] = m;
    size_t n = (size_t)p->nTax * p->nChar;
    for (size_t k = 0; k < n; k++) {
        unsigned char ch = (unsigned char)seqs[k];
        if (ch == 0) return setError(P4G_EINVAL, "pokeSequences: string shorter than nTax*nChar");
        int code = lut[ch];
        if (code == 9999)
            return setError(P4G_EINVAL,
                            "pokeSequences: character '%c' is neither a symbol nor an equate", ch);
        p->sequences[k] = code;
    }
    p->patternsMade = p->invarMade = false;
    p->devValid = false;
    return P4G_OK;
}

// Pf/part.c:317-449: unique columns in first-occurrence order, with counts
// and the site -> pattern index.  Hashing gives the same output as the
// reference's linear scan in O(nChar * nTax).
extern "C" int p4g_makePatterns(p4g_part *pp)
{
    Part *p = P_(pp);
    if (!p) return setError(P4G_EINVAL, "makePatterns: null part");
    const int nTax = p->nTax, nChar = p->nChar;
    size_t cap = 1;
    while (cap < (size_t)nChar * 2 + 16) cap <<= 1;
    std::vector<int> slot(cap, -1);
    std::vector<int> first;   // site of first occurrence per pattern
    first.reserve(nChar);
    p->counts.assign(nChar, 0);
    p->seqPosIdx.assign(nChar, 0);
    const int *S = p->sequences.data();
    for (int i = 0; i < nChar; i++) {
        uint64_t h = 1469598103934665603ULL;
        for (int t = 0; t < nTax; t++) h = (h ^ (uint32_t)S[(size_t)t * nChar + i]) * 1099511628211ULL;
        size_t s = (size_t)(h & (cap - 1));
        for (;;) {
            int pidx = slot[s];
            if (pidx < 0) {
                slot[s] = (int)first.size();
                p->seqPosIdx[i] = (int)first.size();
                p->counts[first.size()] = 1;
                first.push_back(i);
                break;
            }
            int f = first[pidx], t = 0;
            for (; t < nTax; t++)
                if (S[(size_t)t * nChar + f] != S[(size_t)t * nChar + i]) break;
            if (t == nTax) {
                p->counts[pidx]++;
                p->seqPosIdx[i] = pidx;
                break;
            }
            s = (s + 1) & (cap - 1);
        }
    }
    const int nPat = (int)first.size();
    p->nPatterns = nPat;
    p->counts.resize(nPat);
    p->patterns.assign((size_t)nTax * nPat, 0);
    for (int t = 0; t < nTax; t++)
        for (int k = 0; k < nPat; k++) p->patterns[(size_t)t * nPat + k] = S[(size_t)t * nChar + first[k]];
    p->patternsMade = true;
    p->invarMade = false;
    p->devValid = false;
    return P4G_OK;
}

extern "C" int p4g_partPatternCount(p4g_part *pp, int *n)
{
    Part *p = P_(pp);
    if (!p || !n) return setError(P4G_EINVAL, "partPatternCount: null argument");
    *n = p->nPatterns;
    return P4G_OK;
}

// Pf/part.c:716-848: a pattern is invariant in state j if every taxon's
// character admits j; vec = number of such states, arr[j][pattern] = 0/1.
extern "C" int p4g_setGlobalInvarSitesVec(p4g_part *pp)
{
    Part *p = P_(pp);
    if (!p || !p->patternsMade) return setError(P4G_ESTATE, "setGlobalInvarSitesVec: no patterns");
    const int nPat = p->nPatterns, dim = p->dim;
    p->invVec.assign(nPat, 0);
    p->invArr.assign((size_t)dim * nPat, 0);
    for (int k = 0; k < nPat; k++) {
        int sum = 0;
        for (int j = 0; j < dim; j++) {
            int all = 1;
            for (int t = 0; t < p->nTax && all; t++) {
                int c = p->patterns[(size_t)t * nPat + k];
                int ok;
                if (c >= 0) ok = (c == j);
                else if (c == N_LIKE || c == GAP_CODE || c == QMARK_CODE) ok = 1;
                else ok = p->equates[(size_t)(c - EQUATES_BASE) * dim + j];
                if (!ok) all = 0;
            }
            p->invArr[(size_t)j * nPat + k] = all;
            sum += all;
        }
        p->invVec[k] = sum;
    }
    p->invarMade = true;
    p->devValid = false;
    return P4G_OK;
}

extern "C" int p4g_getPatterns(p4g_part *pp, int *patterns, int *counts, int *seqPosIdx)
{
    Part *p = P_(pp);
    if (!p || !p->patternsMade) return setError(P4G_ESTATE, "getPatterns: no patterns");
    if (patterns) memcpy(patterns, p->patterns.data(), sizeof(int) * p->patterns.size());
    if (counts) memcpy(counts, p->counts.data(), sizeof(int) * p->nPatterns);
    if (seqPosIdx) memcpy(seqPosIdx, p->seqPosIdx.data(), sizeof(int) * p->nChar);
    return P4G_OK;
}

extern "C" int p4g_getInvarSites(p4g_part *pp, int *vec, int *arr)
{
    Part *p = P_(pp);
    if (!p || !p->invarMade) return setError(P4G_ESTATE, "getInvarSites: not computed");
    if (vec) memcpy(vec, p->invVec.data(), sizeof(int) * p->nPatterns);
    if (arr) memcpy(arr, p->invArr.data(), sizeof(int) * p->invArr.size());
    return P4G_OK;
}

extern "C" int p4g_getSiteLikes(p4g_part *pp, double *out)
{
    Part *p = P_(pp);
    if (!p || p->siteLikes.empty())
        return setError(P4G_ESTATE, "getSiteLikes: no evaluation with getSiteLikes=1 yet");
    memcpy(out, p->siteLikes.data(), sizeof(double) * p->nChar);
    return P4G_OK;
}

// Compact codes for the kernels: 0..dim-1 states, dim = all-ones (gap, ?,
// N-like equates), dim+1+q = partial equate q.
void buildCompact(Part *p)
{
    p->partialOfEquate.assign(p->nEquates, -1);
    p->partialMask.clear();
    for (int e = 0; e < p->nEquates; e++) {
        uint32_t m = 0;
        int all = 1;
        for (int j = 0; j < p->dim; j++) {
            if (p->equates[(size_t)e * p->dim + j]) m |= 1u << j;
            else all = 0;
        }
        if (!all) {
            p->partialOfEquate[e] = (int)p->partialMask.size();
            p->partialMask.push_back(m);
        }
    }
    p->nPartial = (int)p->partialMask.size();
}

int compactCode(const Part *p, int c)
{
    if (c >= 0) return c;
    if (c == GAP_CODE || c == QMARK_CODE || c == N_LIKE) return p->dim;
    int e = c - EQUATES_BASE;
    int q = p->partialOfEquate[e];
    return q < 0 ? p->dim : p->dim + 1 + q;
}

static unsigned long long g_gen = 0;   // source of Part::gen and TreeDev::devGen

int Part::upload(cudaStream_t s)
{
    if (devValid) return P4G_OK;
    gen = ++g_gen;
    if (!patternsMade) return setError(P4G_ESTATE, "part has no patterns (makePatterns not called)");
    if (!invarMade) RET(p4g_setGlobalInvarSitesVec(reinterpret_cast<p4g_part *>(this)));
    buildCompact(this);
    if (dim + 1 + nPartial > 255) return setError(P4G_EUNSUPPORTED, "too many equates for 8-bit codes");
    nPatPad = (nPatterns + 511) / 512 * 512;   // the largest tile is 512 patterns
    std::vector<uint8_t> codes((size_t)nTax * nPatPad, 0);
    for (int t = 0; t < nTax; t++)
        for (int k = 0; k < nPatterns; k++)
            codes[(size_t)t * nPatPad + k] = (uint8_t)compactCode(this, patterns[(size_t)t * nPatterns + k]);
    std::vector<double> cnt(nPatterns);
    std::vector<uint32_t> inv(nPatterns, 0);
    for (int k = 0; k < nPatterns; k++) {
        cnt[k] = (double)counts[k];
        uint32_t m = 0;
        for (int j = 0; j < dim; j++)
            if (invArr[(size_t)j * nPatterns + k]) m |= 1u << j;
        inv[k] = m;
    }
    RET(dCodes.ensure(codes.size()));
    RET(dCounts.ensure(sizeof(double) * nPatterns));
    RET(dInvMask.ensure(sizeof(uint32_t) * nPatterns));
    RET(dEquates.ensure(sizeof(uint32_t) * (nPartial + 1)));
    P4G_CUDA(cudaMemcpyAsync(dCodes.ptr, codes.data(), codes.size(), cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaMemcpyAsync(dCounts.ptr, cnt.data(), sizeof(double) * nPatterns, cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaMemcpyAsync(dInvMask.ptr, inv.data(), sizeof(uint32_t) * nPatterns, cudaMemcpyHostToDevice, s));
    if (nPartial)
        P4G_CUDA(cudaMemcpyAsync(dEquates.ptr, partialMask.data(), sizeof(uint32_t) * nPartial,
                                 cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaStreamSynchronize(s));   // host vectors go out of scope
    devValid = true;
    return P4G_OK;
}

extern "C" int p4g_getCompactCodes(p4g_part *pp, unsigned char *codes, unsigned *partialMasks)
{
    Part *p = P_(pp);
    if (!p || !p->patternsMade) return setError(P4G_ESTATE, "getCompactCodes: no patterns");
    buildCompact(p);
    if (codes)
        for (int t = 0; t < p->nTax; t++)
            for (int k = 0; k < p->nPatterns; k++)
                codes[(size_t)t * p->nPatterns + k] =
                    (unsigned char)compactCode(p, p->patterns[(size_t)t * p->nPatterns + k]);
    if (partialMasks)
        for (int q = 0; q < p->nPartial; q++) partialMasks[q] = p->partialMask[q];
    return P4G_OK;
}

// ====================================================================== model
extern "C" p4g_model *p4g_newModel(int nParts, int doRelRates, int relRatesAreFree, int nFreePrams,
                                   int isHet, int *rMatrixNormalizeTo1, double *PINVAR_MIN,
                                   double *PINVAR_MAX, double *KAPPA_MIN, double *KAPPA_MAX,
                                   double *GAMMA_SHAPE_MIN, double *GAMMA_SHAPE_MAX,
                                   double *PIVEC_MIN, double *PIVEC_MAX, double *RATE_MIN,
                                   double *RATE_MAX, double *RELRATE_MIN, double *RELRATE_MAX,
                                   double *BRLEN_MIN, double *BRLEN_MAX)
{
    if (nParts < 1) {
        setError(P4G_EINVAL, "newModel: nParts=%d", nParts);
        return nullptr;
    }
    Model *m = new Model;
    m->nParts = nParts;
    m->doRelRates = doRelRates;
    m->relRatesAreFree = relRatesAreFree;
    m->nFreePrams = nFreePrams;
    m->isHet = isHet;
    m->rMatrixNormalizeTo1 = rMatrixNormalizeTo1;
    double *b[14] = {PINVAR_MIN, PINVAR_MAX, KAPPA_MIN, KAPPA_MAX, GAMMA_SHAPE_MIN,
                     GAMMA_SHAPE_MAX, PIVEC_MIN, PIVEC_MAX, RATE_MIN, RATE_MAX,
                     RELRATE_MIN, RELRATE_MAX, BRLEN_MIN, BRLEN_MAX};
    for (int i = 0; i < 14; i++) m->bounds[i] = b[i];
    m->parts.resize(nParts);
    return reinterpret_cast<p4g_model *>(m);
}

extern "C" int p4g_freeModel(p4g_model *mm)
{
    Model *m = M_(mm);
    if (!m) return P4G_OK;
    for (auto &mp : m->parts)
        for (auto *g : mp.gdasrvs) delete g;
    delete m;
    return P4G_OK;
}

extern "C" int p4g_newModelPart(p4g_model *mm, int pNum, int dim, int nComps, int nRMatrices,
                                int nGdasrvs, int nCat, int pInvarFree, int *bQETneedsReset)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts) return setError(P4G_EINVAL, "newModelPart: bad pNum");
    if (dim < 2 || dim > MAX_DIM || nComps < 1 || nRMatrices < 1 || nCat < 1 || nCat > MAX_CAT ||
        nGdasrvs < 0 || (nCat > 1 && nGdasrvs < 1))
        return setError(P4G_EINVAL, "newModelPart: dim=%d nComps=%d nR=%d nG=%d nCat=%d", dim,
                        nComps, nRMatrices, nGdasrvs, nCat);
    ModelPart &mp = m->parts[pNum];
    mp.dim = dim;
    mp.nComps = nComps;
    mp.nRMatrices = nRMatrices;
    mp.nGdasrvs = nGdasrvs;
    mp.nCat = nCat;
    mp.pInvarFree = pInvarFree;
    mp.pInvar = 0.0;
    mp.relRate = 1.0;
    mp.comps.assign(nComps, Comp());
    mp.rMatrices.assign(nRMatrices, RMatrix());
    mp.gdasrvs.assign(nGdasrvs, nullptr);
    mp.bQETneedsReset = bQETneedsReset;
    return P4G_OK;
}

extern "C" int p4g_newComp(p4g_model *mm, int pNum, int mNum, int free, double *val)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts || mNum < 0 || mNum >= m->parts[pNum].nComps || !val)
        return setError(P4G_EINVAL, "newComp: bad arguments");
    m->parts[pNum].comps[mNum].free = free;
    m->parts[pNum].comps[mNum].val = val;
    return P4G_OK;
}

// Two-parameter R (Pf/p4_tree.c:286-312, Pf/pfmodule.c:1741-1780):
// transitions kappa/3, transversions 1/3.
static void setTwoP(RMatrix &r, int dim, double kappa)
{
    double a = 1.0 / 3.0, b = a * kappa;
    const double t[16] = {0, a, b, a, a, 0, a, b, b, a, 0, a, a, b, a, 0};
    r.kappa = kappa;
    if (dim == 4)
        for (int i = 0; i < 16; i++) r.bigR[i] = t[i];
}

// The empirical protein exchangeability matrices p4 ships (generated from
// p4's Pf/proteinModels.c by make_protein_models.py).
#include "p4g_protein_models.inc"

// Row of kProteinR for an empirical protein spec (101..120), else -1.
static int proteinModelIndex(int spec)
{
    for (int k = 0; k < (int)(sizeof(kProteinSpecs) / sizeof(kProteinSpecs[0])); k++)
        if (kProteinSpecs[k] == spec) return k;
    return -1;
}

extern "C" int p4g_newRMatrix(p4g_model *mm, int pNum, int mNum, int free, int spec)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts || mNum < 0 || mNum >= m->parts[pNum].nRMatrices)
        return setError(P4G_EINVAL, "newRMatrix: bad arguments");
    ModelPart &mp = m->parts[pNum];
    RMatrix &r = mp.rMatrices[mNum];
    r.free = free;
    r.spec = spec;
    r.bigR.assign((size_t)mp.dim * mp.dim, 1.0);
    const int em = proteinModelIndex(spec);
    if (spec == 5) {
        if (mp.dim != 4) return setError(P4G_EINVAL, "newRMatrix: 2p spec needs dim 4");
        setTwoP(r, 4, 2.0);
    } else if (em >= 0) {   // an empirical protein matrix (Pf/p4_model.c:366-420)
        if (mp.dim != 20)
            return setError(P4G_EINVAL, "newRMatrix: spec %d is a 20-state protein matrix (part dim %d)", spec,
                            mp.dim);
        if (!kProteinSymmetric[em])
            return setError(P4G_EUNSUPPORTED, "newRMatrix: spec %d is not symmetric", spec);
        r.bigR.assign(kProteinR[em], kProteinR[em] + 400);
    }
    // any other spec: all ones, the reference's default (poisson, JC, and
    // specified matrices whose values are poked in later)
    return P4G_OK;
}

extern "C" int p4g_getBigR(int spec, double *out)
{
    const int em = proteinModelIndex(spec);
    if (em < 0 || !out) return setError(P4G_EINVAL, "getBigR: spec %d is not an empirical protein matrix", spec);
    memcpy(out, kProteinR[em], sizeof(double) * 400);
    return P4G_OK;
}

extern "C" p4g_gdasrv *p4g_newGdasrv(p4g_model *mm, int pNum, int mNum, int nCat, int free,
                                     double *val, double *freqs, double *rates)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts || mNum < 0 || mNum >= m->parts[pNum].nGdasrvs ||
        !val || !freqs || !rates || nCat != m->parts[pNum].nCat) {
        setError(P4G_EINVAL, "newGdasrv: bad arguments");
        return nullptr;
    }
    Gdasrv *g = new Gdasrv;
    g->free = free;
    g->nCat = nCat;
    g->val = val;
    g->freqs = freqs;
    g->rates = rates;
    delete m->parts[pNum].gdasrvs[mNum];
    m->parts[pNum].gdasrvs[mNum] = g;
    return reinterpret_cast<p4g_gdasrv *>(g);
}

extern "C" int p4g_gdasrvCalcRates_np(int nCat, double val, double *freqs, double *rates)
{
    if (nCat < 1 || nCat > MAX_CAT || !(val > 0) || !freqs || !rates)
        return setError(P4G_EINVAL, "gdasrvCalcRates: nCat=%d val=%g", nCat, val);
    if (discreteGammaHost(val, nCat, rates))
        return setError(P4G_ENUMERIC, "discrete gamma failed for shape %g", val);
    for (int i = 0; i < nCat; i++) freqs[i] = 1.0 / nCat;
    return P4G_OK;
}

extern "C" int p4g_gdasrvCalcRates(p4g_gdasrv *gg)
{
    Gdasrv *g = G_(gg);
    if (!g) return setError(P4G_EINVAL, "gdasrvCalcRates: null");
    return p4g_gdasrvCalcRates_np(g->nCat, g->val[0], g->freqs, g->rates);
}

extern "C" int p4g_setRMatrixBigR(p4g_model *mm, int pNum, int rNum, int i, int j, double val)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts || rNum < 0 || rNum >= m->parts[pNum].nRMatrices)
        return setError(P4G_EINVAL, "setRMatrixBigR: bad part/matrix");
    ModelPart &mp = m->parts[pNum];
    if (i < 0 || j < 0 || i >= mp.dim || j >= mp.dim)
        return setError(P4G_EINVAL, "setRMatrixBigR: index out of range");
    mp.rMatrices[rNum].bigR[(size_t)i * mp.dim + j] = val;
    mp.rMatrices[rNum].bigR[(size_t)j * mp.dim + i] = val;
    return P4G_OK;
}

extern "C" int p4g_setKappa(p4g_model *mm, int pNum, int rNum, double kappa)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts || rNum < 0 || rNum >= m->parts[pNum].nRMatrices)
        return setError(P4G_EINVAL, "setKappa: bad part/matrix");
    ModelPart &mp = m->parts[pNum];
    if (mp.dim != 4) return setError(P4G_EINVAL, "setKappa: dim must be 4");
    setTwoP(mp.rMatrices[rNum], 4, kappa);
    return P4G_OK;
}

extern "C" int p4g_setPInvarVal(p4g_model *mm, int pNum, double val)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts) return setError(P4G_EINVAL, "setPInvarVal: bad pNum");
    if (!(val >= 0.0 && val < 1.0)) return setError(P4G_EINVAL, "setPInvarVal: %g not in [0,1)", val);
    m->parts[pNum].pInvar = val;
    return P4G_OK;
}

extern "C" int p4g_setRelRateVal(p4g_model *mm, int pNum, double val)
{
    Model *m = M_(mm);
    if (!m || pNum < 0 || pNum >= m->nParts) return setError(P4G_EINVAL, "setRelRateVal: bad pNum");
    if (!(val > 0.0)) return setError(P4G_EINVAL, "setRelRateVal: %g", val);
    m->parts[pNum].relRate = val;
    return P4G_OK;
}

// ======================================================================= tree
extern "C" p4g_tree *p4g_newTree(int nNodes, int nLeaves, int *preOrder, int *postOrder,
                                 int *passLimit, double *partLikes, p4g_data *dd, p4g_model *mm)
{
    Data *d = D_(dd);
    Model *m = M_(mm);
    if (nNodes < 1 || nNodes >= (1 << 14) || !d || !m || !partLikes || d->nParts != m->nParts) {
        setError(P4G_EINVAL, "newTree: nNodes=%d (max %d) or data/model mismatch", nNodes,
                 (1 << 14) - 1);
        return nullptr;
    }
    Tree *t = new Tree;
    t->nNodes = nNodes;
    t->nLeaves = nLeaves;
    t->nParts = d->nParts;
    t->preOrder = preOrder;
    t->postOrder = postOrder;
    t->passLimit = passLimit;
    t->partLikes = partLikes;
    t->data = d;
    t->model = m;
    t->nodes.assign(nNodes, nullptr);
    return reinterpret_cast<p4g_tree *>(t);
}

static void releaseTreeDev(TreeDev &dv)
{
    if (dv.imgFree) cudaEventDestroy(dv.imgFree);
    dv.imgFree = nullptr;
    if (dv.cladeUp) cudaEventDestroy(dv.cladeUp);
    dv.cladeUp = nullptr;
    dv.setPramsGraph.release();
    dv.pruneGraph.release();
}

extern "C" int p4g_freeTree(p4g_tree *tt)
{
    Tree *t = T_(tt);
    if (!t) return P4G_OK;
    if (g_ctx.stream) cudaStreamSynchronize(g_ctx.stream);
    for (Node *n : t->nodes) delete n;
    releaseTreeDev(t->dev);
    delete t;
    return P4G_OK;
}

extern "C" p4g_node *p4g_newNode(int nodeNum, p4g_tree *tt, int seqNum, int isLeaf, int inTree)
{
    Tree *t = T_(tt);
    if (!t || nodeNum < 0 || nodeNum >= t->nNodes) {
        setError(P4G_EINVAL, "newNode: bad node number %d", nodeNum);
        return nullptr;
    }
    if (isLeaf && (seqNum < 0 || seqNum >= t->data->nTax)) {
        setError(P4G_EINVAL, "newNode: leaf %d with seqNum %d (nTax %d)", nodeNum, seqNum,
                 t->data->nTax);
        return nullptr;
    }
    Node *n = new Node;
    n->nodeNum = nodeNum;
    n->tree = t;
    n->seqNum = seqNum;
    n->isLeaf = isLeaf;
    n->inTree = inTree;
    n->compNums.assign(t->nParts, 0);
    n->rMatrixNums.assign(t->nParts, 0);
    n->gdasrvNums.assign(t->nParts, 0);
    delete t->nodes[nodeNum];
    t->nodes[nodeNum] = n;
    t->topoDirty = true;
    t->dev.progDirty = true;
    return reinterpret_cast<p4g_node *>(n);
}

extern "C" int p4g_setNodeRelation(p4g_node *nn, int relation, int relNum)
{
    Node *n = N_(nn);
    if (!n || relNum < -1 || relNum >= n->tree->nNodes)
        return setError(P4G_EINVAL, "setNodeRelation: bad node %d", relNum);
    int *slot = relation == 0 ? &n->parent : relation == 1 ? &n->leftChild
                                          : relation == 2 ? &n->sibling : nullptr;
    if (!slot) return setError(P4G_EINVAL, "setNodeRelation: relation %d out of range", relation);
    if (*slot != relNum) {
        *slot = relNum;
        n->tree->dev.progDirty = true;
    }
    return P4G_OK;
}

extern "C" int p4g_setTreeRoot(p4g_tree *tt, p4g_node *nn)
{
    Tree *t = T_(tt);
    Node *n = N_(nn);
    if (!t || !n || n->tree != t) return setError(P4G_EINVAL, "setTreeRoot: bad node");
    if (t->root != n->nodeNum) {
        t->root = n->nodeNum;
        t->dev.progDirty = true;
    }
    return P4G_OK;
}

extern "C" int p4g_setBrLen(p4g_node *nn, double len)
{
    Node *n = N_(nn);
    if (!n) return setError(P4G_EINVAL, "setBrLen: null node");
    n->brLen = len;
    return P4G_OK;
}

static int setNodeNum(p4g_node *nn, int pNum, int num, int which)
{
    Node *n = N_(nn);
    if (!n || pNum < 0 || pNum >= n->tree->nParts || num < 0)
        return setError(P4G_EINVAL, "set model number: bad arguments");
    (which == 0 ? n->compNums : which == 1 ? n->rMatrixNums : n->gdasrvNums)[pNum] = num;
    return P4G_OK;
}
extern "C" int p4g_setCompNum(p4g_node *n, int pNum, int v) { return setNodeNum(n, pNum, v, 0); }
extern "C" int p4g_setRMatrixNum(p4g_node *n, int pNum, int v) { return setNodeNum(n, pNum, v, 1); }
extern "C" int p4g_setGdasrvNum(p4g_node *n, int pNum, int v) { return setNodeNum(n, pNum, v, 2); }

// ---------------------------------------------------------------- program
// The pruning program: a post-order walk with a small stack of partial
// products.  A non-root node's rescale and its parent-edge transform are one
// op (OP_SCALE_XFORM).
//
// Post-order of the tree from the root, and every node's Sethi-Ullman stack
// need: need(v) = max over v's internal children, in decreasing need order,
// of need(c_i) + (i > 0).
int computeNeed(Tree *t, std::vector<int> &need, std::vector<int> &order)
{
    const int nn = t->nNodes;
    if (t->root < 0 || !t->nodes[t->root]) return setError(P4G_ESTATE, "tree has no root");
    need.assign(nn, 0);
    order.clear();
    order.reserve(nn);
    // iterative post-order over relations from the root
    std::vector<int> stack{t->root};
    std::vector<char> seen(nn, 0);
    while (!stack.empty()) {
        int v = stack.back();
        Node *nv = t->nodes[v];
        if (!nv) return setError(P4G_ESTATE, "node %d referenced but not created", v);
        if (!seen[v]) {
            seen[v] = 1;
            for (int c = nv->leftChild; c >= 0; c = t->nodes[c] ? t->nodes[c]->sibling : -1) {
                if (!t->nodes[c]) return setError(P4G_ESTATE, "node %d referenced but not created", c);
                if (seen[c]) return setError(P4G_ESTATE, "cycle in tree relations at node %d", c);
                stack.push_back(c);
            }
        } else {
            stack.pop_back();
            order.push_back(v);
        }
    }
    for (int v : order) {
        Node *nv = t->nodes[v];
        if (nv->isLeaf && v != t->root) continue;
        if (nv->leftChild < 0) return setError(P4G_ESTATE, "internal node %d has no children", v);
        int best = 0;
        std::vector<int> ns;
        for (int c = nv->leftChild; c >= 0; c = t->nodes[c]->sibling)
            if (!t->nodes[c]->isLeaf) ns.push_back(need[c]);
        std::sort(ns.begin(), ns.end(), std::greater<int>());
        for (size_t i = 0; i < ns.size(); i++) best = std::max(best, ns[i] + (i > 0 ? 1 : 0));
        need[v] = best;
    }
    return P4G_OK;
}

// Program of the subtree rooted at r: internal children first (largest stack
// need first, stable in sibling order), tips after, in sibling order.  At
// the tree's root the program ends with a rescale; for another node r it
// ends with r's rescale + parent-edge transform (the program of a clade
// table).  cherries (nullable): a non-root node whose only children are two
// leaves is preceded by a table lookup (OP_CHERRY + OP_ARG) that replaces its
// TIPSET, TIPMUL, SCALE_XFORM for jobs with a cherry table (the kernels skip
// those three ops; jobs without one skip the lookup), and is listed in
// *cherries as (node, first leaf, second leaf).  cladeOf (nullable): a node
// with cladeOf[v] >= 0 is one OP_CLADE instead of its subtree.  rowOf
// (nullable): the code row of each leaf instead of its sequence number.
int emitProgram(Tree *t, int r, const std::vector<int> &need, std::vector<int> &prog,
                std::vector<int4> *cherries, const std::vector<int> *cladeOf, const std::vector<int> *rowOf)
{
    prog.clear();
    if (cherries) cherries->clear();
    auto cherryOf = [&](int v, int &a, int &b) {
        if (!cherries || v == t->root || t->nodes[v]->isLeaf) return false;
        a = t->nodes[v]->leftChild;
        if (a < 0 || !t->nodes[a]->isLeaf) return false;
        b = t->nodes[a]->sibling;
        return b >= 0 && t->nodes[b]->isLeaf && t->nodes[b]->sibling < 0;
    };
    auto rowOfLeaf = [&](int leaf) { return rowOf ? (*rowOf)[leaf] : t->nodes[leaf]->seqNum; };
    struct Frame {
        int v;
        std::vector<int> kids;
        size_t k;
        int depth;
    };
    std::vector<Frame> fs;
    auto open = [&](int v, int depth) {
        Frame f;
        f.v = v;
        f.k = 0;
        f.depth = depth;
        for (int c = t->nodes[v]->leftChild; c >= 0; c = t->nodes[c]->sibling)
            if (!t->nodes[c]->isLeaf) f.kids.push_back(c);
        std::stable_sort(f.kids.begin(), f.kids.end(), [&](int a, int b) { return need[a] > need[b]; });
        fs.push_back(std::move(f));
    };
    open(r, 0);
    while (!fs.empty()) {
        Frame &f = fs.back();
        if (f.k < f.kids.size()) {
            int c = f.kids[f.k];
            if (f.k > 0) prog.push_back(mkIns(OP_PUSH, f.depth, 0));
            int d = f.depth + (f.k > 0 ? 1 : 0);
            f.k++;
            if (cladeOf && (*cladeOf)[c] >= 0) {   // the whole subtree from its table
                prog.push_back(mkIns(OP_CLADE, (*cladeOf)[c], 0));
                if (f.k > 1) prog.push_back(mkIns(OP_MULSLOT, f.depth, 0));
                continue;
            }
            int la, lb;
            if (cherryOf(c, la, lb)) {   // then the cherry's own ops, for jobs without a table
                prog.push_back(mkIns(OP_CHERRY, (int)cherries->size(), rowOfLeaf(la)));
                prog.push_back(mkIns(OP_ARG, 0, rowOfLeaf(lb)));
                cherries->push_back(make_int4(c, la, lb, 0));
            }
            open(c, d);
            continue;
        }
        // all internal children done (each closed below); tips now
        int v = f.v;
        bool first = f.kids.empty();
        for (int c = t->nodes[v]->leftChild; c >= 0; c = t->nodes[c]->sibling) {
            if (!t->nodes[c]->isLeaf) continue;
            prog.push_back(mkIns(first ? OP_TIPSET : OP_TIPMUL, c, rowOfLeaf(c)));
            first = false;
        }
        fs.pop_back();
        if (fs.empty()) {
            // the tree's root: rescale only; a clade root: rescale + its transform
            prog.push_back(v == t->root ? mkIns(OP_SCALE, 0, 0) : mkIns(OP_SCALE_XFORM, v, 0));
            break;
        }
        // close this child inside its parent: rescale + transform, then combine
        Frame &par = fs.back();
        prog.push_back(mkIns(OP_SCALE_XFORM, v, 0));
        if (par.k > 1) prog.push_back(mkIns(OP_MULSLOT, par.depth, 0));
    }
    return P4G_OK;
}

// The whole tree's program (see emitProgram) and its stack slot count.
int buildProgram(Tree *t, std::vector<int> &prog, int &nSlots, std::vector<int4> *cherries)
{
    std::vector<int> need, order;
    RET(computeNeed(t, need, order));
    nSlots = need[t->root];
    RET(emitProgram(t, t->root, need, prog, cherries, nullptr, nullptr));
    if ((int)prog.size() > t->dev.progCap && t->dev.progCap > 0)
        return setError(P4G_ESTATE, "program longer than its buffer");
    return P4G_OK;
}

// ---------------------------------------------------------------- device state
static inline size_t alignUp(size_t x, size_t a) { return (x + a - 1) / a * a; }

int defaultShape(int dim) { return dim == 4 ? 3 : 0; }

// Tile list of every pruning group for its current shape, written into the
// image's block region, with each job's tile count.
static int layoutBlocks(Tree *t)
{
    TreeDev &dv = t->dev;
    Model *m = t->model;
    Data *d = t->data;
    dv.blocks.clear();
    PruneJob *jobs = (PruneJob *)((char *)dv.hImg.ptr + dv.oJobs);
    for (auto &g : dv.groups) {
        g.blk0 = (int)dv.blocks.size();
        const int tile = pruneTile(g.dim, g.shape);
        for (int p = 0; p < t->nParts; p++) {
            if (m->parts[p].dim != g.dim || m->parts[p].nCat != g.nCat) continue;
            const int nb = (d->parts[p]->nPatterns + tile - 1) / tile;
            for (int b = 0; b < nb; b++) dv.blocks.push_back(BlockDesc{p, b * tile, b, 0});
            jobs[p].nBlocks = nb;
        }
        g.nBlk = (int)dv.blocks.size() - g.blk0;
    }
    if ((int)dv.blocks.size() > dv.blockCap) return setError(P4G_ESTATE, "block list overflow");
    memcpy((char *)dv.hImg.ptr + dv.oBlocks, dv.blocks.data(), sizeof(BlockDesc) * dv.blocks.size());
    return P4G_OK;
}

// The setPrams status int, right after the part lnLs in dOut.
static int *treeStatus(Tree *t)
{
    return (int *)((char *)t->dev.dOut.ptr + sizeof(double) * t->nParts);
}

static int allocTreeDev(Tree *t)
{
    TreeDev &dv = t->dev;
    if (dv.allocated) return P4G_OK;
    RET(ensureCtx());
    dv.devGen = ++g_gen;
    Model *m = t->model;
    Data *d = t->data;
    const int nP = t->nParts, nn = t->nNodes;
    for (int p = 0; p < nP; p++) {
        if (!d->parts[p]) return setError(P4G_ESTATE, "data part %d missing", p);
        if (m->parts[p].dim != d->parts[p]->dim)
            return setError(P4G_EINVAL, "part %d: model dim %d != data dim %d", p, m->parts[p].dim,
                            d->parts[p]->dim);
        if (d->parts[p]->nTax != d->nTax) return setError(P4G_EINVAL, "part %d: nTax mismatch", p);
        RET(d->parts[p]->upload(g_ctx.stream));
    }
    // image layout
    size_t o = 0;
    dv.oPmat = o;
    o = alignUp(o + sizeof(PmatPart) * nP, 256);
    dv.oJobs = o;
    o = alignUp(o + sizeof(PruneJob) * nP, 256);
    dv.oPrefix = o;
    o = alignUp(o + sizeof(int) * nP, 256);
    {
        size_t nPairs = 0, nGd = 0;
        for (int p = 0; p < nP; p++) {
            nPairs += (size_t)m->parts[p].nComps * m->parts[p].nRMatrices;
            nGd += m->parts[p].nGdasrvs;
        }
        dv.oEigTasks = o;
        o = alignUp(o + sizeof(int2) * std::max<size_t>(nPairs, 1), 256);
        dv.oGammaTasks = o;
        o = alignUp(o + sizeof(int2) * std::max<size_t>(nGd, 1), 256);
    }
    dv.oComps.resize(nP);
    dv.oR.resize(nP);
    dv.oG.resize(nP);
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        dv.oComps[p] = o;
        o = alignUp(o + sizeof(double) * mp.nComps * mp.dim, 16);
        dv.oR[p] = o;
        o = alignUp(o + sizeof(double) * mp.nRMatrices * mp.dim * mp.dim, 16);
        dv.oG[p] = o;
        o = alignUp(o + sizeof(double) * std::max(mp.nGdasrvs, 1), 16);
    }
    dv.oBrLen = o;
    o = alignUp(o + sizeof(double) * nn, 16);
    dv.oNodeIdx = o;
    o = alignUp(o + sizeof(int) * nn * nP * 3, 16);
    dv.oIsLeaf = o;
    o = alignUp(o + sizeof(int) * nn, 16);
    dv.progCap = 4 * nn + 16;
    dv.oProg = o;
    o = alignUp(o + sizeof(int) * dv.progCap, 16);
    dv.capCherry = t->nLeaves / 2 + 1;
    dv.oCherries = o;
    o = alignUp(o + sizeof(int4) * dv.capCherry, 16);
    dv.oMaps = o;
    o = alignUp(o + sizeof(int) * 2 * (nn + d->nTax), 16);
    // pruning groups by (dim, nCat); blocks are laid out by layoutBlocks()
    dv.groups.clear();
    std::vector<std::pair<int, int>> keys;
    for (int p = 0; p < nP; p++) {
        std::pair<int, int> k(m->parts[p].dim, m->parts[p].nCat);
        if (std::find(keys.begin(), keys.end(), k) == keys.end()) keys.push_back(k);
    }
    for (auto &k : keys) dv.groups.push_back(PruneGroup{k.first, k.second, 0, 0, 0, defaultShape(k.first)});
    dv.oPartials.assign(nP, 0);
    size_t nPartials = 0;
    dv.blockCap = 0;
    for (int p = 0; p < nP; p++) {
        const int nb = (d->parts[p]->nPatterns + 63) / 64;   // every tile holds at least 64 patterns
        dv.oPartials[p] = nPartials;
        nPartials += nb;
        dv.blockCap += nb;
    }
    dv.oBlocks = o;
    o = alignUp(o + sizeof(BlockDesc) * dv.blockCap, 256);
    dv.imgBytes = o;
    RET(dv.hImg.ensure(dv.imgBytes));
    RET(dv.dImg.ensure(dv.imgBytes));
    memset(dv.hImg.ptr, 0, dv.imgBytes);
    dv.shadow.clear();
    {   // the pinned image's address on the device (mapped pinned memory)
        void *dp = nullptr;
        if (cudaHostGetDevicePointer(&dp, dv.hImg.ptr, 0) == cudaSuccess) {
            dv.hImgDev = dp;
        } else {
            (void)cudaGetLastError();
            dv.hImgDev = nullptr;
        }
    }
    // derived buffers
    size_t nRates = 0, nEig = 0, nDeck = 0, nEq = 0, nTc = 0;
    dv.oRates.resize(nP);
    dv.oEig.resize(nP);
    dv.oDecks.resize(nP);
    dv.oEqTab.resize(nP);
    dv.oTcB.assign(nP, (size_t)-1);
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        const int dim = mp.dim;
        dv.oRates[p] = nRates;
        nRates += (size_t)std::max(mp.nGdasrvs, 1) * mp.nCat;
        dv.oEig[p] = nEig;
        nEig += (size_t)mp.nComps * mp.nRMatrices * eigRecDoubles(dim);
        dv.oDecks[p] = nDeck;
        nDeck += alignUp((size_t)nn * mp.nCat * dim * dim, 4);
        dv.oEqTab[p] = nEq;
        nEq += alignUp((size_t)nn * std::max(d->parts[p]->nPartial, 1) * mp.nCat * dim, 4);   // 16-byte rows
        if (dim == 20 && mp.nCat == 4) {   // parts the tensor-core kernel can take
            dv.oTcB[p] = nTc;
            nTc += (size_t)nn * mp.nCat * 1536;
        }
    }
    RET(dv.dRates.ensure(sizeof(double) * nRates));
    RET(dv.dEig.ensure(sizeof(double) * nEig));
    RET(dv.dDecks32.ensure(sizeof(float) * nDeck));
    RET(dv.dDecks64.ensure(sizeof(double) * nDeck));
    RET(dv.dEqTab.ensure(sizeof(float) * nEq));
    RET(dv.dPartials.ensure(sizeof(double) * std::max<size_t>(nPartials, 1)));
    // part lnLs, then the setPrams status int: one device->host copy per evaluation
    RET(dv.dOut.ensure(sizeof(double) * nP + 16));
    RET(dv.dTicket.ensure(sizeof(int) * nP));
    RET(dv.dBad.ensure(sizeof(int) * nP));
    {   // cherry tables: capCherry x K x K x nCat x dim floats per part
        size_t nCh = 0;
        dv.oCherryTab.resize(nP);
        for (int p = 0; p < nP; p++) {
            const int K = m->parts[p].dim + 1 + d->parts[p]->nPartial;
            dv.oCherryTab[p] = (size_t)-1;
            if (m->parts[p].dim < 20) continue;   // measured: pays for 20 states, not for 4
            // a table of K x K code pairs is built every evaluation: it pays only
            // when the part has clearly more patterns than code pairs
            if (d->parts[p]->nPatterns < 2 * K * K) continue;
            dv.oCherryTab[p] = nCh;
            nCh += alignUp((size_t)dv.capCherry * K * K * m->parts[p].nCat * m->parts[p].dim, 4);
        }
        if (nCh) RET(dv.dCherryTab.ensure(sizeof(float) * nCh));
    }
    if (nTc) {
        RET(dv.dTcB.ensure(sizeof(float) * nTc));
        P4G_CUDA(cudaMemsetAsync(dv.dTcB.ptr, 0, dv.dTcB.bytes, g_ctx.stream));   // padding stays zero
    }
    P4G_CUDA(cudaMemsetAsync(dv.dDecks32.ptr, 0, dv.dDecks32.bytes, g_ctx.stream));
    P4G_CUDA(cudaMemsetAsync(dv.dDecks64.ptr, 0, dv.dDecks64.bytes, g_ctx.stream));
    P4G_CUDA(cudaMemsetAsync(dv.dEqTab.ptr, 0, dv.dEqTab.bytes, g_ctx.stream));
    P4G_CUDA(cudaMemsetAsync(dv.dTicket.ptr, 0, sizeof(int) * nP, g_ctx.stream));
    P4G_CUDA(cudaMemsetAsync(dv.dBad.ptr, 0, sizeof(int) * nP, g_ctx.stream));
    P4G_CUDA(cudaMemsetAsync(treeStatus(t), 0, sizeof(int), g_ctx.stream));
    RET(dv.hOut.ensure(sizeof(double) * nP + 16));
    P4G_CUDA(cudaEventCreateWithFlags(&dv.imgFree, cudaEventDisableTiming));
    // static parts of the jobs
    char *base = (char *)dv.dImg.ptr;
    PruneJob *jobs = (PruneJob *)((char *)dv.hImg.ptr + dv.oJobs);
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        Part *dp = d->parts[p];
        PruneJob &J = jobs[p];
        J.decks = dv.dDecks32.as<float>() + dv.oDecks[p];
        J.eqTab = dv.dEqTab.as<float>() + dv.oEqTab[p];
        J.codes = dp->dCodes.as<uint8_t>();
        J.counts = dp->dCounts.as<double>();
        J.invMask = dp->dInvMask.as<uint32_t>();
        J.partialMask = dp->dEquates.as<uint32_t>();
        J.tcB = dv.oTcB[p] == (size_t)-1 ? nullptr : dv.dTcB.as<float>() + dv.oTcB[p];
        J.cherryTab = dv.oCherryTab[p] == (size_t)-1 ? nullptr : dv.dCherryTab.as<float>() + dv.oCherryTab[p];
        J.cherries = (const int4 *)(base + dv.oCherries);
        J.prog = (const int *)(base + dv.oProg);
        J.partials = dv.dPartials.as<double>() + dv.oPartials[p];
        J.out = dv.dOut.as<double>() + p;
        J.ticket = dv.dTicket.as<int>() + p;
        J.badFlag = dv.dBad.as<int>() + p;
        J.nPat = dp->nPatterns;
        J.nPatPad = dp->nPatPad;
        J.nPartial = dp->nPartial;
        J.nNodes = nn;
        J.nTax = d->nTax;
        J.dim = mp.dim;
        J.nCat = mp.nCat;
        J.deckMap = nullptr;
        J.rowMap = nullptr;
        J.nDeck = nn;
        J.nRow = d->nTax;
    }
    dv.nDeck = nn;
    dv.nRow = d->nTax;
    dv.allocated = true;
    dv.progDirty = true;
    RET(layoutBlocks(t));
    return P4G_OK;
}

// Model-value checks the reference enforces with exit(1) (Pf/p4_tree.c:424-452).
int validateModel(Tree *t, int pNum)
{
    Model *m = t->model;
    const double pivMin = m->PIVEC_MIN();
    for (int p = 0; p < t->nParts; p++) {
        if (pNum >= 0 && p != pNum) continue;
        const ModelPart &mp = m->parts[p];
        if (mp.dim == 0) return setError(P4G_ESTATE, "model part %d not created", p);
        for (int c = 0; c < mp.nComps; c++) {
            const double *v = mp.comps[c].val;
            if (!v) return setError(P4G_ESTATE, "part %d comp %d has no values", p, c);
            double sum = 0.0;
            for (int j = 0; j < mp.dim; j++) {
                if (!(v[j] >= pivMin))
                    return setError(P4G_EINVAL, "part %d, comp %d, value %d is %g (< PIVEC_MIN %g)", p,
                                    c, j, v[j], pivMin);
                sum += v[j];
            }
            if (fabs(sum - 1.0) > 1e-14)
                return setError(P4G_EINVAL, "part %d, comp %d values do not sum to 1 (sum-1 = %g)", p,
                                c, sum - 1.0);
        }
        for (int g = 0; g < mp.nGdasrvs; g++)
            if (!mp.gdasrvs[g] || !(mp.gdasrvs[g]->val[0] > 0))
                return setError(P4G_EINVAL, "part %d gdasrv %d has no positive shape", p, g);
        for (int r = 0; r < mp.nRMatrices; r++)
            for (int i = 0; i < mp.dim; i++)
                for (int j = i + 1; j < mp.dim; j++)
                    if (!(mp.rMatrices[r].bigR[(size_t)i * mp.dim + j] >= 0))   // empirical matrices hold zeros
                        return setError(P4G_EINVAL, "part %d rMatrix %d entry (%d,%d) negative or not a number",
                                        p, r, i, j);
    }
    for (int v = 0; v < t->nNodes; v++) {
        Node *n = t->nodes[v];
        if (!n) continue;
        for (int p = 0; p < t->nParts; p++) {
            const ModelPart &mp = m->parts[p];
            if (n->compNums[p] >= mp.nComps || n->rMatrixNums[p] >= mp.nRMatrices ||
                (mp.nGdasrvs && n->gdasrvNums[p] >= mp.nGdasrvs))
                return setError(P4G_EINVAL, "node %d part %d: model component number out of range", v, p);
        }
        if (n->inTree && v != t->root && !(n->brLen >= 0.0 && n->brLen < 1e300))
            return setError(P4G_EINVAL, "node %d: branch length %g", v, n->brLen);
    }
    return P4G_OK;
}

// Fill the program region and the topology-dependent job fields.
static int refreshProgram(Tree *t)
{
    TreeDev &dv = t->dev;
    if (!dv.progDirty) return P4G_OK;
    {
        std::vector<int> need, order;
        RET(computeNeed(t, need, order));
        dv.nSlots = need[t->root];
        const int nC = cladeSelect(t, order, dv.cladeOf);
        // cherry lookups only without clade tables (every cherry is inside a
        // clade then) and only when some part has a cherry table
        bool anyTable = false;
        for (size_t p = 0; p < dv.oCherryTab.size(); p++) anyTable |= dv.oCherryTab[p] != (size_t)-1;
        const bool cherries = anyTable && nC == 0;
        RET(emitProgram(t, t->root, need, dv.prog, cherries ? &dv.cherryList : nullptr,
                        nC ? &dv.cladeOf : nullptr, nullptr));
        if (!cherries) dv.cherryList.clear();
        if (nC) {
            // number the clades in the order the program reads them, so that
            // a kernel knows which tables come next (clade k is the k-th OP_CLADE)
            std::vector<int> rank(nC, -1);
            int k = 0;
            for (int &ins : dv.prog) {
                if ((ins & 15) != OP_CLADE) continue;
                const int c = (ins >> 4) & 0x3fff;
                rank[c] = k++;
                ins = mkIns(OP_CLADE, rank[c], 0);
            }
            if (k != nC) return setError(P4G_ESTATE, "clade program: %d of %d clades read", k, nC);
            for (int &c : dv.cladeOf)
                if (c >= 0) c = rank[c];
        }
        RET(cladeBuild(t, need, dv.cladeOf));
    }
    dv.table64Dirty = true;
    if ((int)dv.prog.size() > dv.progCap) return setError(P4G_ESTATE, "program too long");
    if ((int)dv.cherryList.size() > dv.capCherry) return setError(P4G_ESTATE, "cherry list too long");
    dv.nProg = (int)dv.prog.size();
    memcpy((char *)dv.hImg.ptr + dv.oProg, dv.prog.data(), sizeof(int) * dv.nProg);
    memcpy((char *)dv.hImg.ptr + dv.oCherries, dv.cherryList.data(), sizeof(int4) * dv.cherryList.size());
    PruneJob *jobs = (PruneJob *)((char *)dv.hImg.ptr + dv.oJobs);
    Node *rootNode = t->nodes[t->root];
    // With clade tables most leaves and edges sit inside the clades: a tile
    // of the whole-tree program stages only the decks and code rows its ops read
    const int nTax = t->data->nTax;
    dv.nDeck = t->nNodes;
    dv.nRow = nTax;
    const bool maps = dv.nClade > 0;
    if (maps) {
        const int nn = t->nNodes;
        int *deckOf = (int *)((char *)dv.hImg.ptr + dv.oMaps), *deckNode = deckOf + nn;
        int *rowOf = deckNode + nn, *rowTax = rowOf + nTax;
        std::fill(deckOf, deckOf + 2 * (nn + nTax), 0);
        std::vector<char> seenD(nn, 0), seenR(nTax, 0);
        int nd = 0, nr = 0;
        auto useRow = [&](int b) {
            if (!seenR[b]) {
                seenR[b] = 1;
                rowOf[b] = nr;
                rowTax[nr++] = b;
            }
        };
        for (size_t i = 0; i < dv.prog.size(); i++) {
            const int ins = dv.prog[i], op = ins & 15, a = (ins >> 4) & 0x3fff, b = ins >> 18;
            if (op == OP_TIPSET || op == OP_TIPMUL || op == OP_XFORM || op == OP_SCALE_XFORM) {
                if (a >= nn) return setError(P4G_ESTATE, "program deck %d out of range", a);
                if (!seenD[a]) {
                    seenD[a] = 1;
                    deckOf[a] = nd;
                    deckNode[nd++] = a;
                }
            }
            if (op == OP_TIPSET || op == OP_TIPMUL) {
                if (b >= nTax) return setError(P4G_ESTATE, "program code row %d out of range", b);
                useRow(b);
            }
            if (op == OP_CHERRY) {
                if (i + 1 >= dv.prog.size() || b >= nTax || (dv.prog[i + 1] >> 18) >= nTax)
                    return setError(P4G_ESTATE, "program cherry rows out of range");
                useRow(b);
                useRow(dv.prog[i + 1] >> 18);
            }
        }
        if (rootNode->isLeaf) useRow(rootNode->seqNum);
        dv.nDeck = nd;
        dv.nRow = nr;
    }
    const char *dBase = (const char *)dv.dImg.ptr;
    dv.cherryWork = 0;
    for (int p = 0; p < t->nParts; p++) {
        jobs[p].deckMap = maps ? (const int *)(dBase + dv.oMaps) : nullptr;
        jobs[p].rowMap = maps ? (const int *)(dBase + dv.oMaps) + 2 * t->nNodes : nullptr;
        jobs[p].nDeck = dv.nDeck;
        jobs[p].nRow = dv.nRow;
        jobs[p].nProg = dv.nProg;
        jobs[p].nSlots = dv.nSlots;
        jobs[p].rootLeafRow = rootNode->isLeaf ? rootNode->seqNum : -1;
        jobs[p].nCherry = (int)dv.cherryList.size();
        jobs[p].nClade = dv.nClade;
        if (jobs[p].cherryTab)
            dv.cherryWork = std::max(dv.cherryWork, (long long)dv.cherryList.size() * jobs[p].nCat);
    }
    for (auto &g : dv.groups) {
        g.smem = pruneSmemBytes(g.dim, g.nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, g.shape,
                                dv.nClade, dv.nDeck, dv.nRow);
        if (g.smem > 227 * 1024) {   // a large tree: the tile shape with the smallest footprint
            int best = -1, bestSmem = 0;
            for (int sh = 0; sh < pruneNumShapes(g.dim); sh++) {
                if (!pruneShapeValid(g.dim, g.nCat, sh)) continue;
                const int sm = pruneSmemBytes(g.dim, g.nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, sh,
                                              dv.nClade, dv.nDeck, dv.nRow);
                if (sm <= 227 * 1024 && (best < 0 || sm < bestSmem)) {
                    best = sh;
                    bestSmem = sm;
                }
            }
            if (best < 0)
                return setError(P4G_EUNSUPPORTED,
                                "tree too large for the fused kernel's shared memory (%d bytes)", g.smem);
            g.shape = best;
            g.smem = bestSmem;
        }
    }
    dv.progDirty = false;
    return P4G_OK;
}

// Write parameter values and setPrams descriptors into the pinned image.
static bool sameVals(const std::vector<double> &cache, const double *v, size_t n)
{
    return cache.size() == n && memcmp(cache.data(), v, sizeof(double) * n) == 0;
}

static int packParams(Tree *t, int pNum, int &nDesc, int &nG, int &nE, int &nD, int &maxDim)
{
    TreeDev &dv = t->dev;
    Model *m = t->model;
    Data *d = t->data;
    char *h = (char *)dv.hImg.ptr;
    char *g = (char *)dv.dImg.ptr;
    const int nP = t->nParts, nn = t->nNodes;
    double *brLen = (double *)(h + dv.oBrLen);
    int *nodeIdx = (int *)(h + dv.oNodeIdx);
    int *isLeaf = (int *)(h + dv.oIsLeaf);
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
    PmatPart *desc = (PmatPart *)(h + dv.oPmat);
    PruneJob *jobs = (PruneJob *)(h + dv.oJobs);
    int *prefix = (int *)(h + dv.oPrefix);
    int2 *eigTasks = (int2 *)(h + dv.oEigTasks);
    int2 *gammaTasks = (int2 *)(h + dv.oGammaTasks);
    if (!dv.cacheValid) {
        dv.cComps.assign(nP, {});
        dv.cR.assign(nP, {});
        dv.cG.assign(nP, {});
    }
    nDesc = nG = nE = nD = 0;
    maxDim = 0;
    for (int p = 0; p < nP; p++) {
        const ModelPart &mp = m->parts[p];
        const int dim = mp.dim;
        double *comps = (double *)(h + dv.oComps[p]);
        for (int c = 0; c < mp.nComps; c++) memcpy(comps + c * dim, mp.comps[c].val, sizeof(double) * dim);
        double *R = (double *)(h + dv.oR[p]);
        for (int r = 0; r < mp.nRMatrices; r++)
            memcpy(R + (size_t)r * dim * dim, mp.rMatrices[r].bigR.data(), sizeof(double) * dim * dim);
        double *gv = (double *)(h + dv.oG[p]);
        for (int k = 0; k < mp.nGdasrvs; k++) gv[k] = mp.gdasrvs[k]->val[0];
        // pruning job parameters
        PruneJob &J = jobs[p];
        J.rootComp = (const double *)(g + dv.oComps[p]) + (size_t)t->nodes[t->root]->compNums[p] * dim;
        J.pInvar = mp.pInvar;
        J.varScale = (1.0 - mp.pInvar) / (double)mp.nCat;
        J.logScale = (mp.pInvar != 0.0) ? log(J.varScale) : (mp.nCat > 1 ? log(1.0 / mp.nCat) : 0.0);
        if (pNum >= 0 && p != pNum) continue;
        PmatPart &P = desc[nDesc];
        P.comps = (const double *)(g + dv.oComps[p]);
        P.R = (const double *)(g + dv.oR[p]);
        P.gval = (const double *)(g + dv.oG[p]);
        P.brLen = dv.hImgDev ? (const double *)((const char *)dv.hImgDev + dv.oBrLen)
                             : (const double *)(g + dv.oBrLen);
        P.nodeIdx = (const int *)(g + dv.oNodeIdx);
        P.isLeaf = (const int *)(g + dv.oIsLeaf);
        P.rates = dv.dRates.as<double>() + dv.oRates[p];
        P.eig = dv.dEig.as<double>() + dv.oEig[p];
        P.decks32 = dv.dDecks32.as<float>() + dv.oDecks[p];
        P.eqTab = dv.dEqTab.as<float>() + dv.oEqTab[p];
        P.decks64 = dv.dDecks64.as<double>() + dv.oDecks[p];
        P.tcB = dv.oTcB[p] == (size_t)-1 ? nullptr : dv.dTcB.as<float>() + dv.oTcB[p];
        P.partialMask = d->parts[p]->dEquates.as<uint32_t>();
        P.pInvar = mp.pInvar;
        P.relRate = mp.relRate;
        P.dim = dim;
        P.nCat = mp.nCat;
        P.nComps = mp.nComps;
        P.nR = mp.nRMatrices;
        P.nG = mp.nGdasrvs;
        P.nNodes = nn;
        P.root = t->root;
        P.nPartial = d->parts[p]->nPartial;
        P.partIdx = p;
        P.nParts = nP;
        // only the eigensystems / gamma rates whose inputs changed
        const size_t nc = (size_t)mp.nComps * dim, nr = (size_t)mp.nRMatrices * dim * dim;
        std::vector<char> compCh(mp.nComps, 1), rCh(mp.nRMatrices, 1);
        if (dv.cComps[p].size() == nc)
            for (int c = 0; c < mp.nComps; c++)
                compCh[c] = memcmp(dv.cComps[p].data() + (size_t)c * dim, comps + (size_t)c * dim,
                                   sizeof(double) * dim) != 0;
        if (dv.cR[p].size() == nr)
            for (int r = 0; r < mp.nRMatrices; r++)
                rCh[r] = memcmp(dv.cR[p].data() + (size_t)r * dim * dim, R + (size_t)r * dim * dim,
                                sizeof(double) * dim * dim) != 0;
        for (int c = 0; c < mp.nComps; c++)
            for (int r = 0; r < mp.nRMatrices; r++)
                if (compCh[c] || rCh[r]) eigTasks[nE++] = make_int2(nDesc, c * mp.nRMatrices + r);
        for (int k = 0; k < mp.nGdasrvs; k++)
            if (dv.cG[p].size() != (size_t)mp.nGdasrvs || dv.cG[p][k] != gv[k])
                gammaTasks[nG++] = make_int2(nDesc, k);
        dv.cComps[p].assign(comps, comps + nc);
        dv.cR[p].assign(R, R + nr);
        dv.cG[p].assign(gv, gv + mp.nGdasrvs);
        prefix[nDesc] = nD;
        nD += pdeckTasks(dim, nn, mp.nCat);
        maxDim = std::max(maxDim, dim);
        nDesc++;
    }
    dv.cacheValid = true;
    return P4G_OK;
}

static int uploadImage(Tree *t)
{
    TreeDev &dv = t->dev;
    P4G_CUDA(cudaMemcpyAsync(dv.dImg.ptr, dv.hImg.ptr, dv.imgBytes, cudaMemcpyHostToDevice, g_ctx.stream));
    P4G_CUDA(cudaEventRecord(dv.imgFree, g_ctx.stream));
    dv.shadow.assign((const char *)dv.hImg.ptr, (const char *)dv.hImg.ptr + dv.imgBytes);
    dv.cladeFresh = false;
    return P4G_OK;
}

// Whether the host image differs from the device copy anywhere but in the
// branch lengths (which the P-deck kernel reads from host memory).
static bool imageDirty(const Tree *t)
{
    const TreeDev &dv = t->dev;
    if (!dv.hImgDev || dv.shadow.size() != dv.imgBytes) return true;
    const char *h = (const char *)dv.hImg.ptr, *sh = dv.shadow.data();
    const size_t b0 = dv.oBrLen, b1 = dv.oBrLen + sizeof(double) * t->nNodes;
    return memcmp(h, sh, b0) != 0 || memcmp(h + b1, sh + b1, dv.imgBytes - b1) != 0;
}

static int waitImage(Tree *t)
{
    if (t->dev.imgFree) P4G_CUDA(cudaEventSynchronize(t->dev.imgFree));
    return P4G_OK;
}

// Enqueue setPrams for a tree (no synchronisation).
// A launch sequence replayed from a CUDA graph while its signature (every
// value the sequence's launches depend on) is unchanged; otherwise it runs
// once plainly (launch attributes, occupancy queries), then is captured.
int GraphSlot::run(const std::vector<long long> &s, cudaStream_t st, const std::function<int()> &enqueue)
{
    clock++;
    Entry *victim = &e[0];
    for (auto &x : e) {
        if (x.exec && x.sig == s) {
            x.used = clock;
            P4G_CUDA(cudaGraphLaunch(x.exec, st));
            return P4G_OK;
        }
        if (!x.exec) victim = &x;   // an empty way first, else the least recently used
        else if (victim->exec && x.used < victim->used) victim = &x;
    }
    if (victim->exec) cudaGraphExecDestroy(victim->exec);
    if (victim->graph) cudaGraphDestroy(victim->graph);
    *victim = Entry();
    RET(enqueue());
    P4G_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue();
    cudaGraph_t g = nullptr;
    cudaError_t err = cudaStreamEndCapture(st, &g);
    if (rc != P4G_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (err != cudaSuccess) return setError(P4G_ECUDA, "graph capture: %s", cudaGetErrorString(err));
    victim->graph = g;
    P4G_CUDA(cudaGraphInstantiate(&victim->exec, g, 0));
    victim->sig = s;
    victim->used = clock;
    return P4G_OK;
}

void GraphSlot::release()
{
    for (auto &x : e) {
        if (x.exec) cudaGraphExecDestroy(x.exec);
        if (x.graph) cudaGraphDestroy(x.graph);
        x = Entry();
    }
}

static int enqueueSetPrams(Tree *t, int pNum)
{
    RET(validateModel(t, pNum));
    RET(allocTreeDev(t));
    RET(waitImage(t));
    RET(refreshProgram(t));
    int nDesc, nG, nE, nD, maxDim;
    RET(packParams(t, pNum, nDesc, nG, nE, nD, maxDim));
    TreeDev &dv = t->dev;
    const char *g = (const char *)dv.dImg.ptr;
    const PmatPart *dDesc = (const PmatPart *)(g + dv.oPmat);
    const int *pre = (const int *)(g + dv.oPrefix);
    // the image copy is left out when only branch lengths changed since the
    // last one (the P-deck kernel reads those from the pinned host image)
    const bool upload = imageDirty(t);
    if (upload) dv.shadow.assign((const char *)dv.hImg.ptr, (const char *)dv.hImg.ptr + dv.imgBytes);
    auto enqueue = [&]() -> int {
        if (upload)
            P4G_CUDA(cudaMemcpyAsync(dv.dImg.ptr, dv.hImg.ptr, dv.imgBytes, cudaMemcpyHostToDevice, g_ctx.stream));
        return launchPmat(dDesc, (const int2 *)(g + dv.oEigTasks), nE, (const int2 *)(g + dv.oGammaTasks), nG,
                          pre, nDesc, nD, maxDim, treeStatus(t), g_ctx.stream);
    };
    if (dv.useGraphs && dv.tuned) {
        const std::vector<long long> sig = {nDesc, nG, nE, nD, maxDim, (long long)(size_t)dv.dImg.ptr,
                                            (long long)dv.imgBytes, (long long)(size_t)dv.hImg.ptr, upload};
        RET(dv.setPramsGraph.run(sig, g_ctx.stream, enqueue));
    } else {
        RET(enqueue());
    }
    if (upload || nD > 0) dv.cladeFresh = false;
    // the image may be rewritten once its copy is done (recorded outside any
    // capture; after the setPrams kernels, which is later than needed)
    P4G_CUDA(cudaEventRecord(dv.imgFree, g_ctx.stream));
    dv.lastLaunches = (nE + nG > 0 ? 1 : 0) + (nD > 0 ? 1 : 0);
    dv.haveParams = true;
    return P4G_OK;
}

extern "C" int p4g_setPrams(p4g_tree *tt, int pNum)
{
    Tree *t = T_(tt);
    if (!t) return setError(P4G_EINVAL, "setPrams: null tree");
    if (pNum < -1 || pNum >= t->nParts) return setError(P4G_EINVAL, "setPrams: bad part %d", pNum);
    return enqueueSetPrams(t, pNum);
}

// Per-pattern outputs (only allocated once getSiteLikes is asked for).
static int setSiteOutputs(Tree *t, bool on)
{
    TreeDev &dv = t->dev;
    if (on && dv.oPat.empty()) {
        size_t n = 0, nc = 0;
        dv.oPat.resize(t->nParts);
        dv.oCatLike.resize(t->nParts);
        for (int p = 0; p < t->nParts; p++) {
            dv.oPat[p] = n;
            dv.oCatLike[p] = nc;
            n += t->data->parts[p]->nPatterns;
            nc += (size_t)t->data->parts[p]->nPatterns * t->model->parts[p].nCat;
        }
        RET(dv.dLike.ensure(sizeof(float) * n));
        RET(dv.dExp.ensure(sizeof(int) * n));
        RET(dv.dLnl.ensure(sizeof(double) * n));
        RET(dv.dCatLike.ensure(sizeof(float) * nc));
    }
    const bool cl = on && dv.rootCLOn;
    if (cl && dv.oRootCL.empty()) {
        size_t n = 0;
        dv.oRootCL.resize(t->nParts);
        for (int p = 0; p < t->nParts; p++) {
            dv.oRootCL[p] = n;
            n += (size_t)t->data->parts[p]->nPatterns * t->model->parts[p].nCat * t->model->parts[p].dim;
        }
        RET(dv.dRootCL.ensure(sizeof(float) * n));
    }
    if (on == dv.jobsSiteOutputs && cl == dv.jobsRootCL) return P4G_OK;
    PruneJob *jobs = (PruneJob *)((char *)dv.hImg.ptr + dv.oJobs);
    for (int p = 0; p < t->nParts; p++) {
        jobs[p].likeScaled = on ? dv.dLike.as<float>() + dv.oPat[p] : nullptr;
        jobs[p].exps = on ? dv.dExp.as<int>() + dv.oPat[p] : nullptr;
        jobs[p].lnl = on ? dv.dLnl.as<double>() + dv.oPat[p] : nullptr;
        jobs[p].catLikes = on ? dv.dCatLike.as<float>() + dv.oCatLike[p] : nullptr;
        jobs[p].rootCL = cl ? dv.dRootCL.as<float>() + dv.oRootCL[p] : nullptr;
    }
    dv.jobsSiteOutputs = on;
    dv.jobsRootCL = cl;
    return P4G_OK;
}

static int enqueueLogLike64(Tree *t);

// Pruning tile-shape autotuner: for each (dim, nCat) group, time every
// candidate shape on this tree (3 launches each, CUDA events) and keep the
// fastest; decisions are cached per (dim, nCat, nTax, pattern-count bucket).
static std::unordered_map<unsigned long long, int> g_tuneCache;
static bool g_autotune = true;

static int autotune(Tree *t, bool fresh = false)
{
    TreeDev &dv = t->dev;
    const char *g = (const char *)dv.dImg.ptr;
    const PruneJob *dJobs = (const PruneJob *)(g + dv.oJobs);
    const BlockDesc *dBlocks = (const BlockDesc *)(g + dv.oBlocks);
    for (auto &gr : dv.groups) {
        long long nPat = 0;
        for (int p = 0; p < t->nParts; p++)
            if (t->model->parts[p].dim == gr.dim && t->model->parts[p].nCat == gr.nCat)
                nPat += t->data->parts[p]->nPatterns;
        int bucket = 0;
        while ((1LL << bucket) < nPat) bucket++;
        unsigned long long key = ((unsigned long long)gr.dim << 48) ^ ((unsigned long long)gr.nCat << 40) ^
                                 ((unsigned long long)t->data->nTax << 16) ^ (unsigned long long)bucket;
        auto it = fresh ? g_tuneCache.end() : g_tuneCache.find(key);
        const int nShapes = pruneNumShapes(gr.dim);
        if (it != g_tuneCache.end() || !g_autotune || nShapes == 1) {
            gr.shape = (it != g_tuneCache.end()) ? it->second : defaultShape(gr.dim);
            continue;
        }
        cudaEvent_t e0, e1;
        P4G_CUDA(cudaEventCreate(&e0));
        P4G_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        int bestShape = defaultShape(gr.dim);
        // the first shapes should not be timed on a GPU still raising its
        // clocks: run the default shape a few times first
        gr.shape = bestShape;
        gr.smem = pruneSmemBytes(gr.dim, gr.nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, bestShape,
                                 dv.nClade, dv.nDeck, dv.nRow);
        if (gr.smem <= 227 * 1024) {
            RET(waitImage(t));
            RET(layoutBlocks(t));
            RET(uploadImage(t));
            for (int r = 0; r < 8; r++)
                RET(launchPrune(dJobs, dBlocks + gr.blk0, gr.nBlk, gr.dim, gr.nCat, gr.smem, bestShape,
                                g_ctx.stream));
        }
        // two alternating rounds, each shape's best kept: a drift of the
        // clocks or a slow launch does not decide between close shapes
        std::vector<float> shapeMs(nShapes, 1e30f);
        for (int round = 0; round < 2; round++)
            for (int sh = 0; sh < nShapes; sh++) {
                if (!pruneShapeValid(gr.dim, gr.nCat, sh)) continue;
                gr.shape = sh;
                gr.smem = pruneSmemBytes(gr.dim, gr.nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, sh,
                                         dv.nClade, dv.nDeck, dv.nRow);
                if (gr.smem > 227 * 1024) continue;
                RET(waitImage(t));
                RET(layoutBlocks(t));
                RET(uploadImage(t));
                int rc = launchPrune(dJobs, dBlocks + gr.blk0, gr.nBlk, gr.dim, gr.nCat, gr.smem, sh, g_ctx.stream);
                if (rc != P4G_OK) continue;
                P4G_CUDA(cudaEventRecord(e0, g_ctx.stream));
                for (int r = 0; r < 3; r++)
                    RET(launchPrune(dJobs, dBlocks + gr.blk0, gr.nBlk, gr.dim, gr.nCat, gr.smem, sh,
                                    g_ctx.stream));
                P4G_CUDA(cudaEventRecord(e1, g_ctx.stream));
                P4G_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                P4G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                shapeMs[sh] = std::min(shapeMs[sh], ms);
            }
        for (int sh = 0; sh < nShapes; sh++)
            if (shapeMs[sh] < best) {
                best = shapeMs[sh];
                bestShape = sh;
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        gr.shape = bestShape;
        g_tuneCache[key] = bestShape;
    }
    for (auto &gr : dv.groups)
        gr.smem = pruneSmemBytes(gr.dim, gr.nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, gr.shape,
                                 dv.nClade, dv.nDeck, dv.nRow);
    RET(waitImage(t));
    RET(layoutBlocks(t));
    RET(uploadImage(t));
    dv.tuned = true;
    return P4G_OK;
}

// Launches of one evaluation's pruning (clade tables, cherry tables, then
// every group), three times, timed on the stream.  Each pass leaves complete
// tables behind, so the evaluation's own launches can follow.
static int timePruning(Tree *t, float &ms)
{
    TreeDev &dv = t->dev;
    const char *g = (const char *)dv.dImg.ptr;
    const PruneJob *dJobs = (const PruneJob *)(g + dv.oJobs);
    const BlockDesc *dBlocks = (const BlockDesc *)(g + dv.oBlocks);
    cudaEvent_t e0, e1;
    P4G_CUDA(cudaEventCreate(&e0));
    P4G_CUDA(cudaEventCreate(&e1));
    RET(cladeLaunch(t, g_ctx.stream));   // warm
    RET(launchCherry(dJobs, t->nParts, dv.cherryWork, g_ctx.stream));
    for (auto &gr : dv.groups)
        RET(launchPrune(dJobs, dBlocks + gr.blk0, gr.nBlk, gr.dim, gr.nCat, gr.smem, gr.shape, g_ctx.stream));
    P4G_CUDA(cudaEventRecord(e0, g_ctx.stream));
    for (int r = 0; r < 3; r++) {
        RET(cladeLaunch(t, g_ctx.stream));
        RET(launchCherry(dJobs, t->nParts, dv.cherryWork, g_ctx.stream));
        for (auto &gr : dv.groups)
            RET(launchPrune(dJobs, dBlocks + gr.blk0, gr.nBlk, gr.dim, gr.nCat, gr.smem, gr.shape, g_ctx.stream));
    }
    P4G_CUDA(cudaEventRecord(e1, g_ctx.stream));
    P4G_CUDA(cudaEventSynchronize(e1));
    P4G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return P4G_OK;
}

static int rebuildProgram(Tree *t)
{
    TreeDev &dv = t->dev;
    RET(waitImage(t));
    dv.progDirty = true;
    RET(refreshProgram(t));
    RET(layoutBlocks(t));
    return uploadImage(t);
}

// On a tree's first evaluation (unless the caller set the clade size): keep
// the clade tables only if they make the pruning faster.  A tree whose
// patterns do not fill the GPU gains nothing from a shorter whole-tree
// program and pays the extra launch.
// The clade-table launches alone, three times, timed on the stream.
static int timeCladeLaunch(Tree *t, float &ms)
{
    cudaEvent_t e0, e1;
    P4G_CUDA(cudaEventCreate(&e0));
    P4G_CUDA(cudaEventCreate(&e1));
    RET(cladeLaunch(t, g_ctx.stream));   // warm
    P4G_CUDA(cudaEventRecord(e0, g_ctx.stream));
    for (int r = 0; r < 3; r++) RET(cladeLaunch(t, g_ctx.stream));
    P4G_CUDA(cudaEventRecord(e1, g_ctx.stream));
    P4G_CUDA(cudaEventSynchronize(e1));
    P4G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return P4G_OK;
}

// Tile shape of each clade-table group: every CUDA-core shape of its
// (dim, nCat), timed twice in alternation, the fastest kept.  The tables
// are small (the tree's clade combinations), so latency decides: lane
// groups spread them over more blocks, shared-memory decks replace one L1
// round trip per op by one staging burst.
static int tuneCladeShapes(Tree *t)
{
    TreeDev &dv = t->dev;
    std::vector<std::pair<int, int>> keys;
    for (auto &g : dv.cladeGroups) keys.push_back({g.dim, g.nCat});
    for (auto &k : keys) {
        const int key = k.first * 64 + k.second;
        std::vector<int> cand;
        for (int sh = 0; sh < pruneNumShapes(k.first); sh++)
            if (pruneShapeValid(k.first, k.second, sh)) cand.push_back(sh);
        std::vector<float> best(cand.size(), 1e30f);
        for (int round = 0; round < 2; round++)
            for (size_t c = 0; c < cand.size(); c++) {
                dv.cladeShape[key] = cand[c];
                if (rebuildProgram(t) != P4G_OK) continue;   // e.g. shared memory too small for the shape
                float ms = 0.f;
                if (timeCladeLaunch(t, ms) == P4G_OK) best[c] = std::min(best[c], ms);
            }
        size_t b = 0;
        for (size_t c = 1; c < cand.size(); c++)
            if (best[c] < best[b]) b = c;
        dv.cladeShape[key] = cand[b];
    }
    return rebuildProgram(t);
}

static int tuneClades(Tree *t)
{
    TreeDev &dv = t->dev;
    dv.cladeChecked = true;
    if (!g_autotune || dv.nClade == 0) return P4G_OK;
    // the largest clade size: the default and smaller ones (fewer leaves,
    // fewer distinct combinations per table, more of the tree left to the
    // whole-tree program) and no tables at all, the programs timed in
    // alternation (three rounds, each one's best) so that a clock ramp at the
    // start of the process favours none; then the clade launches' tile
    // shape for the size kept
    std::vector<int> sizes{0};
    for (int L : {dv.cladeSize, 8, 6, 4, 3, 2})
        if (L >= 2 && L <= 8 && std::find(sizes.begin(), sizes.end(), L) == sizes.end()) sizes.push_back(L);
    std::vector<float> best(sizes.size(), 1e30f);
    for (int round = 0; round < 3; round++)
        for (size_t k = 0; k < sizes.size(); k++) {
            dv.cladeOff = sizes[k] == 0;
            if (sizes[k]) dv.cladeSize = sizes[k];
            if (rebuildProgram(t) != P4G_OK) continue;
            if (!dv.cladeOff && dv.nClade == 0) continue;   // no clade of that size
            float ms = 0.f;
            RET(timePruning(t, ms));
            best[k] = std::min(best[k], ms);
        }
    size_t b = 0;
    for (size_t k = 1; k < sizes.size(); k++)
        if (best[k] < best[b]) b = k;
    dv.cladeOff = sizes[b] == 0;
    if (sizes[b]) dv.cladeSize = sizes[b];
    RET(rebuildProgram(t));
    if (!dv.cladeOff) {
        RET(tuneCladeShapes(t));
        float ms = 0.f;
        RET(timePruning(t, ms));   // renumbered combinations: this evaluation's tables
    }
    return P4G_OK;
}

extern "C" int p4g_setCladeShape(p4g_tree *tt, int group, int shape)
{
    Tree *t = T_(tt);
    if (!t || group < 0 || group >= (int)t->dev.groups.size())
        return setError(P4G_EINVAL, "setCladeShape: bad tree or group (evaluate the tree once first)");
    TreeDev &dv = t->dev;
    const PruneGroup &gr = dv.groups[group];
    if (!pruneShapeValid(gr.dim, gr.nCat, shape))
        return setError(P4G_EINVAL, "setCladeShape: shape %d does not apply to dim=%d nCat=%d", shape, gr.dim,
                        gr.nCat);
    RET(waitImage(t));
    dv.cladeShape[gr.dim * 64 + gr.nCat] = shape;
    dv.cladeChecked = true;
    dv.progDirty = true;
    return P4G_OK;
}

extern "C" int p4g_setGraphs(p4g_tree *tt, int on)
{
    Tree *t = T_(tt);
    if (!t) return setError(P4G_EINVAL, "setGraphs: null tree");
    if (g_ctx.stream) P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    t->dev.useGraphs = on != 0;
    t->dev.setPramsGraph.release();
    t->dev.pruneGraph.release();
    return P4G_OK;
}

extern "C" int p4g_setProgrammaticLaunch(int on)
{
    g_pdl = on != 0;
    return P4G_OK;
}

extern "C" int p4g_setAutotune(int on)
{
    g_autotune = on != 0;
    if (!on) g_tuneCache.clear();
    return P4G_OK;
}

extern "C" int p4g_setPruneShape(p4g_tree *tt, int group, int shape)
{
    Tree *t = T_(tt);
    if (!t || group < 0 || group >= (int)t->dev.groups.size())
        return setError(P4G_EINVAL, "setPruneShape: bad tree or group (evaluate the tree once first)");
    TreeDev &dv = t->dev;
    PruneGroup &gr = dv.groups[group];
    if (!pruneShapeValid(gr.dim, gr.nCat, shape))
        return setError(P4G_EINVAL, "setPruneShape: shape %d does not apply to dim=%d nCat=%d", shape, gr.dim,
                        gr.nCat);
    RET(waitImage(t));
    if (dv.progDirty) RET(refreshProgram(t));
    const int smem = pruneSmemBytes(gr.dim, gr.nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, shape, dv.nClade,
                                    dv.nDeck, dv.nRow);
    if (smem > 227 * 1024)
        return setError(P4G_EUNSUPPORTED, "setPruneShape: shape %d needs %d bytes of shared memory", shape, smem);
    gr.shape = shape;
    gr.smem = smem;
    RET(layoutBlocks(t));
    RET(uploadImage(t));
    dv.tuned = true;
    return P4G_OK;
}

extern "C" int p4g_setCladeSize(p4g_tree *tt, int maxLeaves)
{
    Tree *t = T_(tt);
    if (!t || maxLeaves < 0 || maxLeaves > 8) return setError(P4G_EINVAL, "setCladeSize: 0..8 leaves");
    TreeDev &dv = t->dev;
    if (dv.cladeSize != maxLeaves || dv.cladeOff) {
        RET(waitImage(t));
        dv.cladeSize = maxLeaves;
        dv.cladeOff = false;
        dv.progDirty = true;
    }
    dv.cladeChecked = true;   // the caller's choice; no timed decision
    return P4G_OK;
}

extern "C" int p4g_getPruneShape(p4g_tree *tt, int group, int *shape, int *tile)
{
    Tree *t = T_(tt);
    if (!t || group < 0 || group >= (int)t->dev.groups.size())
        return setError(P4G_EINVAL, "getPruneShape: bad group");
    if (shape) *shape = t->dev.groups[group].shape;
    if (tile) *tile = pruneTile(t->dev.groups[group].dim, t->dev.groups[group].shape);
    return P4G_OK;
}

// Enqueue pruning + result copy for a tree (no synchronisation).
static int enqueueLogLike(Tree *t, bool siteLikes)
{
    TreeDev &dv = t->dev;
    if (dv.precision == 1) {
        if (siteLikes)
            return setError(P4G_EUNSUPPORTED, "site likelihoods come from the FP32 path (precision 0)");
        return enqueueLogLike64(t);
    }
    if (!dv.allocated || !dv.haveParams)
        return setError(P4G_ESTATE, "treeLogLike before setPrams");
    bool reupload = false;
    if (dv.progDirty) {
        RET(waitImage(t));
        RET(refreshProgram(t));
        reupload = true;
    }
    if (siteLikes != dv.jobsSiteOutputs || (siteLikes && dv.rootCLOn) != dv.jobsRootCL) {
        RET(waitImage(t));
        RET(setSiteOutputs(t, siteLikes));
        reupload = true;
    }
    if (reupload) RET(uploadImage(t));
    const char *g = (const char *)dv.dImg.ptr;
    const PruneJob *dJobs = (const PruneJob *)(g + dv.oJobs);
    const BlockDesc *dBlocks = (const BlockDesc *)(g + dv.oBlocks);
    // the clade launch stages its jobs and codes before its wait unless the
    // stream's last kernel numbered this tree's clades
    const int earlyC = dv.cladeFresh ? 0 : PDL_EARLY_JOBS;
    auto enqueue = [&]() -> int {
        RET(cladeLaunch(t, g_ctx.stream, earlyC));
        RET(launchCherry(dJobs, t->nParts, dv.cherryWork, g_ctx.stream));
        // A whole-tree launch that follows a clade-table or cherry-table launch
        // (or another whole-tree launch) may stage its program, codes and P
        // decks before its wait: those kernels write only their own tables
        // and sums.  The first launch of the sequence waits first.
        bool safePrev = dv.cherryWork > 0 && t->nParts > 0;
        for (const auto &cg : dv.cladeGroups)
            if (dv.nClade && cg.nBlk > 0) safePrev = true;
        for (auto &gr : dv.groups) {
            const int early = safePrev ? (PDL_EARLY_JOBS | PDL_EARLY_DECKS) : 0;
            RET(launchPrune(dJobs, dBlocks + gr.blk0, gr.nBlk, gr.dim, gr.nCat, gr.smem, gr.shape, g_ctx.stream,
                            nullptr, early));
            if (gr.nBlk > 0) safePrev = true;
        }
        P4G_CUDA(cudaMemcpyAsync(dv.hOut.ptr, dv.dOut.ptr, sizeof(double) * t->nParts + sizeof(int),
                                 cudaMemcpyDeviceToHost, g_ctx.stream));
        return P4G_OK;
    };
    if (!dv.tuned || !dv.cladeChecked) {   // first evaluation: tables, then the timed choices
        RET(cladeLaunch(t, g_ctx.stream));
        RET(launchCherry(dJobs, t->nParts, dv.cherryWork, g_ctx.stream));
        const bool shapesTimed = !dv.tuned;   // not pinned by the caller
        if (!dv.tuned) RET(autotune(t));
        if (!dv.cladeChecked) {
            const int size0 = dv.cladeSize;
            const bool off0 = dv.cladeOff;
            RET(tuneClades(t));
            // the shapes were timed with the default clade size: time them
            // again with the size kept, so that the pair is chosen together
            if (shapesTimed && g_autotune && (dv.cladeSize != size0 || dv.cladeOff != off0))
                RET(autotune(t, true));
        }
        for (auto &gr : dv.groups)
            RET(launchPrune(dJobs, dBlocks + gr.blk0, gr.nBlk, gr.dim, gr.nCat, gr.smem, gr.shape, g_ctx.stream));
        P4G_CUDA(cudaMemcpyAsync(dv.hOut.ptr, dv.dOut.ptr, sizeof(double) * t->nParts + sizeof(int),
                                 cudaMemcpyDeviceToHost, g_ctx.stream));
        return P4G_OK;
    }
    if (!dv.useGraphs) return enqueue();
    // the launch sequence depends on the image and clade buffers (kernel
    // arguments), the tile layout of every group and the cherry work
    std::vector<long long> sig = {(long long)(size_t)dv.dImg.ptr, (long long)(size_t)dv.hOut.ptr,
                                  (long long)(size_t)dv.dOut.ptr, t->nParts, dv.cherryWork, dv.nClade,
                                  (long long)(size_t)dv.dCladeMeta.ptr, (long long)(size_t)dv.dCladeBlocks.ptr,
                                  (long long)(size_t)dv.dCladeMisc.ptr, siteLikes, dv.jobsRootCL, earlyC};
    for (auto &gr : dv.groups)
        sig.insert(sig.end(), {gr.dim, gr.nCat, gr.blk0, gr.nBlk, gr.smem, gr.shape});
    for (auto &gr : dv.cladeGroups)
        sig.insert(sig.end(), {gr.dim, gr.nCat, gr.blk0, gr.nBlk, gr.smem, gr.shape});
    return dv.pruneGraph.run(sig, g_ctx.stream, enqueue);
}

// ---------------------------------------------------------------- plain FP64
int Part::upload64(cudaStream_t s)
{
    if (dev64Valid) return P4G_OK;
    RET(dPat32.ensure(sizeof(int) * patterns.size()));
    RET(dEqInt.ensure(sizeof(int) * std::max<size_t>(equates.size(), 1)));
    P4G_CUDA(cudaMemcpyAsync(dPat32.ptr, patterns.data(), sizeof(int) * patterns.size(),
                             cudaMemcpyHostToDevice, s));
    if (!equates.empty())
        P4G_CUDA(cudaMemcpyAsync(dEqInt.ptr, equates.data(), sizeof(int) * equates.size(),
                                 cudaMemcpyHostToDevice, s));
    P4G_CUDA(cudaStreamSynchronize(s));
    dev64Valid = true;
    return P4G_OK;
}

// Post-order table of internal nodes: self, nKids, (child, kind, ref) per
// child in sibling order; kind 0 = leaf (ref = seqNum), 1 = internal (ref =
// the child's post-order index).  The root (leaf or not) is last.
static int buildTable64(Tree *t)
{
    TreeDev &dv = t->dev;
    std::vector<int> order;
    std::vector<int> stack{t->root};
    std::vector<char> seen(t->nNodes, 0);
    while (!stack.empty()) {
        int v = stack.back();
        if (!seen[v]) {
            seen[v] = 1;
            for (int c = t->nodes[v]->leftChild; c >= 0; c = t->nodes[c]->sibling) stack.push_back(c);
        } else {
            stack.pop_back();
            if (!t->nodes[v]->isLeaf || v == t->root) order.push_back(v);
        }
    }
    std::vector<int> idx(t->nNodes, -1);
    for (size_t k = 0; k < order.size(); k++) idx[order[k]] = (int)k;
    dv.table64.clear();
    dv.nodeStart64.clear();
    for (int v : order) {
        dv.nodeStart64.push_back((int)dv.table64.size());
        dv.table64.push_back(v);
        int nk = 0;
        size_t at = dv.table64.size();
        dv.table64.push_back(0);
        for (int c = t->nodes[v]->leftChild; c >= 0; c = t->nodes[c]->sibling) {
            Node *nc = t->nodes[c];
            bool leaf = nc->isLeaf != 0;
            dv.table64.push_back(c);
            dv.table64.push_back(leaf ? 0 : 1);
            dv.table64.push_back(leaf ? nc->seqNum : idx[c]);
            nk++;
        }
        dv.table64[at] = nk;
    }
    dv.nInternal64 = (int)order.size();
    std::vector<int> blob(dv.nodeStart64);
    blob.insert(blob.end(), dv.table64.begin(), dv.table64.end());
    RET(dv.dTable64.ensure(sizeof(int) * blob.size()));
    P4G_CUDA(cudaMemcpyAsync(dv.dTable64.ptr, blob.data(), sizeof(int) * blob.size(),
                             cudaMemcpyHostToDevice, g_ctx.stream));
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    // conditional likelihood storage and root partials per part
    size_t nCl = 0, nPartials = 0;
    dv.oCl64.assign(t->nParts, 0);
    dv.oPartials64.assign(t->nParts, 0);
    for (int p = 0; p < t->nParts; p++) {
        const ModelPart &mp = t->model->parts[p];
        Part *dp = t->data->parts[p];
        dv.oCl64[p] = nCl;
        nCl += (size_t)dv.nInternal64 * mp.nCat * mp.dim * dp->nPatPad;
        dv.oPartials64[p] = nPartials;
        nPartials += (dp->nPatterns + 127) / 128;
    }
    RET(dv.dCl64.ensure(sizeof(double) * nCl));
    RET(dv.dPartials64.ensure(sizeof(double) * nPartials));
    dv.table64Dirty = false;
    return P4G_OK;
}

static int enqueueLogLike64(Tree *t)
{
    TreeDev &dv = t->dev;
    if (!dv.allocated || !dv.haveParams) return setError(P4G_ESTATE, "treeLogLike before setPrams");
    if (dv.progDirty) {
        RET(waitImage(t));
        RET(refreshProgram(t));
        RET(uploadImage(t));
    }
    for (int p = 0; p < t->nParts; p++) RET(t->data->parts[p]->upload64(g_ctx.stream));
    if (dv.table64Dirty) RET(buildTable64(t));
    const PruneJob *hj = (const PruneJob *)((const char *)dv.hImg.ptr + dv.oJobs);
    std::vector<Node64Job> jobs(t->nParts);
    for (int p = 0; p < t->nParts; p++) {
        const ModelPart &mp = t->model->parts[p];
        Part *dp = t->data->parts[p];
        Node64Job &J = jobs[p];
        J.decks64 = dv.dDecks64.as<double>() + dv.oDecks[p];
        J.patterns = dp->dPat32.as<int>();
        J.equates = dp->dEqInt.as<int>();
        J.nodeStart = dv.dTable64.as<int>();
        J.table = dv.dTable64.as<int>() + dv.nInternal64;
        J.cl = dv.dCl64.as<double>() + dv.oCl64[p];
        J.rootComp = hj[p].rootComp;
        J.counts = dp->dCounts.as<double>();
        J.invMask = dp->dInvMask.as<uint32_t>();
        J.partials = dv.dPartials64.as<double>() + dv.oPartials64[p];
        J.out = dv.dOut.as<double>() + p;
        J.ticket = dv.dTicket.as<int>() + p;
        J.badFlag = dv.dBad.as<int>() + p;
        J.pInvar = mp.pInvar;
        J.varScale = (1.0 - mp.pInvar) / (double)mp.nCat;
        J.nPat = dp->nPatterns;
        J.nPatPad = dp->nPatPad;
        J.nCat = mp.nCat;
        J.dim = mp.dim;
        J.nInternal = dv.nInternal64;
        J.rootInternal = dv.nInternal64 - 1;
        Node *rn = t->nodes[t->root];
        J.rootLeafRow = rn->isLeaf ? rn->seqNum : -1;
    }
    RET(dv.dJobs64.ensure(sizeof(Node64Job) * t->nParts));
    P4G_CUDA(cudaMemcpyAsync(dv.dJobs64.ptr, jobs.data(), sizeof(Node64Job) * t->nParts,
                             cudaMemcpyHostToDevice, g_ctx.stream));
    dv.jobs64 = jobs;
    for (int p = 0; p < t->nParts; p++)
        RET(launchPrune64(dv.dJobs64.as<Node64Job>() + p, jobs[p], g_ctx.stream));
    P4G_CUDA(cudaMemcpyAsync(dv.hOut.ptr, dv.dOut.ptr, sizeof(double) * t->nParts + sizeof(int),
                             cudaMemcpyDeviceToHost, g_ctx.stream));
    return P4G_OK;
}

extern "C" int p4g_setPrecision(p4g_tree *tt, int mode)
{
    Tree *t = T_(tt);
    if (!t || (mode != 0 && mode != 1)) return setError(P4G_EINVAL, "setPrecision: mode must be 0 or 1");
    t->dev.precision = mode;
    return P4G_OK;
}

// After the stream is synchronised: part likes, total, status.
static int finishLogLike(Tree *t, bool siteLikes, double *lnL)
{
    TreeDev &dv = t->dev;
    const double *out = dv.hOut.as<double>();
    int status = *(const int *)((const char *)dv.hOut.ptr + sizeof(double) * t->nParts);
    if (status) {
        cudaMemsetAsync(treeStatus(t), 0, sizeof(int), g_ctx.stream);
        return setError(P4G_ENUMERIC, "setPrams: %s did not converge",
                        (status & 1) ? "discrete gamma" : "eigensystem");
    }
    for (int p = 0; p < t->nParts; p++)
        if (out[p] != out[p]) return setError(P4G_ETIMEOUT, "pruning: a device-side check failed (a tensor-core completion wait gave up, or a clade-table index was out of range)");
    double sum = 0.0;
    for (int p = 0; p < t->nParts; p++) {
        t->partLikes[p] = out[p];
        sum += out[p];
    }
    t->logLike = sum;
    *lnL = sum;
    if (siteLikes) {
        for (int p = 0; p < t->nParts; p++) {
            Part *dp = t->data->parts[p];
            std::vector<double> lnl(dp->nPatterns);
            P4G_CUDA(cudaMemcpy(lnl.data(), dv.dLnl.as<double>() + dv.oPat[p],
                                sizeof(double) * dp->nPatterns, cudaMemcpyDeviceToHost));
            dp->siteLikes.resize(dp->nChar);
            for (int i = 0; i < dp->nChar; i++) dp->siteLikes[i] = exp(lnl[dp->seqPosIdx[i]]);
        }
    }
    return P4G_OK;
}

extern "C" int p4g_treeLogLike(p4g_tree *tt, int getSiteLikes, double *lnL)
{
    Tree *t = T_(tt);
    if (!t || !lnL) return setError(P4G_EINVAL, "treeLogLike: null argument");
    RET(enqueueLogLike(t, getSiteLikes != 0));
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    return finishLogLike(t, getSiteLikes != 0, lnL);
}

extern "C" int p4g_partLogLike(p4g_tree *tt, p4g_part *pp, int pNum, int getSiteLikes, double *lnL)
{
    Tree *t = T_(tt);
    if (!t || !lnL || pNum < 0 || pNum >= t->nParts || (pp && P_(pp) != t->data->parts[pNum]))
        return setError(P4G_EINVAL, "partLogLike: bad arguments");
    double total;
    RET(p4g_treeLogLike(tt, getSiteLikes, &total));
    *lnL = t->partLikes[pNum];
    return P4G_OK;
}

extern "C" int p4g_calculateAllBigPDecksAllParts(p4g_tree *tt) { return p4g_setPrams(tt, -1); }

extern "C" int p4g_calculateBigPDecks(p4g_node *nn)
{
    Node *n = N_(nn);
    if (!n) return setError(P4G_EINVAL, "calculateBigPDecks: null node");
    // decks of every node are recomputed together on the device (cheap
    // next to pruning); the eigensystems are refreshed with them
    return p4g_setPrams(reinterpret_cast<p4g_tree *>(n->tree), -1);
}

extern "C" int p4g_treeLogLikeBatch(p4g_tree **trees, int nTrees, int doSetPrams, double *lnL)
{
    if (!trees || nTrees < 1 || !lnL) return setError(P4G_EINVAL, "treeLogLikeBatch: bad arguments");
    for (int i = 0; i < nTrees; i++) {
        Tree *t = T_(trees[i]);
        if (doSetPrams) RET(enqueueSetPrams(t, -1));
        RET(enqueueLogLike(t, false));
    }
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    for (int i = 0; i < nTrees; i++) RET(finishLogLike(T_(trees[i]), false, &lnL[i]));
    return P4G_OK;
}

extern "C" int p4g_setBrLens(p4g_tree *tt, const double *brLens)
{
    Tree *t = T_(tt);
    if (!t || !brLens) return setError(P4G_EINVAL, "setBrLens: null argument");
    for (int v = 0; v < t->nNodes; v++)
        if (t->nodes[v] && v != t->root) t->nodes[v]->brLen = brLens[v];
    return P4G_OK;
}

extern "C" int p4g_setTopology(p4g_tree *tt, const int *parent, const int *leftChild,
                               const int *sibling, int root)
{
    Tree *t = T_(tt);
    if (!t || !parent || !leftChild || !sibling || root < 0 || root >= t->nNodes || !t->nodes[root])
        return setError(P4G_EINVAL, "setTopology: bad arguments");
    bool changed = (t->root != root);
    for (int v = 0; v < t->nNodes; v++) {
        Node *n = t->nodes[v];
        if (!n) continue;
        if (parent[v] < -1 || parent[v] >= t->nNodes || leftChild[v] < -1 ||
            leftChild[v] >= t->nNodes || sibling[v] < -1 || sibling[v] >= t->nNodes)
            return setError(P4G_EINVAL, "setTopology: node %d relation out of range", v);
        changed |= n->parent != parent[v] || n->leftChild != leftChild[v] || n->sibling != sibling[v];
        n->parent = parent[v];
        n->leftChild = leftChild[v];
        n->sibling = sibling[v];
    }
    t->root = root;
    if (changed) t->dev.progDirty = true;
    return P4G_OK;
}

extern "C" int p4g_setRMatrixUpper(p4g_model *mm, int pNum, int rNum, const double *vals)
{
    Model *m = M_(mm);
    if (!m || !vals || pNum < 0 || pNum >= m->nParts || rNum < 0 || rNum >= m->parts[pNum].nRMatrices)
        return setError(P4G_EINVAL, "setRMatrixUpper: bad arguments");
    ModelPart &mp = m->parts[pNum];
    std::vector<double> &R = mp.rMatrices[rNum].bigR;
    int k = 0;
    for (int i = 0; i < mp.dim - 1; i++)
        for (int j = i + 1; j < mp.dim; j++, k++) {
            R[(size_t)i * mp.dim + j] = vals[k];
            R[(size_t)j * mp.dim + i] = vals[k];
        }
    return P4G_OK;
}

extern "C" int p4g_treeLogLikeAsync(p4g_tree *tt, int doSetPrams)
{
    Tree *t = T_(tt);
    if (!t) return setError(P4G_EINVAL, "treeLogLikeAsync: null tree");
    if (doSetPrams) RET(enqueueSetPrams(t, -1));
    return enqueueLogLike(t, false);
}

extern "C" int p4g_treeLogLikeWait(p4g_tree *tt, double *lnL)
{
    Tree *t = T_(tt);
    if (!t || !lnL) return setError(P4G_EINVAL, "treeLogLikeWait: null argument");
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    return finishLogLike(t, false, lnL);
}

extern "C" int p4g_treeInfo(p4g_tree *tt, long long *info)
{
    Tree *t = T_(tt);
    if (!t || !info) return setError(P4G_EINVAL, "treeInfo: null argument");
    RET(validateModel(t, -1));
    RET(allocTreeDev(t));
    RET(refreshProgram(t));
    int launches = (int)t->dev.groups.size();
    int nG = 0, nE = 0, nD = 0;
    long long nPat = 0;
    for (int p = 0; p < t->nParts; p++) {
        const ModelPart &mp = t->model->parts[p];
        nG += mp.nGdasrvs;
        nE += mp.nComps * mp.nRMatrices;
        nD += 1;
        nPat += t->data->parts[p]->nPatterns;
    }
    launches += (nG > 0) + (nE > 0) + (nD > 0);
    info[0] = t->dev.hImgDev ? (long long)(sizeof(double) * t->nNodes) : (long long)t->dev.imgBytes;
    info[1] = launches;
    info[2] = nPat;
    info[3] = t->dev.nSlots;
    info[4] = t->dev.nProg;
    info[5] = (long long)(sizeof(double) * t->nParts + sizeof(int));
    info[6] = t->dev.nClade;
    return P4G_OK;
}

extern "C" int p4g_treeDeviceBytes(p4g_tree *tt, long long *treeBytes, long long *dataBytes)
{
    Tree *t = T_(tt);
    if (!t || !treeBytes || !dataBytes) return setError(P4G_EINVAL, "treeDeviceBytes: null argument");
    const TreeDev &dv = t->dev;
    *treeBytes = dv.allocated ? (long long)(dv.dImg.bytes + dv.dRates.bytes + dv.dEig.bytes + dv.dDecks32.bytes +
                                            dv.dEqTab.bytes + dv.dDecks64.bytes + dv.dPartials.bytes +
                                            dv.dOut.bytes + dv.dTicket.bytes + dv.dBad.bytes)
                              : 0;
    long long db = 0;
    if (t->data)
        for (int p = 0; p < t->nParts; p++) {
            const Part *dp = t->data->parts[p];
            if (dp)
                db += (long long)(dp->dCodes.bytes + dp->dCounts.bytes + dp->dInvMask.bytes + dp->dEquates.bytes +
                                  dp->dPat32.bytes + dp->dEqInt.bytes);
        }
    *dataBytes = db;
    return P4G_OK;
}

static int copyDev(DevBuf &dst, const DevBuf &src)
{
    if (!src.ptr || !dst.ptr || dst.bytes < src.bytes) return setError(P4G_ESTATE, "copy: shapes differ");
    P4G_CUDA(cudaMemcpyAsync(dst.ptr, src.ptr, src.bytes, cudaMemcpyDeviceToDevice, g_ctx.stream));
    return P4G_OK;
}

extern "C" int p4g_copyBigPDecks(p4g_tree *a, p4g_tree *b, int doAll)
{
    (void)doAll;
    Tree *ta = T_(a), *tb = T_(b);
    if (!ta || !tb) return setError(P4G_EINVAL, "copyBigPDecks: null tree");
    RET(allocTreeDev(tb));
    RET(copyDev(tb->dev.dDecks32, ta->dev.dDecks32));
    RET(copyDev(tb->dev.dDecks64, ta->dev.dDecks64));
    RET(copyDev(tb->dev.dEqTab, ta->dev.dEqTab));
    RET(copyDev(tb->dev.dEig, ta->dev.dEig));
    RET(copyDev(tb->dev.dRates, ta->dev.dRates));
    tb->dev.haveParams = ta->dev.haveParams;
    tb->dev.cacheValid = false;
    return P4G_OK;
}

extern "C" int p4g_copyCondLikes(p4g_tree *a, p4g_tree *b, int doAll)
{
    // The fused kernels keep no per-node conditional likelihoods between
    // calls, so there is nothing to copy; the call is accepted for API parity.
    (void)a;
    (void)b;
    (void)doAll;
    return P4G_OK;
}

extern "C" int p4g_copyModelPrams(p4g_tree *a, p4g_tree *b)
{
    Tree *ta = T_(a), *tb = T_(b);
    if (!ta || !tb || ta->nParts != tb->nParts) return setError(P4G_EINVAL, "copyModelPrams: bad trees");
    for (int p = 0; p < ta->nParts; p++) {
        ModelPart &A = ta->model->parts[p], &B = tb->model->parts[p];
        if (A.dim != B.dim || A.nComps != B.nComps || A.nRMatrices != B.nRMatrices ||
            A.nGdasrvs != B.nGdasrvs)
            return setError(P4G_EINVAL, "copyModelPrams: model shapes differ");
        for (int c = 0; c < A.nComps; c++) memcpy(B.comps[c].val, A.comps[c].val, sizeof(double) * A.dim);
        for (int r = 0; r < A.nRMatrices; r++) B.rMatrices[r].bigR = A.rMatrices[r].bigR;
        for (int g = 0; g < A.nGdasrvs; g++) {
            B.gdasrvs[g]->val[0] = A.gdasrvs[g]->val[0];
            memcpy(B.gdasrvs[g]->rates, A.gdasrvs[g]->rates, sizeof(double) * A.nCat);
            memcpy(B.gdasrvs[g]->freqs, A.gdasrvs[g]->freqs, sizeof(double) * A.nCat);
        }
        B.pInvar = A.pInvar;
        B.relRate = A.relRate;
    }
    return P4G_OK;
}

// ============================================================= introspection
extern "C" int p4g_getPDeck(p4g_node *nn, int pNum, int cat, double *out)
{
    Node *n = N_(nn);
    if (!n || !out) return setError(P4G_EINVAL, "getPDeck: null argument");
    Tree *t = n->tree;
    if (!t->dev.haveParams) return setError(P4G_ESTATE, "getPDeck before setPrams");
    const ModelPart &mp = t->model->parts[pNum];
    if (cat < 0 || cat >= mp.nCat) return setError(P4G_EINVAL, "getPDeck: bad cat");
    const double *src = t->dev.dDecks64.as<double>() + t->dev.oDecks[pNum] +
                        ((size_t)n->nodeNum * mp.nCat + cat) * mp.dim * mp.dim;
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    P4G_CUDA(cudaMemcpy(out, src, sizeof(double) * mp.dim * mp.dim, cudaMemcpyDeviceToHost));
    return P4G_OK;
}

extern "C" int p4g_getDecks32(p4g_tree *tt, int pNum, float *decks, float *eqTab, int *nPartial)
{
    Tree *t = T_(tt);
    if (!t || pNum < 0 || pNum >= t->nParts) return setError(P4G_EINVAL, "getDecks32: bad arguments");
    if (!t->dev.haveParams) return setError(P4G_ESTATE, "getDecks32 before setPrams");
    const ModelPart &mp = t->model->parts[pNum];
    const Part *dp = t->data->parts[pNum];
    const int dim = mp.dim, nn = t->nNodes;
    const size_t per = (size_t)dim * dim;
    std::vector<float> raw((size_t)nn * mp.nCat * per);
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    P4G_CUDA(cudaMemcpy(raw.data(), t->dev.dDecks32.as<float>() + t->dev.oDecks[pNum],
                        sizeof(float) * raw.size(), cudaMemcpyDeviceToHost));
    if (decks)
        for (int v = 0; v < nn; v++) {
            bool leaf = t->nodes[v] && t->nodes[v]->isLeaf;
            for (int c = 0; c < mp.nCat; c++) {
                const float *src = raw.data() + ((size_t)v * mp.nCat + c) * per;
                float *dst = decks + ((size_t)v * mp.nCat + c) * per;
                for (int i = 0; i < dim; i++)
                    for (int j = 0; j < dim; j++) dst[i * dim + j] = leaf ? src[j * dim + i] : src[i * dim + j];
            }
        }
    if (nPartial) *nPartial = dp->nPartial;
    if (eqTab && dp->nPartial)
        P4G_CUDA(cudaMemcpy(eqTab, t->dev.dEqTab.as<float>() + t->dev.oEqTab[pNum],
                            sizeof(float) * (size_t)nn * dp->nPartial * mp.nCat * dim,
                            cudaMemcpyDeviceToHost));
    return P4G_OK;
}

extern "C" int p4g_getPatternLikes(p4g_tree *tt, int pNum, float *likeScaled, int *exps, double *lnl)
{
    Tree *t = T_(tt);
    if (!t || pNum < 0 || pNum >= t->nParts) return setError(P4G_EINVAL, "getPatternLikes: bad arguments");
    if (t->dev.oPat.empty()) return setError(P4G_ESTATE, "getPatternLikes: no getSiteLikes evaluation yet");
    const int n = t->data->parts[pNum]->nPatterns;
    const size_t o = t->dev.oPat[pNum];
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    if (likeScaled)
        P4G_CUDA(cudaMemcpy(likeScaled, t->dev.dLike.as<float>() + o, sizeof(float) * n, cudaMemcpyDeviceToHost));
    if (exps) P4G_CUDA(cudaMemcpy(exps, t->dev.dExp.as<int>() + o, sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (lnl) P4G_CUDA(cudaMemcpy(lnl, t->dev.dLnl.as<double>() + o, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return P4G_OK;
}

// pf.getSiteRates (Pf/pfmodule.c:398) = p4_partLogLikeSiteRates
// (Pf/p4_tree.c:1383-1627): a fresh evaluation with per-pattern outputs, then
// per pattern work[c] = sum_s pi_s cl_root[c][s] (the kernel's FP32 sums,
// unscaled in FP64), the site likelihood from them as the reference forms it,
// the first category of largest work and the rate sum_c work[c] (1/nCat)
// rate[c] / like, expanded to sites.
// ---------------------------------------------------------------- draws
// (p4g_sim.cu) setPrams + a site-output evaluation of every part.
int treeLogLikeSites(Tree *t, double *lnL)
{
    RET(enqueueSetPrams(t, -1));
    RET(enqueueLogLike(t, true));
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    return finishLogLike(t, true, lnL);
}

// setPrams alone, finished: the FP64 decks of every node are current.
int setPramsForDraws(Tree *t)
{
    RET(enqueueSetPrams(t, -1));
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    return P4G_OK;
}

// (p4g_newt.cu) setPrams, then the plain FP64 evaluation: every internal
// node's FP64 CL is left in dCl64 and dv.jobs64 describes it.
int fp64Evaluate(Tree *t, bool doSetPrams, double *lnL)
{
    if (doSetPrams) RET(enqueueSetPrams(t, -1));
    RET(enqueueLogLike64(t));
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    return finishLogLike(t, false, lnL);
}

// Drop the tree's device state (its sizes follow the parts' pattern
// counts); the next setPrams rebuilds it.  The caller's settings survive.
int resetTreeDev(Tree *t)
{
    if (g_ctx.stream) P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    TreeDev &dv = t->dev;
    const int precision = dv.precision, cladeSize = dv.cladeSize;
    releaseTreeDev(dv);
    dv.~TreeDev();
    new (&dv) TreeDev();
    dv.precision = precision;
    dv.cladeSize = cladeSize;
    return P4G_OK;
}

extern "C" int p4g_getSiteRates(p4g_tree *tt, p4g_part *pp, int pNum, double *siteRates, int *gammaCats)
{
    Tree *t = T_(tt);
    if (!t || !siteRates || !gammaCats || pNum < 0 || pNum >= t->nParts ||
        (pp && P_(pp) != t->data->parts[pNum]))
        return setError(P4G_EINVAL, "getSiteRates: bad arguments");
    const ModelPart &mp = t->model->parts[pNum];
    if (mp.nGdasrvs != 1) return setError(P4G_EINVAL, "getSiteRates: nGdasrvs is %d, should be 1", mp.nGdasrvs);
    if (t->root < 0 || !t->nodes[t->root] || t->nodes[t->root]->isLeaf)
        return setError(P4G_EUNSUPPORTED, "getSiteRates: the root must be an internal node");
    if (t->dev.precision != 0) return setError(P4G_EUNSUPPORTED, "getSiteRates: needs the FP32 path (precision 0)");
    RET(enqueueSetPrams(t, -1));
    RET(enqueueLogLike(t, true));
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    double lnL;
    RET(finishLogLike(t, true, &lnL));
    TreeDev &dv = t->dev;
    Part *dp = t->data->parts[pNum];
    const int n = dp->nPatterns, nc = mp.nCat, dim = mp.dim;
    std::vector<float> cat((size_t)n * nc);
    std::vector<int> ex(n);
    std::vector<double> rates(nc);
    P4G_CUDA(cudaMemcpy(cat.data(), dv.dCatLike.as<float>() + dv.oCatLike[pNum], sizeof(float) * cat.size(),
                        cudaMemcpyDeviceToHost));
    P4G_CUDA(cudaMemcpy(ex.data(), dv.dExp.as<int>() + dv.oPat[pNum], sizeof(int) * n, cudaMemcpyDeviceToHost));
    P4G_CUDA(cudaMemcpy(rates.data(), dv.dRates.as<double>() + dv.oRates[pNum], sizeof(double) * nc,
                        cudaMemcpyDeviceToHost));
    const double *pi = mp.comps[t->nodes[t->root]->compNums[pNum]].val;
    const double pInvar = mp.pInvar;
    std::vector<double> rate(n), work(nc);
    std::vector<int> best(n);
    for (int k = 0; k < n; k++) {
        double like = 0.0;
        for (int c = 0; c < nc; c++) {
            work[c] = ldexp((double)cat[(size_t)k * nc + c], -ex[k]);
            like += work[c];
        }
        if (pInvar != 0.0) {
            like *= (1.0 - pInvar) / (double)nc;
            if (dp->invVec[k] > 0)
                for (int s = 0; s < dim; s++)
                    if (dp->invArr[(size_t)s * n + k]) like += pi[s] * pInvar;
        } else if (nc > 1) {
            like /= (double)nc;
        }
        int b = 0;
        for (int c = 1; c < nc; c++)
            if (work[c] > work[b]) b = c;
        double num = 0.0;
        for (int c = 0; c < nc; c++) num += work[c] * (1.0 / nc) * rates[c];
        best[k] = b;
        rate[k] = num / like;
    }
    for (int i = 0; i < dp->nChar; i++) {
        siteRates[i] = rate[dp->seqPosIdx[i]];
        gammaCats[i] = best[dp->seqPosIdx[i]];
    }
    return P4G_OK;
}

extern "C" int p4g_getGammaRates(p4g_tree *tt, int pNum, int gNum, double *out)
{
    Tree *t = T_(tt);
    if (!t || pNum < 0 || pNum >= t->nParts) return setError(P4G_EINVAL, "getGammaRates: bad arguments");
    const ModelPart &mp = t->model->parts[pNum];
    if (gNum < 0 || gNum >= mp.nGdasrvs) return setError(P4G_EINVAL, "getGammaRates: bad gdasrv");
    if (!t->dev.haveParams) return setError(P4G_ESTATE, "getGammaRates before setPrams");
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    P4G_CUDA(cudaMemcpy(out, t->dev.dRates.as<double>() + t->dev.oRates[pNum] + (size_t)gNum * mp.nCat,
                        sizeof(double) * mp.nCat, cudaMemcpyDeviceToHost));
    return P4G_OK;
}

// ================================================================ batches
// Several trees (the chains of an MCMCMC) evaluated together: one parameter
// image upload per tree, one combined descriptor image, one k_gammaEig + one
// k_pdeck launch for every (tree, part), one k_prune launch per (dim, nCat)
// group over every tree's tiles, one result copy.  After the first call the
// whole sequence is captured as a CUDA graph and replayed; it is re-captured
// only when a tree's topology grows the pruning kernel's shared memory.
namespace p4g {
struct Batch {
    std::vector<Tree *> trees;
    int nParts = 0;
    PinnedBuf hImg;
    DevBuf dImg;
    size_t imgBytes = 0;
    size_t oDesc = 0, oJobs = 0, oEig = 0, oGam = 0, oCounts = 0, oPrefix = 0, oBlocks = 0;
    int capDesc = 0, capE = 0, capG = 0, capBlocks = 0, nD = 0, maxDim = 0;
    std::vector<PruneGroup> groups;
    DevBuf dOut;   // lnLs, then the setPrams status int
    PinnedBuf hOut;
    std::vector<char> shadow;   // hImg as last copied to the device (empty: unknown)
    // Part-granular evaluation (p4's Chain updates only the part a per-part
    // proposal changed): per (tree, part) the lnL of the last batched
    // evaluation and a copy of the inputs it was computed from.  A part whose
    // inputs are unchanged keeps that lnL and is left out of the P decks,
    // cherry tables and pruning launches (their task and tile counts are read
    // from device memory, so the captured graph is unchanged).
    std::vector<std::vector<char>> treeSig, partSig, pendTreeSig, pendPartSig;
    std::vector<double> lnlCache;
    std::vector<char> lnlOk, dirty;
    bool forceAll = false;          // every part evaluated (tile-shape timing)
    std::vector<int> groupCap;      // tiles each group's region of the tile list holds
    bool useGraph = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<int> capturedSmem;
    bool ready = false;
    bool useClades = false;              // clade tables (p4g_batchSetClades)
    bool tuned = false;                  // tile shapes timed on the whole batch
    std::vector<long long> cladeVersions;   // of every tree, as captured
    // every tree's clade-table work in one launch per (dim, nCat) group: the
    // trees' clade jobs and merged tile lists (rebuilt when any tree's
    // clades change); empty cladeGroups when the trees' clade groups differ
    DevBuf dCladeJobs, dCladeBlocks, dCladeCounts, dCladeSrc;
    std::vector<PruneGroup> cladeGroups;
    // otherwise the trees' clade-table launches run side by side: one stream
    // and one event per tree, forked from and joined back into the library stream
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> joined;
    cudaEvent_t forked = nullptr;
    ~Batch()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (cudaStream_t x : side) cudaStreamDestroy(x);
        for (cudaEvent_t x : joined) cudaEventDestroy(x);
        if (forked) cudaEventDestroy(forked);
    }
};

// The setPrams status int of a batch, right after its lnLs in dOut.
static int *batchStatus(Batch *b)
{
    return (int *)((char *)b->dOut.ptr + sizeof(double) * b->capDesc);
}
}  // namespace p4g

static inline Batch *B_(p4g_batch *b) { return reinterpret_cast<Batch *>(b); }

extern "C" p4g_batch *p4g_newBatch(p4g_tree **trees, int nTrees)
{
    if (!trees || nTrees < 1) {
        setError(P4G_EINVAL, "newBatch: no trees");
        return nullptr;
    }
    Batch *b = new Batch;
    for (int i = 0; i < nTrees; i++) b->trees.push_back(T_(trees[i]));
    Tree *t0 = b->trees[0];
    b->nParts = t0->nParts;
    for (Tree *t : b->trees) {
        bool same = t->nParts == t0->nParts && t->data == t0->data && t->nNodes == t0->nNodes;
        for (int p = 0; same && p < t->nParts; p++)
            same = t->model->parts[p].dim == t0->model->parts[p].dim &&
                   t->model->parts[p].nCat == t0->model->parts[p].nCat;
        if (!same) {
            setError(P4G_EINVAL, "newBatch: trees must share data and model shapes");
            delete b;
            return nullptr;
        }
    }
    for (Tree *t : b->trees) {   // batch launch sequences use no clade tables
        t->dev.inBatch = true;
        t->dev.progDirty = true;
    }
    return reinterpret_cast<p4g_batch *>(b);
}

extern "C" int p4g_freeBatch(p4g_batch *bb)
{
    if (g_ctx.stream) cudaStreamSynchronize(g_ctx.stream);
    delete B_(bb);
    return P4G_OK;
}

extern "C" int p4g_batchSetClades(p4g_batch *bb, int on)
{
    Batch *b = B_(bb);
    if (!b) return setError(P4G_EINVAL, "batchSetClades: null");
    if (g_ctx.stream) P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    b->useClades = on != 0;
    // trees whose clade size was neither timed nor set take the first tree's
    // "no tables" when its timing found them slower (the size itself is not
    // copied: a size timed for one tree's launches is not the best for a
    // batch, whose clade launches queue behind one another)
    const TreeDev &d0 = b->trees[0]->dev;
    for (Tree *t : b->trees) {
        if (t != b->trees[0] && !t->dev.cladeChecked && d0.cladeChecked && d0.cladeOff) t->dev.cladeOff = true;
        t->dev.inBatch = !b->useClades;   // clade selection is off for trees without them
        t->dev.cladeChecked = true;       // no timing inside a batch
        t->dev.progDirty = true;
    }
    b->cladeVersions.clear();
    return P4G_OK;
}

extern "C" int p4g_batchSetGraph(p4g_batch *bb, int on)
{
    Batch *b = B_(bb);
    if (!b) return setError(P4G_EINVAL, "batchSetGraph: null");
    b->useGraph = on != 0;
    return P4G_OK;
}

// First call: device state of every tree, tile shapes (tuned on tree 0 by a
// plain evaluation), the combined image layout.
static int batchPrepare(Batch *b)
{
    Tree *t0 = b->trees[0];
    double tmp;
    RET(enqueueSetPrams(t0, -1));
    RET(enqueueLogLike(t0, false));
    P4G_CUDA(cudaStreamSynchronize(g_ctx.stream));
    RET(finishLogLike(t0, false, &tmp));
    for (Tree *t : b->trees) {
        RET(validateModel(t, -1));
        RET(allocTreeDev(t));
        t->dev.groups = t0->dev.groups;      // same shapes as the tuned tree
        t->dev.tuned = true;
        RET(waitImage(t));
        t->dev.progDirty = true;
        RET(refreshProgram(t));
        RET(layoutBlocks(t));
    }
    b->groups = t0->dev.groups;
    int nPairs = 0, nGd = 0, nBlocks = 0;
    for (Tree *t : b->trees) {
        for (int p = 0; p < t->nParts; p++) {
            nPairs += t->model->parts[p].nComps * t->model->parts[p].nRMatrices;
            nGd += t->model->parts[p].nGdasrvs;
        }
        nBlocks += t->dev.blockCap;   // room for the smallest tiles (the batch may retune its shapes)
    }
    const int nT = (int)b->trees.size();
    b->capDesc = nT * b->nParts;
    b->capE = nPairs;
    b->capG = nGd;
    b->capBlocks = nBlocks;
    size_t o = 0;
    b->oDesc = o;
    o = alignUp(o + sizeof(PmatPart) * b->capDesc, 256);
    b->oJobs = o;
    o = alignUp(o + sizeof(PruneJob) * b->capDesc, 256);
    b->oEig = o;
    o = alignUp(o + sizeof(int2) * std::max(b->capE, 1), 256);
    b->oGam = o;
    o = alignUp(o + sizeof(int2) * std::max(b->capG, 1), 256);
    b->oCounts = o;   // eigen and gamma tasks, P-deck tasks and descriptors, then each group's tiles
    o = alignUp(o + sizeof(int) * (4 + std::max<size_t>(b->groups.size(), 1)), 256);
    b->oPrefix = o;
    o = alignUp(o + sizeof(int) * b->capDesc, 256);
    b->oBlocks = o;
    o = alignUp(o + sizeof(BlockDesc) * b->capBlocks, 256);
    b->imgBytes = o;
    RET(b->hImg.ensure(b->imgBytes));
    RET(b->dImg.ensure(b->imgBytes));
    memset(b->hImg.ptr, 0, b->imgBytes);
    RET(b->dOut.ensure(sizeof(double) * b->capDesc + 16));   // lnLs, then the status int
    RET(b->hOut.ensure(sizeof(double) * b->capDesc + 16));
    P4G_CUDA(cudaMemsetAsync(batchStatus(b), 0, sizeof(int), g_ctx.stream));
    b->capturedSmem.assign(b->groups.size(), 0);
    b->treeSig.assign(nT, {});
    b->pendTreeSig.assign(nT, {});
    b->partSig.assign((size_t)nT * b->nParts, {});
    b->pendPartSig.assign((size_t)nT * b->nParts, {});
    b->lnlCache.assign((size_t)nT * b->nParts, 0.0);
    b->lnlOk.assign((size_t)nT * b->nParts, 0);
    b->dirty.assign((size_t)nT * b->nParts, 1);
    b->groupCap.assign(b->groups.size(), 0);
    b->ready = true;
    return P4G_OK;
}

static void appendBytes(std::vector<char> &v, const void *p, size_t n)
{
    v.insert(v.end(), (const char *)p, (const char *)p + n);
}

// The inputs a tree's lnL depends on beyond its parts' model values: branch
// lengths, topology (the program), node model assignments, the device state's
// and the data's generations.
static void treeSignature(const Tree *t, std::vector<char> &v)
{
    const TreeDev &dv = t->dev;
    v.clear();
    const char *h = (const char *)dv.hImg.ptr;
    appendBytes(v, &dv.devGen, sizeof(dv.devGen));
    appendBytes(v, &dv.nProg, sizeof(dv.nProg));
    appendBytes(v, dv.prog.data(), sizeof(int) * dv.prog.size());
    appendBytes(v, h + dv.oBrLen, sizeof(double) * t->nNodes);
    appendBytes(v, h + dv.oNodeIdx, sizeof(int) * 3 * (size_t)t->nNodes * t->nParts);
    appendBytes(v, &t->root, sizeof(t->root));
    for (const Part *p : t->data->parts) appendBytes(v, &p->gen, sizeof(p->gen));
}

// A part's model values (as packed into the parameter image) and settings.
static void partSignature(const Tree *t, int p, std::vector<char> &v)
{
    const TreeDev &dv = t->dev;
    const ModelPart &mp = t->model->parts[p];
    const char *h = (const char *)dv.hImg.ptr;
    v.clear();
    appendBytes(v, h + dv.oComps[p], sizeof(double) * (size_t)mp.nComps * mp.dim);
    appendBytes(v, h + dv.oR[p], sizeof(double) * (size_t)mp.nRMatrices * mp.dim * mp.dim);
    appendBytes(v, h + dv.oG[p], sizeof(double) * (size_t)mp.nGdasrvs);
    appendBytes(v, &mp.pInvar, sizeof(mp.pInvar));
    appendBytes(v, &mp.relRate, sizeof(mp.relRate));
    appendBytes(v, &mp.nCat, sizeof(mp.nCat));
}

// Host side of one batched evaluation: every tree's parameter image and the
// combined descriptors.  Returns whether the launch shape changed.
static int batchPack(Batch *b, bool &reshape)
{
    char *h = (char *)b->hImg.ptr;
    char *g = (char *)b->dImg.ptr;
    PmatPart *desc = (PmatPart *)(h + b->oDesc);
    PruneJob *jobs = (PruneJob *)(h + b->oJobs);
    int2 *eig = (int2 *)(h + b->oEig);
    int2 *gam = (int2 *)(h + b->oGam);
    int *counts = (int *)(h + b->oCounts);
    int *prefix = (int *)(h + b->oPrefix);
    int nDescAll = 0, nE = 0, nG = 0, nD = 0, nDcap = 0, maxDim = 0;
    reshape = false;
    for (size_t ti = 0; ti < b->trees.size(); ti++) {
        Tree *t = b->trees[ti];
        TreeDev &dv = t->dev;
        RET(validateModel(t, -1));
        if (dv.progDirty) RET(refreshProgram(t));
        for (size_t gi = 0; gi < b->groups.size(); gi++) {   // every tree tiled like the batch's launch
            PruneGroup &tg = dv.groups[gi];
            if (tg.shape == b->groups[gi].shape) continue;
            RET(waitImage(t));
            tg.shape = b->groups[gi].shape;
            tg.smem = pruneSmemBytes(tg.dim, tg.nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, tg.shape,
                                     dv.nClade, dv.nDeck, dv.nRow);
            if (tg.smem > 227 * 1024)
                return setError(P4G_EUNSUPPORTED, "batch: tree %d does not fit the batch's tile shape %d",
                                (int)ti, tg.shape);
            RET(layoutBlocks(t));
        }
        int nDesc, tG, tE, tD, md;
        RET(waitImage(t));   // an earlier single evaluation has read the image
        RET(packParams(t, -1, nDesc, tG, tE, tD, md));
        const char *th = (const char *)dv.hImg.ptr;
        const PmatPart *tdesc = (const PmatPart *)(th + dv.oPmat);
        const int2 *te = (const int2 *)(th + dv.oEigTasks);
        const int2 *tg = (const int2 *)(th + dv.oGammaTasks);
        // which parts need evaluating: any whose inputs changed since this
        // batch last evaluated them (all of them when the tree's changed), and
        // any with an eigensystem or Gamma task (descriptor d is part d)
        const size_t j0 = ti * (size_t)b->nParts;
        treeSignature(t, b->pendTreeSig[ti]);
        const bool treeSame = !b->forceAll && !b->useClades && b->pendTreeSig[ti] == b->treeSig[ti];
        for (int p = 0; p < t->nParts; p++) {
            partSignature(t, p, b->pendPartSig[j0 + p]);
            b->dirty[j0 + p] = !(treeSame && b->lnlOk[j0 + p] && b->pendPartSig[j0 + p] == b->partSig[j0 + p]);
        }
        for (int k = 0; k < tE; k++) b->dirty[j0 + te[k].x] = 1;
        for (int k = 0; k < tG; k++) b->dirty[j0 + tg[k].x] = 1;
        // the dirty parts' descriptors, compacted; their P-deck task ranges
        std::vector<int> gdesc(nDesc, -1);
        for (int d = 0; d < nDesc; d++) {
            const ModelPart &mp = t->model->parts[d];
            nDcap += pdeckTasks(mp.dim, t->nNodes, mp.nCat);
            if (!b->dirty[j0 + d]) continue;
            gdesc[d] = nDescAll;
            desc[nDescAll] = tdesc[d];
            prefix[nDescAll] = nD;
            nD += pdeckTasks(mp.dim, t->nNodes, mp.nCat);
            nDescAll++;
        }
        for (int k = 0; k < tE; k++) eig[nE + k] = make_int2(gdesc[te[k].x], te[k].y);
        for (int k = 0; k < tG; k++) gam[nG + k] = make_int2(gdesc[tg[k].x], tg[k].y);
        const PruneJob *tj = (const PruneJob *)(th + dv.oJobs);
        for (int p = 0; p < t->nParts; p++) {
            PruneJob J = tj[p];
            J.out = b->dOut.as<double>() + ti * b->nParts + p;
            if (!b->dirty[j0 + p]) J.nCherry = 0;   // no cherry tables for a part left out
            jobs[ti * b->nParts + p] = J;
        }
        nE += tE;
        nG += tG;
        maxDim = std::max(maxDim, md);
        for (size_t gi = 0; gi < b->groups.size(); gi++)
            b->groups[gi].smem = std::max(b->groups[gi].smem, dv.groups[gi].smem);
        dv.haveParams = true;
    }
    counts[0] = nE;
    counts[1] = nG;
    counts[2] = nD;         // live P-deck tasks
    counts[3] = nDescAll;   // live descriptors
    // tile list: a fixed region per group holding the tiles of every tree, of
    // which the dirty parts' tiles are written; the live count per group
    BlockDesc *blk = (BlockDesc *)(h + b->oBlocks);
    int base = 0;
    for (size_t gi = 0; gi < b->groups.size(); gi++) {
        PruneGroup &G = b->groups[gi];
        int cap = 0;
        for (size_t ti = 0; ti < b->trees.size(); ti++) cap += b->trees[ti]->dev.groups[gi].nBlk;
        if (cap != b->groupCap[gi]) reshape = true;
        b->groupCap[gi] = cap;
        G.blk0 = base;
        int nb = base;
        for (size_t ti = 0; ti < b->trees.size(); ti++) {
            const TreeDev &dv = b->trees[ti]->dev;
            const PruneGroup &tg = dv.groups[gi];
            for (int k = 0; k < tg.nBlk; k++) {
                BlockDesc d = dv.blocks[tg.blk0 + k];
                if (!b->dirty[ti * (size_t)b->nParts + d.job]) continue;
                d.job += (int)ti * b->nParts;
                blk[nb++] = d;
            }
        }
        G.nBlk = cap;   // the launch's capacity
        counts[4 + gi] = nb - base;
        base += cap;
        if (G.smem > b->capturedSmem[gi]) reshape = true;
    }
    if (nDcap != b->nD || maxDim != b->maxDim) reshape = true;
    if (b->useClades) {   // the clade launches follow each tree's current clades
        std::vector<long long> v;
        for (Tree *t : b->trees) v.push_back(t->dev.cladeVersion);
        if (v != b->cladeVersions) {
            reshape = true;
            RET(cladeMerge(b->trees, b->dCladeJobs, b->dCladeBlocks, b->dCladeCounts, b->dCladeSrc,
                           b->cladeGroups, g_ctx.stream));
        }
        b->cladeVersions = v;
    }
    b->nD = nDcap;
    b->maxDim = maxDim;
    (void)g;
    return P4G_OK;
}

// The parameter images of the batch's trees and the batch's own image, each
// copied (ahead of the launch sequence, outside any graph) only when it
// differs from its last copy; branch lengths are not compared, since the
// P-deck kernel reads them from the trees' pinned host images.  An
// evaluation that changes only branch lengths copies nothing.
static int batchUpload(Batch *b)
{
    cudaStream_t s = g_ctx.stream;
    for (Tree *t : b->trees) {
        TreeDev &dv = t->dev;
        if (!imageDirty(t)) continue;
        P4G_CUDA(cudaMemcpyAsync(dv.dImg.ptr, dv.hImg.ptr, dv.imgBytes, cudaMemcpyHostToDevice, s));
        P4G_CUDA(cudaEventRecord(dv.imgFree, s));
        dv.shadow.assign((const char *)dv.hImg.ptr, (const char *)dv.hImg.ptr + dv.imgBytes);
        dv.cladeFresh = false;
    }
    const char *h = (const char *)b->hImg.ptr;
    if (b->shadow.size() != b->imgBytes || memcmp(b->shadow.data(), h, b->imgBytes) != 0) {
        P4G_CUDA(cudaMemcpyAsync(b->dImg.ptr, b->hImg.ptr, b->imgBytes, cudaMemcpyHostToDevice, s));
        b->shadow.assign(h, h + b->imgBytes);
    }
    return P4G_OK;
}

// The batch's kernels and result copy (its inputs copied by batchUpload).
static int batchEnqueue(Batch *b)
{
    cudaStream_t s = g_ctx.stream;
    const char *g = (const char *)b->dImg.ptr;
    RET(launchPmatDev((const PmatPart *)(g + b->oDesc), (const int2 *)(g + b->oEig), b->capE,
                      (const int2 *)(g + b->oGam), b->capG, (const int *)(g + b->oCounts),
                      (const int *)(g + b->oPrefix), b->capDesc, b->nD, b->maxDim, batchStatus(b), s));
    const PruneJob *dJobs = (const PruneJob *)(g + b->oJobs);
    const BlockDesc *dBlocks = (const BlockDesc *)(g + b->oBlocks);
    if (b->useClades && !b->cladeGroups.empty()) {   // every tree's clade tables in one launch per group
        const PruneJob *cj = b->dCladeJobs.as<PruneJob>();
        for (size_t gi = 0; gi < b->cladeGroups.size(); gi++) {
            const PruneGroup &G = b->cladeGroups[gi];
            RET(launchPrune(cj, b->dCladeBlocks.as<BlockDesc>() + G.blk0, G.nBlk, G.dim, G.nCat, G.smem, G.shape, s,
                            b->dCladeCounts.as<int>() + gi));
        }
    } else if (b->useClades) {   // every tree's clade tables, side by side (they read only the decks)
        if (b->side.size() != b->trees.size()) {
            for (size_t i = b->side.size(); i < b->trees.size(); i++) {
                cudaStream_t x;
                cudaEvent_t e;
                P4G_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
                P4G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                b->side.push_back(x);
                b->joined.push_back(e);
            }
            if (!b->forked) P4G_CUDA(cudaEventCreateWithFlags(&b->forked, cudaEventDisableTiming));
        }
        P4G_CUDA(cudaEventRecord(b->forked, s));
        for (size_t i = 0; i < b->trees.size(); i++) {
            P4G_CUDA(cudaStreamWaitEvent(b->side[i], b->forked, 0));
            RET(cladeLaunch(b->trees[i], b->side[i]));
            P4G_CUDA(cudaEventRecord(b->joined[i], b->side[i]));
            P4G_CUDA(cudaStreamWaitEvent(s, b->joined[i], 0));
        }
    }
    {   // cherry tables of every (tree, part); the launch shape uses the list
        // capacity, so a captured graph stays valid when topologies change
        const Tree *t0 = b->trees[0];
        long long work = 0;
        for (int p = 0; p < b->nParts; p++) {
            if (t0->dev.oCherryTab[p] == (size_t)-1) continue;
            work = std::max(work, (long long)t0->dev.capCherry * t0->model->parts[p].nCat);
        }
        RET(launchCherry(dJobs, (int)b->trees.size() * b->nParts, work, s));
    }
    // each group over its region's capacity; the live tile count (the parts
    // being evaluated) is read from device memory
    const int *dCounts = (const int *)(g + b->oCounts);
    for (size_t gi = 0; gi < b->groups.size(); gi++) {
        const PruneGroup &G = b->groups[gi];
        RET(launchPrune(dJobs, dBlocks + G.blk0, G.nBlk, G.dim, G.nCat, G.smem, G.shape, s, dCounts + 4 + gi));
    }
    P4G_CUDA(cudaMemcpyAsync(b->hOut.ptr, b->dOut.ptr, sizeof(double) * b->capDesc + sizeof(int),
                             cudaMemcpyDeviceToHost, s));
    return P4G_OK;
}

// Tile shapes of the batch: the single-tree choice is made for one tree's
// patterns; with every tree's tiles in one launch, occupancy (shared memory
// and registers per block) matters more, so each group's shapes are timed on
// the whole batched evaluation (one plain run, then three timed ones) and the
// fastest kept for every tree of the batch.
static int batchTune(Batch *b)
{
    b->tuned = true;
    if (!g_autotune) return P4G_OK;
    b->forceAll = true;   // every timed run evaluates every part
    struct Restore {
        Batch *b;
        ~Restore() { b->forceAll = false; }
    } restore{b};
    cudaStream_t s = g_ctx.stream;
    cudaEvent_t e0, e1;
    P4G_CUDA(cudaEventCreate(&e0));
    P4G_CUDA(cudaEventCreate(&e1));
    for (size_t gi = 0; gi < b->groups.size(); gi++) {
        const int dim = b->groups[gi].dim, nCat = b->groups[gi].nCat;
        const int keep = b->groups[gi].shape;
        int best = keep;
        float bestMs = 1e30f;
        for (int sh = 0; sh < pruneNumShapes(dim); sh++) {
            if (!pruneShapeValid(dim, nCat, sh)) continue;
            bool fits = true;
            for (Tree *t : b->trees) {
                TreeDev &dv = t->dev;
                RET(waitImage(t));
                dv.groups[gi].shape = sh;
                dv.groups[gi].smem = pruneSmemBytes(dim, nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, sh,
                                                    dv.nClade, dv.nDeck, dv.nRow);
                if (dv.groups[gi].smem > 227 * 1024) fits = false;
                RET(layoutBlocks(t));
            }
            if (!fits) continue;
            b->groups[gi].shape = sh;
            b->groups[gi].smem = 0;
            bool reshape = false;
            RET(batchPack(b, reshape));
            RET(batchUpload(b));
            if (batchEnqueue(b) != P4G_OK) continue;   // e.g. a launch the shape cannot make
            P4G_CUDA(cudaEventRecord(e0, s));
            for (int r = 0; r < 3; r++) RET(batchEnqueue(b));
            P4G_CUDA(cudaEventRecord(e1, s));
            P4G_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            P4G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < bestMs) {
                bestMs = ms;
                best = sh;
            }
        }
        for (Tree *t : b->trees) {
            TreeDev &dv = t->dev;
            RET(waitImage(t));
            dv.groups[gi].shape = best;
            dv.groups[gi].smem = pruneSmemBytes(dim, nCat, dv.nProg, t->nNodes, t->data->nTax, dv.nSlots, best,
                                                dv.nClade, dv.nDeck, dv.nRow);
            RET(layoutBlocks(t));
        }
        b->groups[gi].shape = best;
        b->groups[gi].smem = 0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    P4G_CUDA(cudaStreamSynchronize(s));
    return P4G_OK;
}

extern "C" int p4g_batchLogLike(p4g_batch *bb, double *lnL)
{
    Batch *b = B_(bb);
    if (!b || !lnL) return setError(P4G_EINVAL, "batchLogLike: null argument");
    if (!b->ready) RET(batchPrepare(b));
    if (!b->tuned) RET(batchTune(b));
    bool reshape = false;
    RET(batchPack(b, reshape));
    RET(batchUpload(b));
    cudaStream_t s = g_ctx.stream;
    if (b->useGraph) {
        if (reshape || !b->exec) {
            if (b->exec) cudaGraphExecDestroy(b->exec);
            if (b->graph) cudaGraphDestroy(b->graph);
            b->exec = nullptr;
            b->graph = nullptr;
            // launch attributes (shared memory opt-in, occupancy) are set up
            // outside the capture by one plain run of the sequence
            RET(batchEnqueue(b));
            P4G_CUDA(cudaStreamSynchronize(s));
            P4G_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int rc = batchEnqueue(b);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(s, &graph);
            if (rc != P4G_OK) return rc;
            if (e != cudaSuccess) return setError(P4G_ECUDA, "graph capture: %s", cudaGetErrorString(e));
            b->graph = graph;
            P4G_CUDA(cudaGraphInstantiate(&b->exec, graph, 0));
            for (size_t gi = 0; gi < b->groups.size(); gi++) b->capturedSmem[gi] = b->groups[gi].smem;
        }
        P4G_CUDA(cudaGraphLaunch(b->exec, s));
    } else {
        RET(batchEnqueue(b));
    }
    P4G_CUDA(cudaStreamSynchronize(s));
    const double *out = b->hOut.as<double>();
    const size_t nJ = b->trees.size() * (size_t)b->nParts;
    int status = *(const int *)((const char *)b->hOut.ptr + sizeof(double) * b->capDesc);
    if (status) {
        cudaMemsetAsync(batchStatus(b), 0, sizeof(int), s);
        for (Tree *t : b->trees) t->dev.cacheValid = false;
        b->lnlOk.assign(nJ, 0);
        return setError(P4G_ENUMERIC, "setPrams: %s did not converge", (status & 1) ? "discrete gamma" : "eigensystem");
    }
    for (size_t k = 0; k < nJ; k++)
        if (b->dirty[k] && out[k] != out[k]) {
            b->lnlOk.assign(nJ, 0);
            return setError(P4G_ETIMEOUT, "pruning: a device-side check failed (a tensor-core completion wait gave up, or a clade-table index was out of range)");
        }
    // the evaluated parts' lnLs and inputs become the cache; the others keep theirs
    for (size_t k = 0; k < nJ; k++) {
        if (!b->dirty[k]) continue;
        b->lnlCache[k] = out[k];
        b->lnlOk[k] = 1;
        b->partSig[k].swap(b->pendPartSig[k]);
    }
    for (size_t ti = 0; ti < b->trees.size(); ti++) {
        b->treeSig[ti].swap(b->pendTreeSig[ti]);
        Tree *t = b->trees[ti];
        double sum = 0.0;
        for (int p = 0; p < b->nParts; p++) {
            const double v = b->lnlCache[ti * b->nParts + p];
            t->partLikes[p] = v;
            sum += v;
        }
        t->logLike = sum;
        lnL[ti] = sum;
    }
    return P4G_OK;
}
