/*
 * ref_driver.c -- TEST INFRASTRUCTURE (oracle), never part of the product.
 *
 * A flat C entry layer over the reference p4 likelihood core (Pf/*.c), which
 * oracle/Makefile compiles from the reference source tree into
 * oracle/_ref/libp4ref.so.  The reference normally receives its inputs through
 * the CPython module Pf/pfmodule.c; that module needs GSL and nlopt, which are
 * absent, so this driver fills the reference's own structs (Pf/pftypes.h) the
 * way the pfmodule wrappers do and then calls the reference functions:
 *
 *   newPart / pokeEquatesTable / pokeSequences / makePatterns /
 *   setGlobalInvarSitesVec              Pf/part.c:15,279,127,317,716
 *   p4_newModel / p4_newModelPart /
 *   p4_newRMatrix                       Pf/p4_model.c:11,77,345
 *   p4_newTree / p4_newNode             Pf/p4_tree.c:15, Pf/p4_node.c:10
 *   p4_setPrams / p4_treeLogLike        Pf/p4_tree.c:207,868
 *
 * Comp and Gdasrv structs alias caller buffers, as p4_newComp and
 * p4_newGdasrv do with numpy data (Pf/p4_model.c:328-340, 490-511).  Gdasrvs
 * are marked free so that p4_setPramsPart recomputes the discrete-gamma rates
 * with the reference's DiscreteGamma (Pf/p4_tree.c:235-255).  R matrices use
 * spec RMATRIX_SPECIFIED and are poked into bigR symmetrically as
 * pf_p4_setRMatrixBigR does (Pf/pfmodule.c:1720-1735).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "pftypes.h"
#include "defines.h"
#include "part.h"
#include "p4_model.h"
#include "p4_tree.h"
#include "p4_node.h"
#include <nlopt.h>

void p4_newtAndBrentPowellOpt(p4_tree *aTree);

typedef struct {
    data     *d;
    p4_model *m;
    p4_tree  *t;
    int       nParts;
    int      *preOrder;
    int      *postOrder;
    double   *partLikes;
    int       passLimit;
    int      *rMatrixNormalizeTo1;
    double    bounds[16];
    int     **bqet;           /* per part, nComps*nR ints */
    int      *nComps;
    int      *nR;
} ref_handle;

void *ref_new(int nTax, int nParts)
{
    ref_handle *h = calloc(1, sizeof(ref_handle));
    int i;
    h->nParts = nParts;
    h->d = calloc(1, sizeof(data));
    h->d->nTax = nTax;
    h->d->nParts = nParts;
    h->d->parts = calloc(nParts, sizeof(part *));
    h->rMatrixNormalizeTo1 = calloc(1, sizeof(int));
    h->rMatrixNormalizeTo1[0] = 1;
    /* var.py defaults: PINVAR_MIN/MAX, KAPPA, GAMMA_SHAPE, PIVEC, RATE, RELRATE, BRLEN */
    {
        double b[14] = {0.0, 0.99, 1e-6, 100.0, 0.1, 300.0, 1e-13, 0.999,
                        1e-13, 0.9999999, 1e-8, 1e8, 1e-8, 3.0};
        for (i = 0; i < 14; i++) h->bounds[i] = b[i];
    }
    h->m = p4_newModel(nParts, nParts > 1, 0, 0, 1, h->rMatrixNormalizeTo1,
                       &h->bounds[0], &h->bounds[1], &h->bounds[2], &h->bounds[3],
                       &h->bounds[4], &h->bounds[5], &h->bounds[6], &h->bounds[7],
                       &h->bounds[8], &h->bounds[9], &h->bounds[10], &h->bounds[11],
                       &h->bounds[12], &h->bounds[13]);
    h->bqet = calloc(nParts, sizeof(int *));
    h->nComps = calloc(nParts, sizeof(int));
    h->nR = calloc(nParts, sizeof(int));
    return h;
}

/* The reference's own 20x20 exchangeability matrix for an RMatrix spec, as
 * p4_newRMatrix fills it (Pf/p4_model.c:345-450), into out[400] row-major:
 * the pin for the library's table of empirical protein matrices. */
int ref_getBigR(int spec, double *out)
{
    ref_handle *h = ref_new(1, 1);
    int i, j;
    h->bqet[0] = calloc(1, sizeof(int));
    h->bqet[0][0] = 1;
    p4_newModelPart(h->m, 0, 20, 1, 1, 0, 1, 0, h->bqet[0]);
    p4_newRMatrix(h->m, 0, 0, 0, spec);
    for (i = 0; i < 20; i++)
        for (j = 0; j < 20; j++) out[i * 20 + j] = h->m->parts[0]->rMatrices[0]->bigR[i][j];
    return 0;
}

/* One data part: seqs is nTax*nChar characters, row-major by taxon.
 * equatesTable is nEquates*dim characters '0'/'1' (p4/alignment.py:5838-5862). */
int ref_part(void *vh, int pNum, int dim, int nChar, const char *symbols,
             const char *equateSymbols, int nEquates, const char *equatesTable,
             const char *seqs)
{
    ref_handle *h = vh;
    part *p = newPart(h->d->nTax, nChar, (char *)equateSymbols, nEquates, (char *)symbols, dim);
    if (!p) return -1;
    if (nEquates > 0) pokeEquatesTable(p, (char *)equatesTable);
    pokeSequences(p, (char *)seqs);
    makePatterns(p);
    setGlobalInvarSitesVec(p);
    p->data = h->d;
    h->d->parts[pNum] = p;
    return p->nPatterns;
}

int ref_nPatterns(void *vh, int pNum) { return ((ref_handle *)vh)->d->parts[pNum]->nPatterns; }

/* patterns out: nTax*nPatterns ints (taxon-major), counts: nPatterns,
 * seqPosIndex: nChar, invarVec: nPatterns, invarArray: dim*nPatterns. */
void ref_getPatterns(void *vh, int pNum, int *patterns, int *counts, int *seqPosIndex,
                     int *invarVec, int *invarArray)
{
    ref_handle *h = vh;
    part *p = h->d->parts[pNum];
    int t, i, s;
    for (t = 0; t < p->nTax; t++)
        for (i = 0; i < p->nPatterns; i++) patterns[t * p->nPatterns + i] = p->patterns[t][i];
    for (i = 0; i < p->nPatterns; i++) counts[i] = p->patternCounts[i];
    for (i = 0; i < p->nChar; i++) seqPosIndex[i] = p->sequencePositionPatternIndex[i];
    for (i = 0; i < p->nPatterns; i++) invarVec[i] = p->globalInvarSitesVec[i];
    for (s = 0; s < p->dim; s++)
        for (i = 0; i < p->nPatterns; i++) invarArray[s * p->nPatterns + i] = p->globalInvarSitesArray[s][i];
}

/* comps: nComps*dim; rmats: nR*dim*dim (full symmetric bigR, diagonal ignored);
 * gammaShapes: nG values (caller-owned, aliased); pInvar, relRate scalars. */
int ref_modelPart(void *vh, int pNum, int dim, int nComps, double *comps, int nR,
                  const double *rmats, int nG, double *gammaShapes, double *gammaFreqs,
                  double *gammaRates, int nCat, double pInvar, double relRate)
{
    ref_handle *h = vh;
    p4_modelPart *mp;
    int i, r, a, b;
    h->bqet[pNum] = calloc(nComps * nR, sizeof(int));
    for (i = 0; i < nComps * nR; i++) h->bqet[pNum][i] = 1;
    h->nComps[pNum] = nComps;
    h->nR[pNum] = nR;
    p4_newModelPart(h->m, pNum, dim, nComps, nR, nG, nCat, 0, h->bqet[pNum]);
    mp = h->m->parts[pNum];
    for (i = 0; i < nComps; i++) {
        p4_comp *c = malloc(sizeof(p4_comp));
        c->free = 1;
        c->val = comps + (size_t)i * dim;
        mp->comps[i] = c;
    }
    for (r = 0; r < nR; r++) {
        p4_newRMatrix(h->m, pNum, r, 1, RMATRIX_SPECIFIED);
        for (a = 0; a < dim; a++)
            for (b = a + 1; b < dim; b++) {
                double v = rmats[(size_t)r * dim * dim + a * dim + b];
                mp->rMatrices[r]->bigR[a][b] = v;
                mp->rMatrices[r]->bigR[b][a] = v;
            }
    }
    for (i = 0; i < nG; i++) {
        p4_gdasrv *g = malloc(sizeof(p4_gdasrv));
        g->free = 1;
        g->nCat = nCat;
        g->val = gammaShapes + i;
        g->freqs = gammaFreqs + (size_t)i * nCat;
        g->rates = gammaRates + (size_t)i * nCat;
        mp->gdasrvs[i] = g;
    }
    mp->pInvar->val[0] = pInvar;
    mp->relRate[0] = relRate;
    return 0;
}

/* Tree: relations as node numbers (-1 = none); compNums etc. are nNodes*nParts
 * (node-major).  postOrder/preOrder are node-number arrays of length nNodes. */
int ref_tree(void *vh, int nNodes, int nLeaves, int root, const int *parent,
             const int *leftChild, const int *sibling, const int *seqNum,
             const int *isLeaf, const double *brLen, const int *compNums,
             const int *rMatrixNums, const int *gdasrvNums, const int *preOrder,
             const int *postOrder)
{
    ref_handle *h = vh;
    int i, p;
    h->preOrder = malloc(nNodes * sizeof(int));
    h->postOrder = malloc(nNodes * sizeof(int));
    memcpy(h->preOrder, preOrder, nNodes * sizeof(int));
    memcpy(h->postOrder, postOrder, nNodes * sizeof(int));
    h->partLikes = calloc(h->nParts, sizeof(double));
    h->passLimit = 50;
    h->t = p4_newTree(nNodes, nLeaves, h->preOrder, h->postOrder, h->partLikes, h->d, h->m,
                      &h->passLimit);
    for (i = 0; i < nNodes; i++) p4_newNode(i, h->t, seqNum[i], isLeaf[i], 1);
    for (i = 0; i < nNodes; i++) {
        p4_node *n = h->t->nodes[i];
        n->parent = parent[i] >= 0 ? h->t->nodes[parent[i]] : NULL;
        n->leftChild = leftChild[i] >= 0 ? h->t->nodes[leftChild[i]] : NULL;
        n->sibling = sibling[i] >= 0 ? h->t->nodes[sibling[i]] : NULL;
        n->brLen[0] = brLen[i];
        for (p = 0; p < h->nParts; p++) {
            n->compNums[p] = compNums[i * h->nParts + p];
            n->rMatrixNums[p] = rMatrixNums[i * h->nParts + p];
            n->gdasrvNums[p] = gdasrvNums[i * h->nParts + p];
        }
    }
    h->t->root = h->t->nodes[root];
    return 0;
}

void ref_setBrLen(void *vh, int node, double len) { ((ref_handle *)vh)->t->nodes[node]->brLen[0] = len; }

/* What Tree.setCStuff pushes for a new topology (p4/tree.py:9322-9377,
 * pf_p4_setNodeRelation / pf_p4_setTreeRoot, Pf/pfmodule.c:1907-1958): every
 * node's relations as node numbers (-1 = none), the root, and the pre- and
 * post-order arrays the tree reads (p4 aliases them from numpy). */
void ref_setTopology(void *vh, const int *parent, const int *leftChild, const int *sibling, int root,
                     const int *preOrder, const int *postOrder)
{
    ref_handle *h = vh;
    int i, n = h->t->nNodes;
    for (i = 0; i < n; i++) {
        p4_node *nd = h->t->nodes[i];
        nd->parent = parent[i] >= 0 ? h->t->nodes[parent[i]] : NULL;
        nd->leftChild = leftChild[i] >= 0 ? h->t->nodes[leftChild[i]] : NULL;
        nd->sibling = sibling[i] >= 0 ? h->t->nodes[sibling[i]] : NULL;
    }
    h->t->root = h->t->nodes[root];
    memcpy(h->preOrder, preOrder, n * sizeof(int));
    memcpy(h->postOrder, postOrder, n * sizeof(int));
}

/* Every non-root node's branch length (brLens: nNodes values). */
void ref_setBrLens(void *vh, const double *brLens)
{
    ref_handle *h = vh;
    int i;
    for (i = 0; i < h->t->nNodes; i++)
        if (h->t->nodes[i] != h->t->root) h->t->nodes[i]->brLen[0] = brLens[i];
}

/* Model values of one part as Model.setCStuff leaves them (p4/model.py:
 * 153-207): comps (nComps x dim, written through the comps' value pointers,
 * which p4 aliases), R matrices as their upper triangles (nR x dim(dim-1)/2,
 * poked into bigR symmetrically as pf_p4_setRMatrixBigR does), gamma shapes
 * (nG), pInvar and relRate.  The next p4_setPrams recomputes everything. */
void ref_setModelValues(void *vh, int pNum, const double *comps, const double *rUpper, const double *gammaShapes,
                        double pInvar, double relRate)
{
    ref_handle *h = vh;
    p4_modelPart *mp = h->m->parts[pNum];
    int dim = mp->dim, i, r, a, b, k;
    for (i = 0; i < mp->nComps; i++) memcpy(mp->comps[i]->val, comps + (size_t)i * dim, dim * sizeof(double));
    for (r = 0; r < mp->nRMatrices; r++) {
        k = 0;
        for (a = 0; a < dim - 1; a++)
            for (b = a + 1; b < dim; b++) {
                double v = rUpper[(size_t)r * (dim * (dim - 1) / 2) + k++];
                mp->rMatrices[r]->bigR[a][b] = v;
                mp->rMatrices[r]->bigR[b][a] = v;
            }
    }
    for (i = 0; i < mp->nGdasrvs; i++) mp->gdasrvs[i]->val[0] = gammaShapes[i];
    mp->pInvar->val[0] = pInvar;
    mp->relRate[0] = relRate;
}

/* p4_setPrams(-1) + p4_treeLogLike, as Tree.calcLogLike does (p4/tree.py:9400-9412). */
double ref_logLike(void *vh, double *partLikesOut)
{
    ref_handle *h = vh;
    double lnL;
    int p;
    p4_setPrams(h->t);
    lnL = p4_treeLogLike(h->t, 0);
    if (partLikesOut)
        for (p = 0; p < h->nParts; p++) partLikesOut[p] = h->partLikes[p];
    return lnL;
}

/* p4's allBrLens evaluation (p4/chain.py:733-747): every non-root node gets
 * its new branch length and p4_calculateBigPDecks (eigensystems from the last
 * setPrams kept), then every internal node's conditional likelihoods in
 * post-order and each part's log-sum (p4_treeLogLike). */
double ref_allBrLensLogLike(void *vh, const double *brLens)
{
    ref_handle *h = vh;
    int i;
    for (i = 0; i < h->t->nNodes; i++) {
        p4_node *n = h->t->nodes[i];
        if (n == h->t->root) continue;
        n->brLen[0] = brLens[i];
        p4_calculateBigPDecks(n);
    }
    return p4_treeLogLike(h->t, 0);
}

/* A per-part proposal's evaluation (p4/chain.py:316-556, e.g. allCompsDir,
 * gdasrv): p4_setPramsPart, every internal node's conditional likelihoods of
 * that part in post-order, then the part's log-sum.  Returns its lnL. */
double ref_partUpdate(void *vh, int pNum)
{
    ref_handle *h = vh;
    int j;
    p4_setPramsPart(h->t, pNum);
    for (j = 0; j < h->t->nNodes; j++) {
        int i = h->t->postOrder[j];
        if (i == NO_ORDER) continue;
        p4_node *n = h->t->nodes[i];
        if (!n->isLeaf || n == h->t->root) p4_setConditionalLikelihoodsOfInternalNodePart(n, pNum);
    }
    return p4_partLogLike(h->t, h->d->parts[pNum], pNum, 0);
}

/* Only the pruning + root reduction (P decks already set by a previous call). */
double ref_logLikeNoSetPrams(void *vh) { return p4_treeLogLike(((ref_handle *)vh)->t, 0); }

/* Per-site likelihoods (p4_partLogLike with getSiteLikes; Pf/p4_tree.c:1015-1021). */
double ref_siteLikes(void *vh, int pNum, double *out)
{
    ref_handle *h = vh;
    part *dp = h->d->parts[pNum];
    double lnL = p4_partLogLike(h->t, dp, pNum, 1);
    memcpy(out, dp->siteLikes, dp->nChar * sizeof(double));
    return lnL;
}

/* p4_partLogLikeSiteRates (Pf/p4_tree.c:1383-1627) on the root CLs of the
   last evaluation: per site, the posterior mean rate and the most likely
   gamma category.  The part must have exactly one gdasrv. */
double ref_siteRates(void *vh, int pNum, double *siteRates, int *gammaCats)
{
    ref_handle *h = vh;
    part *dp = h->d->parts[pNum];
    double work[64];
    return p4_partLogLikeSiteRates(h->t, dp, pNum, 0, siteRates, gammaCats, work);
}

/* bigPDecks[pNum][cat] of a node, dim*dim row-major (row = parent state). */
void ref_getPDeck(void *vh, int node, int pNum, int cat, double *out)
{
    ref_handle *h = vh;
    int dim = h->m->parts[pNum]->dim, i, j;
    for (i = 0; i < dim; i++)
        for (j = 0; j < dim; j++) out[i * dim + j] = h->t->nodes[node]->bigPDecks[pNum][cat][i][j];
}

/* cl[pNum][cat][state][pattern] of an internal node, cat-major. */
void ref_getCL(void *vh, int node, int pNum, double *out)
{
    ref_handle *h = vh;
    int dim = h->m->parts[pNum]->dim, nCat = h->m->parts[pNum]->nCat;
    int np = h->d->parts[pNum]->nPatterns, c, s, k;
    for (c = 0; c < nCat; c++)
        for (s = 0; s < dim; s++)
            for (k = 0; k < np; k++)
                out[((size_t)c * dim + s) * np + k] = h->t->nodes[node]->cl[pNum][c][s][k];
}

/* ---- draws: Pf/p4_treeSim.c, run as the reference's own code -------------
 *
 * p4_simulate draws its uniforms from GSL (gsl_rng_uniform, the only GSL call
 * in that file).  GSL is absent, so the stub header declares the function and
 * this driver defines it: the n-th call returns the n-th value of the
 * Philox4x32-10 stream of ref_rngSeed (Salmon et al., SC 2011: ten rounds,
 * multipliers 0xD2511F53 / 0xCD9E8D57, Weyl keys 0x9E3779B9 / 0xBB67AE85,
 * first output word times 2^-32), or of a caller's array when one is set.
 * ref_rngCalls counts the calls. */
static unsigned long long ref_rngSeed = 0, ref_rngCalls = 0;
static const double *ref_rngArray = NULL;

static double ref_philox(unsigned long long seed, unsigned long long n)
{
    unsigned int c0 = (unsigned int)n, c1 = (unsigned int)(n >> 32), c2 = 0, c3 = 0;
    unsigned int k0 = (unsigned int)seed, k1 = (unsigned int)(seed >> 32);
    int r;
    for (r = 0; r < 10; r++) {
        unsigned long long p0 = 0xD2511F53ull * c0, p1 = 0xCD9E8D57ull * c2;
        unsigned int n0 = (unsigned int)(p1 >> 32) ^ c1 ^ k0, n2 = (unsigned int)(p0 >> 32) ^ c3 ^ k1;
        c1 = (unsigned int)p1;
        c3 = (unsigned int)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return (double)c0 * (1.0 / 4294967296.0);
}

double ref_philoxUniform(unsigned long long seed, unsigned long long n) { return ref_philox(seed, n); }

double gsl_rng_uniform(const gsl_rng *g)
{
    (void)g;
    double u = ref_rngArray ? ref_rngArray[ref_rngCalls] : ref_philox(ref_rngSeed, ref_rngCalls);
    ref_rngCalls++;
    return u;
}

/* p4_simulate(t, NULL, rng) (Pf/p4_treeSim.c:14-590) after ref_logLike has set
 * the P decks; the leaves' sequences (per part nTax x nChar, parts
 * concatenated) go to seqsOut.  Returns the number of uniforms drawn.  The
 * handle's alignment is the simulated one afterwards. */
long long ref_simulate(void *vh, unsigned long long seed, const double *uniforms, int *seqsOut)
{
    ref_handle *h = vh;
    size_t o = 0;
    int p, i, j;
    ref_rngSeed = seed;
    ref_rngCalls = 0;
    ref_rngArray = uniforms;
    p4_simulate(h->t, NULL, NULL);
    ref_rngArray = NULL;
    for (p = 0; p < h->nParts; p++) {
        part *dp = h->d->parts[p];
        for (i = 0; i < dp->nTax; i++)
            for (j = 0; j < dp->nChar; j++) seqsOut[o++] = dp->sequences[i][j];
    }
    return (long long)ref_rngCalls;
}

/* p4_simulate(t, refTree, rng) (Pf/p4_treeSim.c:223-284) after ref_logLike
 * on both handles: every site's root state and category drawn from refTree's
 * root posterior by p4_drawAncState with libc random() seeded with
 * libcSeed (the uniforms it uses, one per site of every part in part
 * order, go to libcUniformsOut), then the mutation loop from the GSL stream
 * (Philox of seed, or the caller's array).  seqsOut as ref_simulate.
 * Returns the number of GSL uniforms drawn. */
long long ref_simulateRef(void *vsim, void *vref, unsigned int libcSeed, double *libcUniformsOut,
                          unsigned long long seed, const double *uniforms, int *seqsOut)
{
    ref_handle *hs = vsim, *hr = vref;
    size_t o = 0, n = 0;
    int p, i, j;
    for (p = 0; p < hr->nParts; p++) {
        if (hr->m->parts[p]->pInvar->val[0] > 0.0) hr->m->parts[p]->pInvar->free = 1;
        n += hr->d->parts[p]->nChar;
    }
    srandom(libcSeed);
    for (o = 0; o < n; o++) libcUniformsOut[o] = (double)random() / ((double)(RAND_MAX) + 1.0);
    srandom(libcSeed);
    ref_rngSeed = seed;
    ref_rngCalls = 0;
    ref_rngArray = uniforms;
    p4_simulate(hs->t, hr->t, NULL);
    ref_rngArray = NULL;
    o = 0;
    for (p = 0; p < hs->nParts; p++) {
        part *dp = hs->d->parts[p];
        for (i = 0; i < dp->nTax; i++)
            for (j = 0; j < dp->nChar; j++) seqsOut[o++] = dp->sequences[i][j];
    }
    return (long long)ref_rngCalls;
}

/* Tree.ancestralStateDraw's loop (p4/tree.py:9652-9670) for one part on the
 * root CLs of the last evaluation: p4_drawAncStateP per site.  The reference
 * draws with libc random(); srandom(seed) first, and the uniforms it used
 * (random() / (RAND_MAX + 1.0), one per site) are recorded to uniformsOut by
 * replaying the same sequence.  draws: nChar x 4. */
void ref_drawAncStates(void *vh, int pNum, unsigned int seed, double *uniformsOut, int *draws)
{
    ref_handle *h = vh;
    part *dp = h->d->parts[pNum];
    int i;
    if (h->m->parts[pNum]->pInvar->val[0] > 0.0) h->m->parts[pNum]->pInvar->free = 1;
    srandom(seed);
    for (i = 0; i < dp->nChar; i++) uniformsOut[i] = (double)random() / ((double)(RAND_MAX) + 1.0);
    srandom(seed);
    for (i = 0; i < dp->nChar; i++) p4_drawAncStateP(h->t, pNum, i, draws + 4 * i);
}

/* ---- Newton branch lengths: Pf/p4_treeNewt.c, the reference's own code ----
 * p4_newtSetup (cl2 and derivative decks), then p4_newtAround(eps, delta) as
 * p4_newtAndBrentPowellOpt runs it for a model with no free parameters
 * (Pf/p4_treeOpt.c:1207-1212: (1, 10), (0.1, 1), (0.01, 0.1), (1e-5, 1e-7)).
 * The P decks must be set (ref_logLike first).  Returns the final lnL;
 * brLensOut (nNodes) receives every node's branch length. */
double ref_newtOptimize(void *vh, int nCalls, const double *eps, const double *delta, double *brLensOut)
{
    ref_handle *h = vh;
    int k;
    p4_newtSetup(h->t);
    for (k = 0; k < nCalls; k++) p4_newtAround(h->t, eps[k], delta[k]);
    for (k = 0; k < h->t->nNodes; k++) brLensOut[k] = h->t->nodes[k]->brLen[0];
    return p4_treeLogLike(h->t, 0);
}

/* ---- model-parameter optimisation: Pf/p4_treeOpt.c, the reference's own --
 * p4_newtAndBrentPowellOpt (Newton branch lengths alternating with praxis
 * over the free model parameters, Pf/p4_treeOpt.c:1182-1392).  Which values
 * are free is set per part (every comp, every R matrix, every gdasrv and
 * pInvar) and the model's nFreePrams counted as p4_windUpParameters counts
 * them (Pf/p4_treeOpt.c:19-115).  The P decks must be set (ref_logLike
 * first).  Returns the final lnL; brLensOut (nNodes) and, per part, the
 * values are read back by the caller through its aliased buffers. */
void ref_setFree(void *vh, int pNum, int comps, int rMatrices, int gdasrvs, int pInvar)
{
    ref_handle *h = vh;
    p4_modelPart *mp = h->m->parts[pNum];
    int i;
    for (i = 0; i < mp->nComps; i++) mp->comps[i]->free = comps;
    for (i = 0; i < mp->nRMatrices; i++) mp->rMatrices[i]->free = rMatrices;
    for (i = 0; i < mp->nGdasrvs; i++) mp->gdasrvs[i]->free = gdasrvs;
    mp->pInvar->free = pInvar;
}

double ref_optimize(void *vh, double *brLensOut, double *rUpperOut)
{
    ref_handle *h = vh;
    int p, i, n = 0, k;
    for (p = 0; p < h->nParts; p++) {
        p4_modelPart *mp = h->m->parts[p];
        for (i = 0; i < mp->nComps; i++) n += mp->comps[i]->free ? mp->dim - 1 : 0;
        for (i = 0; i < mp->nRMatrices; i++) n += mp->rMatrices[i]->free ? mp->dim * (mp->dim - 1) / 2 - 1 : 0;
        for (i = 0; i < mp->nGdasrvs; i++) n += mp->gdasrvs[i]->free ? 1 : 0;
        n += mp->pInvar->free ? 1 : 0;
    }
    h->m->nFreePrams = n;
    p4_newtSetup(h->t);               /* Tree.optLogLike does this first (p4/tree.py:9468) */
    p4_newtAndBrentPowellOpt(h->t);
    for (i = 0; i < h->t->nNodes; i++) brLensOut[i] = h->t->nodes[i]->brLen[0];
    k = 0;
    for (p = 0; p < h->nParts; p++) {
        p4_modelPart *mp = h->m->parts[p];
        int r, a, b;
        for (r = 0; r < mp->nRMatrices; r++)
            for (a = 0; a < mp->dim - 1; a++)
                for (b = a + 1; b < mp->dim; b++) rUpperOut[k++] = mp->rMatrices[r]->bigR[a][b];
    }
    return p4_treeLogLike(h->t, 0);
}

/* pInvar of a part as the model holds it (the optimiser may have moved it). */
double ref_pInvar(void *vh, int pNum) { return ((ref_handle *)vh)->m->parts[pNum]->pInvar->val[0]; }

/* nlopt is absent; the BOBYQA paths are never taken by the oracle. */
nlopt_opt nlopt_create(nlopt_algorithm algorithm, unsigned n) { (void)algorithm; (void)n; return NULL; }
void nlopt_destroy(nlopt_opt opt) { (void)opt; }
nlopt_result nlopt_set_lower_bounds(nlopt_opt opt, const double *lb) { (void)opt; (void)lb; return NLOPT_FAILURE; }
nlopt_result nlopt_set_upper_bounds(nlopt_opt opt, const double *ub) { (void)opt; (void)ub; return NLOPT_FAILURE; }
nlopt_result nlopt_set_max_objective(nlopt_opt opt, nlopt_func f, void *d) { (void)opt; (void)f; (void)d; return NLOPT_FAILURE; }
nlopt_result nlopt_set_ftol_abs(nlopt_opt opt, double tol) { (void)opt; (void)tol; return NLOPT_FAILURE; }
nlopt_result nlopt_optimize(nlopt_opt opt, double *x, double *f) { (void)opt; (void)x; (void)f; return NLOPT_FAILURE; }
