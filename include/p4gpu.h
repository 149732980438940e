/*
 * p4gpu.h -- C ABI of libp4gpu, the GB300 (sm_103a) likelihood engine that
 * stands in for the likelihood hot path of p4's CPython extension `p4.pf`.
 *
 * Every entry point below replaces one `pf` function of the reference
 * (Pf/pfmodule.c, method table Pf/pfmodule.c:2873-3018) with the same
 * argument meaning.  Differences, all deliberate:
 *   - handles are opaque pointers (the reference passes C pointers as Python
 *     ints, so a ctypes binding keeps the same call shapes);
 *   - every call returns an int status (P4G_OK = 0) instead of printing and
 *     calling exit(1); values come back through out-parameters;
 *   - a non-positive site likelihood still yields the reference's lnL
 *     sentinel -1.0e99 (Pf/p4_tree.c:1134-1183) with status P4G_OK.
 * Buffers that the reference aliases from numpy (comp values, gdasrv
 * val/freqs/rates, preOrder/postOrder, partLikes) are aliased the same way:
 * the library keeps the caller's pointer and reads or writes it during the
 * calls that the reference reads or writes it in.
 *
 * Threading: calls on one tree are serialised by the caller (as in p4); all
 * device work goes to one CUDA stream per process (p4g_setStream overrides).
 */
#ifndef P4GPU_H
#define P4GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    P4G_OK = 0,
    P4G_EINVAL = 1,       /* bad argument / model value the reference would exit(1) on */
    P4G_ENOMEM = 2,
    P4G_ECUDA = 3,        /* CUDA runtime error; message in p4g_lastError() */
    P4G_ENONPOS = 4,      /* reserved: non-positive likelihood reported as status */
    P4G_ETIMEOUT = 5,     /* a bounded device-side wait gave up */
    P4G_ESTATE = 6,       /* call order violated (e.g. lnL before setPrams) */
    P4G_EUNSUPPORTED = 7, /* configuration with no kernel instantiation */
    P4G_ENUMERIC = 8      /* a numerical routine did not converge */
};

typedef struct p4g_data p4g_data;
typedef struct p4g_part p4g_part;
typedef struct p4g_model p4g_model;
typedef struct p4g_gdasrv p4g_gdasrv;
typedef struct p4g_tree p4g_tree;
typedef struct p4g_node p4g_node;

/* ---------------------------------------------------------------- misc */
/* Last error message of the calling thread ("" if none). */
const char *p4g_lastError(void);
/* Select the CUDA device (default: the current device at first use). */
int p4g_init(int device);
/* Use a caller-owned cudaStream_t (passed as void*) for all device work; NULL
 * restores the library's own stream. */
int p4g_setStream(void *cudaStream);
/* The stream device work is enqueued on (a cudaStream_t as void*). */
void *p4g_getStream(void);
/* Library build tag (kernel set, arch). */
const char *p4g_version(void);

/* ---------------------------------------------------------------- data */
/* pf.newData(nTax, nParts)                        Pf/pfmodule.c:29 */
p4g_data *p4g_newData(int nTax, int nParts);
/* pf.freeData(cData)                              Pf/pfmodule.c:43 */
int p4g_freeData(p4g_data *d);
/* pf.pokePartInData(cPart, cData, partNum)        Pf/pfmodule.c:73 */
int p4g_pokePartInData(p4g_part *p, p4g_data *d, int pNum);
/* pf.newPart(nTax, nChar, equateSymbols, nEquates, symbols, dim)
 *                                                 Pf/pfmodule.c:112, Pf/part.c:15 */
p4g_part *p4g_newPart(int nTax, int nChar, const char *equateSymbols, int nEquates,
                      const char *symbols, int dim);
/* pf.freePart(cPart)                              Pf/pfmodule.c:134 */
int p4g_freePart(p4g_part *p);
/* pf.pokeEquatesTable(cPart, "0101...")          Pf/pfmodule.c:151, Pf/part.c:279 */
int p4g_pokeEquatesTable(p4g_part *p, const char *table);
/* pf.pokeSequences(cPart, joinedSequences)        Pf/pfmodule.c:169, Pf/part.c:127 */
int p4g_pokeSequences(p4g_part *p, const char *seqs);
/* pf.symbolSequences(cPart) -> the part's sequences as one string of symbols
 * (nTax * nChar chars + NUL into out)        Pf/pfmodule.c:233, Pf/part.c:604 */
int p4g_symbolSequences(p4g_part *p, char *out);
/* pf.makePatterns(cPart)                          Pf/pfmodule.c:186, Pf/part.c:317 */
int p4g_makePatterns(p4g_part *p);
/* The same compression on the GPU (Pf/part.c:317-449 restated as a hash
 * table with first-occurrence representatives and a prefix sum): identical
 * patterns, counts and site -> pattern index to p4g_makePatterns. */
int p4g_makePatternsDevice(p4g_part *p);
/* pf.partPatternCount(cPart)                      Pf/pfmodule.c:247 */
int p4g_partPatternCount(p4g_part *p, int *nPatterns);
/* pf.setGlobalInvarSitesVec(cPart)                Pf/pfmodule.c:310, Pf/part.c:716 */
int p4g_setGlobalInvarSitesVec(p4g_part *p);
/* Read back the compressed data (the reference keeps it in part->patterns,
 * patternCounts, sequencePositionPatternIndex; Pf/pftypes.h:31-50).
 * patterns: nTax*nPatterns (taxon-major); counts: nPatterns; seqPosIdx: nChar.
 * Any pointer may be NULL. */
int p4g_getPatterns(p4g_part *p, int *patterns, int *counts, int *seqPosIdx);
/* globalInvarSitesVec (nPatterns) and globalInvarSitesArray (dim*nPatterns). */
int p4g_getInvarSites(p4g_part *p, int *vec, int *arr);
/* pf.getSiteLikes(cPart) -> per-site likelihoods of the last evaluation with
 * getSiteLikes=1 (nChar doubles)                 Pf/pfmodule.c:378 */
int p4g_getSiteLikes(p4g_part *p, double *out);
/* pf.getSiteRates(cTree, cPart, pNum, siteRates, gammaCats, work)
 *                       Pf/pfmodule.c:398, Pf/p4_tree.c:1383-1627
 * Evaluates the tree (setPrams + FP32 pruning) and fills, per site, the
 * posterior mean rate and the most likely Gamma category (nChar each).  The
 * part must have one gdasrv and the root must be internal; cPart may be NULL. */
int p4g_getSiteRates(p4g_tree *t, p4g_part *p, int pNum, double *siteRates, int *gammaCats);
/* pf.p4_drawAncState(cTree, pNum, seqPos, draw), for every site at once
 *                       Pf/pfmodule.c:2353, Pf/p4_treeSim.c:591-857
 * Evaluates the tree (setPrams + FP32 pruning) and draws, per site of part
 * pNum, the root state and Gamma category (or the invariant state) from
 * their posterior.  draws: nChar x 4 ints (chState, cat, isInvar,
 * invarState), as the reference's draw vector.  uniforms: nChar values in
 * [0, 1), the site's random number, or NULL for the Philox4x32-10 stream of
 * `seed`, in which the sites of all parts follow one another in part order
 * (site i of part p takes value nChar(0) + ... + nChar(p-1) + i), as the
 * reference's calls draw them.  P4G_ENUMERIC when a site's picker finds no
 * state (where the reference exits). */
int p4g_drawAncStates(p4g_tree *t, int pNum, const double *uniforms, unsigned long long seed, int *draws);
/* pf.p4_simulate(cTree, 0, gsl_rng)             Pf/p4_treeSim.c:14-590
 * Simulates every part of the tree's data down the tree with the current
 * model (setPrams is run first) and writes the leaves' states into the
 * parts' sequences; their patterns are stale until makePatterns, as after
 * the reference.  Random numbers: nUniforms values of the caller, consumed
 * in the reference's order, or (uniforms NULL) the Philox4x32-10 stream of
 * `seed`.  allStates (nullable): per part, nNodes x nChar states of every
 * node, parts concatenated.  The tree's device state is rebuilt on its next
 * evaluation. */
int p4g_simulate(p4g_tree *t, const double *uniforms, long long nUniforms, unsigned long long seed,
                 signed char *allStates);
/* pf.p4_simulate(cTree, refTree, gsl_rng) with a reference tree
 *                                                 Pf/p4_treeSim.c:223-284, p4/tree.py:9527-9600
 * Tree.simulate(refTree=...): every site's root state and Gamma category (or
 * invariant state) is drawn from the posterior at refTree's root given
 * refTree's data (p4_drawAncState per site, the parts in order: as
 * p4g_drawAncStates), then the states are simulated down t with t's model
 * from those roots, as p4g_simulate does after its root loops.  refUniforms:
 * one value in [0, 1) per site of every part, parts concatenated (the
 * reference's libc random() draws), or NULL for the Philox4x32-10 stream of
 * refSeed; uniforms / nUniforms / seed: the mutation loop's (the reference's
 * GSL stream, which this mode uses from its first value).  refTree must be
 * another tree whose parts have t's site counts, state counts and
 * categories; it is evaluated (setPrams + pruning) for the draws. */
int p4g_simulateRef(p4g_tree *t, p4g_tree *refTree, const double *refUniforms, unsigned long long refSeed,
                    const double *uniforms, long long nUniforms, unsigned long long seed,
                    signed char *allStates);
/* pf.p4_newtSetup(cTree)             Pf/pfmodule.c:2274, Pf/p4_treeNewt.c:11
 * Nothing to allocate ahead: each p4g_newtAround sizes its buffers. */
int p4g_newtSetup(p4g_tree *t);
/* p4_newtAround(cTree, epsilon, likeDelta)        Pf/p4_treeNewt.c:79-208
 * Newton-Raphson on every branch length (non-root nodes in the tree's
 * postOrder), in rounds (at most 20) until the lnL changes by less than
 * likeDelta; a branch stops when |d lnL/dt| < epsilon, at BRLEN_MIN/MAX, at
 * 5x its starting length or after 21 steps.  FP64 on the GPU (setPrams is
 * run first); the nodes' branch lengths are updated.  The root must be an
 * internal node. */
int p4g_newtAround(p4g_tree *t, double epsilon, double likeDelta);
/* pf.p4_newtAndBrentPowellOpt(cTree)   Pf/pfmodule.c:2259, Pf/p4_treeOpt.c:1182
 * Maximum likelihood for branch lengths and the model's free parameters
 * (comps, R matrices, gamma shapes, pInvar, relative rates whose free flag
 * is set; their number must equal the model's nFreePrams, P4G_EINVAL
 * otherwise).  With none free: the four p4_newtAround calls of
 * Pf/p4_treeOpt.c:1207-1212.  Otherwise Newton passes over the branch
 * lengths alternate with a Powell conjugate-direction search (Brent line
 * minimisation) over the free parameters until a pass changes lnL by less
 * than 1e-6 or the tree's pass limit is reached (the reference searches with
 * praxis; same outer loop, Pf/p4_treeOpt.c:1226-1334); trees of fewer than
 * 15 nodes then get a search over every parameter and branch length, as the
 * reference's p4_allBrentPowellOptimize.  FP64 evaluations on the GPU; the
 * model values (caller-aliased comps and gamma shapes included) and branch
 * lengths are left at the optimum. */
int p4g_newtAndBrentPowellOpt(p4g_tree *t);
/* pf.p4_getFreePrams(cTree) -> the free parameters in p4_windUpParameters
 * order (comps' first dim-1 values, R rates but the last, gamma shapes,
 * pInvar, per part; then the relative rates of parts 0..nParts-2).  *n
 * receives the count; fails with P4G_EINVAL if it exceeds cap.
 *                                     Pf/pfmodule.c:2304, Pf/p4_treeOpt.c:156 */
int p4g_getFreePrams(p4g_tree *t, double *out, int cap, int *n);
/* pf.p4_getBrLens(cTree) -> every node's branch length (nNodes doubles)
 *                                                 Pf/pfmodule.c:2289 */
int p4g_getBrLens(p4g_tree *t, double *out);

/* ---------------------------------------------------------------- model */
/* pf.p4_newModel(nParts, doRelRates, relRatesAreFree, nFreePrams, isHet,
 *   rMatrixNormalizeTo1, PINVAR_MIN, PINVAR_MAX, KAPPA_MIN, KAPPA_MAX,
 *   GAMMA_SHAPE_MIN, GAMMA_SHAPE_MAX, PIVEC_MIN, PIVEC_MAX, RATE_MIN, RATE_MAX,
 *   RELRATE_MIN, RELRATE_MAX, BRLEN_MIN, BRLEN_MAX)   Pf/pfmodule.c:1484
 * Bound pointers are aliased (1-element arrays, p4/var.py:287-305); NULL
 * means the var.py default. */
p4g_model *p4g_newModel(int nParts, int doRelRates, int relRatesAreFree, int nFreePrams,
                        int isHet, int *rMatrixNormalizeTo1, double *PINVAR_MIN,
                        double *PINVAR_MAX, double *KAPPA_MIN, double *KAPPA_MAX,
                        double *GAMMA_SHAPE_MIN, double *GAMMA_SHAPE_MAX, double *PIVEC_MIN,
                        double *PIVEC_MAX, double *RATE_MIN, double *RATE_MAX,
                        double *RELRATE_MIN, double *RELRATE_MAX, double *BRLEN_MIN,
                        double *BRLEN_MAX);
/* pf.p4_freeModel(cModel)                         Pf/pfmodule.c:1554 */
int p4g_freeModel(p4g_model *m);
/* pf.p4_newModelPart(cModel, pNum, dim, nComps, nRMatrices, nGdasrvs, nCat,
 *   pInvarFree, bQETneedsReset[int32 nComps*nR])   Pf/pfmodule.c:1590 */
int p4g_newModelPart(p4g_model *m, int pNum, int dim, int nComps, int nRMatrices,
                     int nGdasrvs, int nCat, int pInvarFree, int *bQETneedsReset);
/* pf.p4_newComp(cModel, pNum, mNum, free, val[f64 dim]) -- val aliased
 *                                                 Pf/pfmodule.c:1634 */
int p4g_newComp(p4g_model *m, int pNum, int mNum, int free, double *val);
/* pf.p4_newRMatrix(cModel, pNum, mNum, free, spec)  Pf/pfmodule.c:1653
 * spec: 20 specified (values poked in later), 5 two-parameter (kappa), the
 * empirical protein matrices 101-107 and 110-120 (cpREV, d78, jtt, mtREV24,
 * mtmam, wag, blosum62, rtRev, tmjtt94, tmlg99, lg, hivb, mtart, mtzoa,
 * gcpREV, stmtREV, vt, pmb; 20-state parts only, filled from the library's
 * table as Pf/p4_model.c:366-420 fills them), anything else all ones (Poisson
 * / JC, the reference's default). */
int p4g_newRMatrix(p4g_model *m, int pNum, int mNum, int free, int spec);
/* pf.getBigR(spec, a)  Pf/pfmodule.c:1271: the 20x20 exchangeability matrix
 * (row-major) of an empirical protein spec into out[400].  P4G_EINVAL for any
 * other spec (the reference leaves the array unfilled). */
int p4g_getBigR(int spec, double *out);
/* pf.p4_newGdasrv(cModel, pNum, mNum, nCat, free, val, freqs, rates) -- aliased
 *                                                 Pf/pfmodule.c:1672 */
p4g_gdasrv *p4g_newGdasrv(p4g_model *m, int pNum, int mNum, int nCat, int free,
                          double *val, double *freqs, double *rates);
/* pf.gdasrvCalcRates(cGdasrv): fills the aliased rates/freqs from val
 *                                                 Pf/pfmodule.c:1813 */
int p4g_gdasrvCalcRates(p4g_gdasrv *g);
/* pf.gdasrvCalcRates_np(nCat, val, freqs, rates) */
int p4g_gdasrvCalcRates_np(int nCat, double val, double *freqs, double *rates);
/* pf.p4_setRMatrixBigR(cModel, pNum, rNum, i, j, val) (sets [i][j] and [j][i])
 *                                                 Pf/pfmodule.c:1720 */
int p4g_setRMatrixBigR(p4g_model *m, int pNum, int rNum, int i, int j, double val);
/* pf.p4_setKappa(cModel, pNum, rNum, kappa)       Pf/pfmodule.c:1741 */
int p4g_setKappa(p4g_model *m, int pNum, int rNum, double kappa);
/* pf.p4_setPInvarVal(cModel, pNum, val)           Pf/pfmodule.c:1871 */
int p4g_setPInvarVal(p4g_model *m, int pNum, double val);
/* pf.p4_setRelRateVal(cModel, pNum, val)          Pf/pfmodule.c:1887 */
int p4g_setRelRateVal(p4g_model *m, int pNum, double val);

/* ---------------------------------------------------------------- tree */
/* pf.p4_newTree(nNodes, nLeaves, preOrder, postOrder, passLimit, partLikes,
 *   cData, cModel) -- preOrder/postOrder (int32 nNodes) and partLikes
 *   (f64 nParts) aliased                          Pf/pfmodule.c:1383 */
p4g_tree *p4g_newTree(int nNodes, int nLeaves, int *preOrder, int *postOrder,
                      int *passLimit, double *partLikes, p4g_data *d, p4g_model *m);
/* pf.p4_freeTree(cTree)                           Pf/pfmodule.c:1410 */
int p4g_freeTree(p4g_tree *t);
/* pf.p4_newNode(nodeNum, cTree, seqNum, isLeaf, inTree)  Pf/pfmodule.c:1443 */
p4g_node *p4g_newNode(int nodeNum, p4g_tree *t, int seqNum, int isLeaf, int inTree);
/* pf.p4_setNodeRelation(cNode, relation{0 parent,1 leftChild,2 sibling}, nodeNum|-1)
 *                                                 Pf/pfmodule.c:1907 */
int p4g_setNodeRelation(p4g_node *n, int relation, int relNum);
/* pf.p4_setTreeRoot(cTree, cNode)                 Pf/pfmodule.c:1944 */
int p4g_setTreeRoot(p4g_tree *t, p4g_node *n);
/* pf.p4_setBrLen(cNode, len)                      Pf/pfmodule.c:1960 */
int p4g_setBrLen(p4g_node *n, double len);
/* pf.p4_setCompNum / p4_setRMatrixNum / p4_setGdasrvNum(cNode, pNum, num)
 *                                                 Pf/pfmodule.c:2013-2057 */
int p4g_setCompNum(p4g_node *n, int pNum, int num);
int p4g_setRMatrixNum(p4g_node *n, int pNum, int num);
int p4g_setGdasrvNum(p4g_node *n, int pNum, int num);
/* pf.p4_setPrams(cTree, pNum|-1): gamma rates, Q, eigensystems and every
 * P deck, on the GPU in FP64                      Pf/pfmodule.c:2086 */
int p4g_setPrams(p4g_tree *t, int pNum);
/* pf.p4_treeLogLike(cTree, getSiteLikes) -> lnL; also fills the aliased
 * partLikes                                       Pf/pfmodule.c:2132 */
int p4g_treeLogLike(p4g_tree *t, int getSiteLikes, double *lnL);
/* pf.p4_partLogLike(cTree, cPart, pNum, getSiteLikes) -> part lnL
 *                                                 Pf/pfmodule.c:2147 */
int p4g_partLogLike(p4g_tree *t, p4g_part *p, int pNum, int getSiteLikes, double *lnL);
/* pf.p4_calculateBigPDecks(cNode): recompute that node's P decks for every
 * part from the current eigensystems              Pf/pfmodule.c:2165 */
int p4g_calculateBigPDecks(p4g_node *n);
/* pf.p4_calculateAllBigPDecksAllParts(cTree)      Pf/pfmodule.c:2180 */
int p4g_calculateAllBigPDecksAllParts(p4g_tree *t);
/* pf.p4_copyModelPrams / p4_copyBigPDecks / p4_copyCondLikes(treeA, treeB, ...)
 * copy the device state of tree A into tree B (same shape)
 *                                                 Pf/pfmodule.c:2445-2494 */
int p4g_copyModelPrams(p4g_tree *a, p4g_tree *b);
int p4g_copyBigPDecks(p4g_tree *a, p4g_tree *b, int doAll);
int p4g_copyCondLikes(p4g_tree *a, p4g_tree *b, int doAll);

/* ------------------------------------------------- batched (no pf counterpart:
 * replaces the Python loop over chains, p4/mcmc.py:2861-2901) */
/* setPrams (if doSetPrams) + treeLogLike for nTrees trees in one launch
 * sequence on one stream; lnL[i] receives tree i's log likelihood and each
 * tree's aliased partLikes is filled. */
int p4g_treeLogLikeBatch(p4g_tree **trees, int nTrees, int doSetPrams, double *lnL);

/* Evaluation mode of a tree: 0 = fused FP32 pruning with integer scalers
 * (default); 1 = the plain FP64 path, a direct restatement of the
 * reference's per-node loops (one launch per internal node, FP64 CLs,
 * no scaling).  No pf counterpart: the reference has only the FP64 CPU path. */
int p4g_setPrecision(p4g_tree *t, int mode);
/* Set every node's branch length from brLens[nNodes] in one call (the root's
 * entry is ignored); replaces nNodes p4_setBrLen calls (p4/tree.py:9357-9359). */
int p4g_setBrLens(p4g_tree *t, const double *brLens);
/* A batch of trees evaluated together (the chains of an MCMCMC; no pf
 * counterpart -- it replaces the chain loop p4/mcmc.py:2861-2901).  Trees
 * must share one data object and model shapes.  p4g_batchLogLike runs
 * setPrams + treeLogLike for every tree with one k_gammaEig and one k_pdeck
 * launch for all (tree, part) pairs, one pruning launch per (states,
 * categories) group over every tree's tiles and one result copy; after the
 * first call the sequence is captured as a CUDA graph and replayed
 * (p4g_batchSetGraph(b, 0) turns the graph off).  lnL[i] gets tree i's
 * log likelihood; each tree's aliased partLikes is filled. */
typedef struct p4g_batch p4g_batch;
p4g_batch *p4g_newBatch(p4g_tree **trees, int nTrees);
int p4g_freeBatch(p4g_batch *b);
int p4g_batchSetGraph(p4g_batch *b, int on);
/* Clade tables for the batch's trees (off by default: every topology change
 * of a tree renumbers its clades and captures the batch graph again, which
 * pays only when topologies stay fixed).  A tree whose clade size was neither
 * timed by its own first evaluation nor set by p4g_setCladeSize uses no
 * tables when the first tree's timing turned them off. */
int p4g_batchSetClades(p4g_batch *b, int on);
int p4g_batchLogLike(p4g_batch *b, double *lnL);
/* Pruning tile-shape autotuner (on by default): the first evaluation of a
 * tree times each candidate (threads, patterns per thread) shape of the
 * fused kernel and keeps the fastest, cached per (states, categories, taxa,
 * pattern-count bucket).  A shape is (threads per block, patterns per
 * thread, P decks in shared memory or read through L1, lanes per pattern:
 * the categories of a pattern spread over 1, 2 or 4 lanes).
 * p4g_setAutotune(0) turns it off and clears the cache; p4g_getPruneShape
 * reports the shape and tile (patterns per block) chosen for pruning group
 * `group` of a tree (groups = distinct (dim, nCat) pairs in part order);
 * p4g_setPruneShape fixes it (after the tree's first evaluation), returning
 * P4G_EINVAL for a shape that does not apply to the group's (dim, nCat).
 * Every shape computes the same per-pattern values. */
int p4g_setAutotune(int on);
/* Programmatic dependent launch of the P-deck and CUDA-core pruning kernels
 * (default on; no pf counterpart): each of those kernels waits for the
 * stream's previous kernel before it reads anything and lets the next one
 * launch while it runs, so launch latency overlaps the previous kernel's
 * tail.  Affects launches and graph captures made after the call (graphs
 * captured before keep their mode).  Results are the same either way. */
int p4g_setProgrammaticLaunch(int on);
int p4g_getPruneShape(p4g_tree *t, int group, int *shape, int *tile);
int p4g_setPruneShape(p4g_tree *t, int group, int shape);
/* Clade tables (site repeats): every maximal subtree with at most maxLeaves
 * leaves (default 6; < 2 turns them off) is evaluated once per distinct
 * combination of its leaves' codes and read from that table by the
 * whole-tree pruning program; per-pattern results are unchanged.  Takes
 * effect at the tree's next evaluation; trees in a p4g_batch use none. */
int p4g_setCladeSize(p4g_tree *t, int maxLeaves);
/* Whole topology in one call: parent/leftChild/sibling[nNodes] (-1 = none)
 * and the root; replaces 3*nNodes p4_setNodeRelation calls and
 * p4_setTreeRoot (p4/tree.py:9334-9355). */
int p4g_setTopology(p4g_tree *t, const int *parent, const int *leftChild, const int *sibling,
                    int root);
/* Upper-triangle values of R matrix rNum of part pNum, row-major (i<j),
 * dim*(dim-1)/2 entries; replaces that many p4_setRMatrixBigR calls
 * (p4/model.py:184-197). */
int p4g_setRMatrixUpper(p4g_model *m, int pNum, int rNum, const double *vals);
/* Asynchronous form of setPrams (if doSetPrams) + treeLogLike: enqueue the
 * parameter upload, kernels and result copy on the library stream and
 * return; p4g_treeLogLikeWait synchronises and delivers lnL / partLikes. */
int p4g_treeLogLikeAsync(p4g_tree *t, int doSetPrams);
int p4g_treeLogLikeWait(p4g_tree *t, double *lnL);
/* info[0] bytes moved host->device by a setPrams that follows a change of
 * branch lengths only (the branch lengths, which the P-deck kernel reads
 * from the pinned host image; the whole parameter image where the device
 * cannot map it), info[1] kernel launches
 * of one setPrams + treeLogLike, info[2] total patterns, info[3] stack
 * slots of the pruning program, info[4] program length, info[5] bytes
 * copied device->host per treeLogLike, info[6] clade tables in use
 * (info: 7 entries). */
int p4g_treeInfo(p4g_tree *t, long long *info);
/* Device memory the tree's own evaluation state holds (*treeBytes: image,
 * decks, eigensystems, partial sums; 0 before its first evaluation) and its
 * data parts' uploaded copies hold (*dataBytes), as allocated so far.
 * Allocates nothing.  No pf counterpart (introspection for tests). */
int p4g_treeDeviceBytes(p4g_tree *t, long long *treeBytes, long long *dataBytes);
/* Replay the tree's setPrams and pruning launch sequences from CUDA graphs
 * (default on; captured again whenever a sequence changes).  No pf
 * counterpart. */
int p4g_setGraphs(p4g_tree *t, int on);
/* Tile shape of the clade-table launches of pruning group `group` (a shape
 * number of p4g_setPruneShape; protein shape 3 runs the clade programs on
 * the tensor cores), instead of the first evaluation's timed choice.  No pf
 * counterpart. */
int p4g_setCladeShape(p4g_tree *t, int group, int shape);

/* ------------------------------------------------- learned proposal network
 * No pf counterpart: the reference's proposals are all hand-made.  A 3-layer
 * MLP (dIn -> hidden -> hidden -> dOut, tanh), BF16 weights, FP32
 * accumulation, FP32 master weights + Adam, trained by the library's own
 * forward/backward kernels.  dOut = 2d: rows of outputs are (mu[d], s[d]) of
 * a diagonal Gaussian; the loss is its negative log density of the target
 * rows t[d], mean over the batch.  Parameters are ordered W1[h][dIn], b1[h],
 * W2[h][h], b2[h], W3[dOut][h], b3[dOut]. */
typedef struct p4g_mlp p4g_mlp;
p4g_mlp *p4g_mlpNew(int dIn, int hidden, int dOut, int maxBatch, unsigned long long seed);
int p4g_mlpFree(p4g_mlp *m);
int p4g_mlpNumParams(p4g_mlp *m, int *n);
int p4g_mlpGetParams(p4g_mlp *m, float *out);
int p4g_mlpSetParams(p4g_mlp *m, const float *in);
/* y[B][dOut] = network(x[B][dIn]) */
int p4g_mlpForward(p4g_mlp *m, const float *x, int B, float *y);
/* Gradients of the loss (no update); grads nullable, loss nullable. */
int p4g_mlpGradients(p4g_mlp *m, const float *x, const float *t, int B, float *grads, float *loss);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on (x, t); loss nullable. */
int p4g_mlpTrainStep(p4g_mlp *m, const float *x, const float *t, int B, float lr, float *loss);

/* ------------------------------------------------- evaluation without allocation */
/* No counterpart in the reference (p4 evaluates only through its own
 * per-tree buffers).  For callers that may not allocate device memory: code
 * running inside a program whose device memory belongs to another allocator
 * (a framework's caching pool, or an arena a service reserves up front for a
 * fixed memory budget).  There cudaMalloc can fail because the pool already
 * holds the device's memory, and cudaMalloc / cudaFree synchronise the whole
 * device, stalling the rest of the program.
 *
 * Computes what p4g_setPrams(t, -1) followed by p4g_treeLogLike(t, 0, lnL)
 * computes (FP32 pruning path; sets t's partLikes and lnL the same way), but
 * calls no cudaMalloc, cudaFree, pinned-memory or pool routine: every device
 * buffer of the evaluation lives in one fixed array of
 * P4G_NOALLOC_SCRATCH_BYTES inside the library, and the inputs are staged in
 * a fixed host array of the same size.  That host array is ordinary
 * (pageable) memory, so the CUDA driver copies it through its own internal
 * pinned buffers and the call blocks the calling thread until the copy and
 * the evaluation are done.  The tree's own device state is neither allocated
 * nor used.  A tree whose data, parameters and working buffers need more than
 * that returns P4G_EUNSUPPORTED with the size it needs (a 64-taxon,
 * 100,000-pattern DNA part needs about 8 MiB).
 *
 * Every call on a device shares the one array, so two evaluations whose GPU
 * work overlapped would overwrite each other's inputs and partial sums.  The
 * call is synchronous and holds a process-wide lock from staging until its
 * results are back on the host, so calls through this entry point from
 * several host threads run one after another.  The counters that must start
 * at zero (completion tickets, failure flags, status) are cleared by every
 * call, as are the kernels' output buffers.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current) and keeps it for the
 * process; make that first call before any stream capture that could
 * include one.  The array stays resident on every device that loaded the
 * library until the process exits. */
#define P4G_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
int p4g_treeLogLikeNoAlloc(p4g_tree *t, double *lnL);

/* ------------------------------------------------- introspection (tests) */
/* Tensor-core datapath check (no pf counterpart): one tcgen05.mma kind::tf32
 * (M 128, N 32, K 8; A in tensor memory, B in shared memory as K-major core
 * matrices) on TF32-exact inputs, compared with an FP64 product on the host;
 * *maxAbsErr = largest |error| (0 when the datapath is right).  variant 0
 * is the layout the protein kernel uses; variant 1 reads the descriptor's
 * two core-matrix strides the other way round. */
int p4g_tensorSelfTest(int variant, double *maxAbsErr);
/* Measured FP32 FMA throughput (no pf counterpart): 4 blocks of 256 threads
 * per SM, 8 independent FMA chains per thread, `iters` x 128 FMAs per
 * thread; best of three timed launches after a warm-up launch, CUDA events
 * on the library stream.  *tflops = 2 x FMAs / time, *ms = that launch's
 * time.  The roofline denominator of the CUDA-core pruning kernels. */
int p4g_fp32FmaPeak(int iters, double *tflops, double *ms);
/* FP64 P deck [dim*dim] of node/part/cat, row = parent state (bigPDecks); formed in
 * compensated FP32-pair arithmetic, within 1e-12 of the reference's FP64 deck. */
int p4g_getPDeck(p4g_node *n, int pNum, int cat, double *out);
/* FP32 decks of a part as the pruning kernel reads them, in canonical
 * row-major order for every node: nNodes*nCat*dim*dim floats; and the
 * partial-equate tables nNodes*nPartial*nCat*dim. */
int p4g_getDecks32(p4g_tree *t, int pNum, float *decks, float *eqTab, int *nPartial);
/* Compact tip codes used by the kernels (nTax*nPatterns bytes), and the
 * state masks of the partial equates (nPartial). */
int p4g_getCompactCodes(p4g_part *p, unsigned char *codes, unsigned *partialMasks);
/* Per-pattern outputs of the last getSiteLikes evaluation of part pNum:
 * FP32 scaled root likelihood, integer scaler exponent, FP64 log likelihood. */
int p4g_getPatternLikes(p4g_tree *t, int pNum, float *likeScaled, int *exps, double *lnl);
/* GPU-computed gamma rates of gdasrv gNum of part pNum (nCat doubles). */
int p4g_getGammaRates(p4g_tree *t, int pNum, int gNum, double *out);

#ifdef __cplusplus
}
#endif
#endif /* P4GPU_H */
