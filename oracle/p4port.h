/*
 * p4port.h -- TEST INFRASTRUCTURE (oracle).  The project's own CPU
 * restatement of p4's likelihood hot path, used only by tests/ and by the
 * CPU-baseline leg of bench.py.  Never linked into the product library.
 */
#ifndef P4PORT_H
#define P4PORT_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Discrete-gamma category rates (equal weights, bin means); Pf/gamma.c:17-50. */
int port_discreteGamma(double alpha, int K, double *rates);

/* Q = R.diag(pi), diagonal = -row sum, scaled to mean rate 1; Pf/util.c:44-115. */
int port_bigQ(int dim, const double *R, const double *pi, double *Q);

/* Eigensystem of the reversible Q through its symmetric form
 * S = diag(pi)^1/2 Q diag(pi)^-1/2 (cyclic Jacobi, FP64).
 * Out: U (dim*dim, columns = eigenvectors of S), lam (dim). */
int port_eigSym(int dim, const double *Q, const double *pi, double *U, double *lam);

/* P(t) = diag(pi)^-1/2 U exp(lam t) U^T diag(pi)^1/2, row = parent state. */
void port_pmatrix(int dim, const double *U, const double *lam, const double *pi,
                  double t, double *P);

/* char -> code as Pf/part.c:127-277 (symbols 0..dim-1, '-' -1, '?' -2,
 * equate m -> -64+m).  Returns 0, or -1 on an unknown character. */
int port_encode(int nTax, int nChar, const char *seqs, const char *symbols, int dim,
                const char *equateSymbols, int nEquates, int *codes);

/* First-occurrence pattern compression, same output as Pf/part.c:317-449.
 * codes: nTax*nChar; patterns: nTax*nChar capacity (row stride nChar).
 * Returns nPatterns. */
int port_makePatterns(int nTax, int nChar, const int *codes, int *patterns, int *counts,
                      int *seqPosIdx);

/* Invariant-site vector/array, Pf/part.c:716-848.  patterns row stride = nPat. */
void port_invarSites(int nTax, int nPat, int dim, int nEquates, const int *equates,
                     const int *patterns, int *invarVec, int *invarArr);

/* Reference-semantics FP64 part log likelihood (no scaling):
 * pruning Pf/p4_node.c:636-857, root reduction Pf/p4_tree.c:924-1197.
 * pdecks: nNodes*nCat*dim*dim (row = parent state); patterns: nTax*nPat.
 * patLikes (nullable) receives per-pattern likelihoods; catWork (nullable,
 * nPat*nCat) the per-category root sums sum_s pi_s cl[cat][s] that the
 * reference's site-rate routine uses (Pf/p4_tree.c:1383-1627). */
double port_partLogLike64(int nNodes, int root, const int *leftChild, const int *sibling,
                          const int *isLeaf, const int *seqNum, const int *postOrder,
                          int dim, int nCat, int nPat, int nEquates, const int *equates,
                          const int *patterns, const int *counts, const double *pdecks,
                          const double *rootComp, double pInvar, const int *invarVec,
                          const int *invarArr, double *patLikes, double *catWork);

/* FP32 mirror of the fused GPU pruning kernel, bit-exact by construction:
 * same evaluation schedule, same FP32 operation order (explicit fmaf),
 * same power-of-two rescaling rule, same FP32 root sum.
 *   decks32:   nNodes*nCat*dim*dim FP32 P (row = parent state)
 *   eqTab32:   nNodes*nPartial*nCat*dim FP32 sums over partial-equate members
 *   ccodes:    nTax*nPat compact codes (0..dim-1 state, dim = all-ones,
 *              dim+1+q = partial equate q)
 *   rootComp:  FP64 root composition; partialMask: state masks of the
 *              partial equates; invMask: per-pattern invariant-state mask;
 *              counts: FP64 pattern weights.
 * Out: likeScaled (FP32 root like * 2^E), exps (E), lnl (FP64 log like).
 * cherries != 0: like the GPU program, no rescale step at a non-root node
 * whose only children are two leaves.
 * Returns the pattern-weighted sum, or -1e99 if any like <= 0. */
double port_partPrune32(int nNodes, int root, const int *leftChild, const int *sibling,
                        const int *isLeaf, const int *seqNum, int dim, int nCat, int nPat,
                        int nPartial, const float *decks32, const float *eqTab32,
                        const uint8_t *ccodes, const double *rootComp, double pInvar,
                        const uint32_t *partialMask, const uint32_t *invMask,
                        const double *counts, float *likeScaled, int *exps, double *lnl, int cherries);

/* Threshold below which a pattern's CL block is rescaled: 2^-PORT_SCALE_LOG2. */
#define PORT_SCALE_LOG2 32

/* The next port_partLogLike64 copies the root CL (nCat x dim x nPat) to out. */
void port_setRootCLOut(double *out);

#ifdef __cplusplus
}
#endif

#endif
