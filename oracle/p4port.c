/*
 * p4port.c -- TEST INFRASTRUCTURE (oracle): the project's CPU restatement of
 * p4's likelihood hot path.  Only tests/ and the CPU-baseline leg of bench.py
 * load it (as oracle/_ref/libp4port.so); the product library never does.
 *
 * Parity anchors (reference files, by path within the p4 project):
 *   discrete gamma ............ Pf/gamma.c:17-50 (Yang 1994), with the
 *                               published algorithms it uses: AS91 (Best &
 *                               Roberts 1975) chi-square quantile, AS32
 *                               (Bhattacharjee 1970) incomplete gamma ratio,
 *                               ACM 291 (Pike & Hill 1966) log gamma, AS70
 *                               (Odeh & Evans 1974) normal quantile.
 *   Q build + normalisation ... Pf/util.c:44-115
 *   P = exp(Qt) ............... Pf/eig.c:163-223 (here via the symmetric form
 *                               of the reversible Q instead of a general
 *                               real eigensystem; same matrix up to rounding)
 *   char coding ............... Pf/part.c:127-277
 *   pattern compression ....... Pf/part.c:317-449 (first-occurrence order;
 *                               hashed here, same output)
 *   invariant sites ........... Pf/part.c:716-848
 *   pruning ................... Pf/p4_node.c:636-857
 *   root reduction ............ Pf/p4_tree.c:924-1378
 */
#include "p4port.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define GAP_CODE (-1)
#define QMARK_CODE (-2)
#define N_LIKE (-3)
#define EQUATES_BASE (-64)

/* ------------------------------------------------------------------ gamma */

static double lnGammaPH(double alpha)
{
    /* Pike & Hill: shift the argument up to >= 7, then Stirling's series. */
    double x = alpha, f = 0.0, z;
    if (x < 7.0) {
        f = 1.0;
        z = x - 1.0;
        for (;;) {
            z += 1.0;
            if (!(z < 7.0)) break;
            f *= z;
        }
        x = z;
        f = -log(f);
    }
    z = 1.0 / (x * x);
    return f + (x - 0.5) * log(x) - x + 0.918938533204673 +
           (((-0.000595238095238 * z + 0.000793650793651) * z - 0.002777777777778) * z +
            0.083333333333333) / x;
}

static double incGammaRatio(double x, double p, double lnGammaP)
{
    /* AS32: series for x <= 1 or x < p, else continued fraction. */
    const double accurate = 1e-8, overflow = 1e30;
    double factor, gin, rn, a, b, an, dif, term, pn[6];
    int i, it;
    if (x == 0.0) return 0.0;
    if (x < 0 || p <= 0) return -1.0;
    factor = exp(p * log(x) - x - lnGammaP);
    if (!(x > 1 && x >= p)) {
        gin = 1.0;
        term = 1.0;
        rn = p;
        for (it = 0; it < 100000; it++) {
            rn += 1.0;
            term *= x / rn;
            gin += term;
            if (!(term > accurate)) break;
        }
        return gin * (factor / p);
    }
    a = 1.0 - p;
    b = a + x + 1.0;
    term = 0.0;
    pn[0] = 1.0;
    pn[1] = x;
    pn[2] = x + 1;
    pn[3] = x * b;
    gin = pn[2] / pn[3];
    for (it = 0; it < 100000; it++) {
        a += 1.0;
        b += 2.0;
        term += 1.0;
        an = a * term;
        for (i = 0; i < 2; i++) pn[i + 4] = b * pn[i + 2] - an * pn[i];
        if (pn[5] != 0) {
            rn = pn[4] / pn[5];
            dif = fabs(gin - rn);
            if (!(dif > accurate) && dif <= accurate * rn) return 1.0 - factor * gin;
            gin = rn;
        }
        for (i = 0; i < 4; i++) pn[i] = pn[i + 2];
        if (!(fabs(pn[4]) < overflow))
            for (i = 0; i < 4; i++) pn[i] /= overflow;
    }
    return -1.0;
}

static double normalQuantile(double prob)
{
    /* AS70 rational approximation. */
    const double a0 = -0.322232431088, a1 = -1.0, a2 = -0.342242088547,
                 a3 = -0.0204231210245, a4 = -0.453642210148e-4, b0 = 0.0993484626060,
                 b1 = 0.588581570495, b2 = 0.531103462366, b3 = 0.103537752850,
                 b4 = 0.0038560700634;
    double p1 = prob < 0.5 ? prob : 1 - prob, y, z;
    if (p1 < 1e-20) return -9999;
    y = sqrt(log(1 / (p1 * p1)));
    z = y + ((((y * a4 + a3) * y + a2) * y + a1) * y + a0) /
                ((((y * b4 + b3) * y + b2) * y + b1) * y + b0);
    return prob < 0.5 ? -z : z;
}

static double chi2Quantile(double prob, double v)
{
    /* AS91 (percentage points of chi-square with v d.f.). */
    const double e = 0.5e-6, aa = 0.6931471805;
    double p = prob, g, xx, c, ch, a = 0, q, p1, p2, t, x, b, s1, s2, s3, s4, s5, s6;
    int it;
    if (p < 0.000002 || p > 0.999998 || v <= 0.0) return -1.0;
    g = lnGammaPH(v / 2.0);
    xx = v / 2.0;
    c = xx - 1.0;
    if (v < -1.24 * log(p)) {
        ch = pow(p * xx * exp(g + xx * aa), 1.0 / xx);
        if (ch - e < 0) return ch;
    } else if (v <= 0.32) {
        ch = 0.4;
        a = log(1.0 - p);
        for (it = 0; it < 100000; it++) {
            q = ch;
            p1 = 1.0 + ch * (4.67 + ch);
            p2 = ch * (6.73 + ch * (6.66 + ch));
            t = -0.5 + (4.67 + 2.0 * ch) / p1 - (6.73 + ch * (13.32 + 3.0 * ch)) / p2;
            ch -= (1.0 - exp(a + g + 0.5 * ch + c * aa) * p2 / p1) / t;
            if (fabs(q / ch - 1.0) - 0.01 <= 0.0) break;
        }
    } else {
        x = normalQuantile(p);
        p1 = 0.222222 / v;
        ch = v * pow((x * sqrt(p1) + 1.0 - p1), 3.0);
        if (ch > 2.2 * v + 6.0) ch = -2.0 * (log(1.0 - p) - c * log(0.5 * ch) + g);
    }
    for (it = 0; it < 100000; it++) {
        q = ch;
        p1 = 0.5 * ch;
        t = incGammaRatio(p1, xx, g);
        if (t < 0.0) return -1.0;
        p2 = p - t;
        t = p2 * exp(xx * aa + g + p1 - c * log(ch));
        b = t / ch;
        a = 0.5 * t - b * c;
        s1 = (210.0 + a * (140.0 + a * (105.0 + a * (84.0 + a * (70.0 + 60.0 * a))))) / 420.0;
        s2 = (420.0 + a * (735.0 + a * (966.0 + a * (1141.0 + 1278.0 * a)))) / 2520.0;
        s3 = (210.0 + a * (462.0 + a * (707.0 + 932.0 * a))) / 2520.0;
        s4 = (252.0 + a * (672.0 + 1182.0 * a) + c * (294.0 + a * (889.0 + 1740.0 * a))) / 5040.0;
        s5 = (84.0 + 264.0 * a + c * (175.0 + 606.0 * a)) / 2520.0;
        s6 = (120.0 + c * (346.0 + 127.0 * c)) / 5040.0;
        ch += t * (1 + 0.5 * t * s1 - b * c * (s1 - b * (s2 - b * (s3 - b * (s4 - b * (s5 - b * s6))))));
        if (!(fabs(q / ch - 1.0) > e)) return ch;
    }
    return -1.0;
}

int port_discreteGamma(double alpha, int K, double *rates)
{
    /* Yang (1994) equal-probability categories, rate = mean of each bin,
     * Gamma(alpha, beta=alpha). */
    double *cut, factor = alpha / alpha * K, lnga1;
    int i;
    if (K < 1 || !(alpha > 0)) return -1;
    if (K == 1) {
        rates[0] = 1.0;
        return 0;
    }
    cut = malloc(sizeof(double) * K);
    lnga1 = lnGammaPH(alpha + 1);
    for (i = 0; i < K - 1; i++) cut[i] = chi2Quantile((i + 1.0) / K, 2.0 * alpha) / (2.0 * alpha);
    for (i = 0; i < K - 1; i++) cut[i] = incGammaRatio(cut[i] * alpha, alpha + 1, lnga1);
    rates[0] = cut[0] * factor;
    rates[K - 1] = (1 - cut[K - 2]) * factor;
    for (i = 1; i < K - 1; i++) rates[i] = (cut[i] - cut[i - 1]) * factor;
    free(cut);
    return 0;
}

/* -------------------------------------------------------------- Q and P */

int port_bigQ(int dim, const double *R, const double *pi, double *Q)
{
    int i, j;
    double sum, ode;
    for (j = 0; j < dim; j++)
        for (i = 0; i < dim; i++) Q[i * dim + j] = R[i * dim + j] * pi[j];
    for (i = 0; i < dim; i++) {
        sum = 0.0;
        for (j = 0; j < dim; j++)
            if (i != j) sum = sum + Q[i * dim + j];
        Q[i * dim + i] = -sum;
    }
    sum = 0.0;
    for (i = 0; i < dim; i++) sum = sum + pi[i];
    if (sum < 0.999 || sum > 1.001) return -1;
    ode = 0.0;
    for (i = 0; i < dim; i++)
        for (j = 0; j < dim; j++)
            if (i != j) ode = ode + pi[i] * Q[i * dim + j];
    ode = 1.0 / ode;
    for (i = 0; i < dim * dim; i++) Q[i] = Q[i] * ode;
    return 0;
}

int port_eigSym(int dim, const double *Q, const double *pi, double *U, double *lam)
{
    /* Cyclic Jacobi on S = diag(sqrt pi) Q diag(1/sqrt pi) (symmetric when Q
     * is reversible).  Rotation per pair (p,q): theta = (s_qq - s_pp)/(2 s_pq),
     * t = sgn(theta)/(|theta| + sqrt(theta^2+1)), c = 1/sqrt(t^2+1), s = t c. */
    double *S = malloc(sizeof(double) * dim * dim);
    double *sq = malloc(sizeof(double) * dim);
    int i, j, k, p, q, sweep, rc = -1;
    for (i = 0; i < dim; i++) sq[i] = sqrt(pi[i]);
    for (i = 0; i < dim; i++)
        for (j = 0; j < dim; j++) {
            if (i == j) S[i * dim + j] = Q[i * dim + j];
            else if (j > i) S[i * dim + j] = Q[i * dim + j] * sq[i] / sq[j];
            else S[i * dim + j] = S[j * dim + i];
        }
    for (i = 0; i < dim * dim; i++) U[i] = 0.0;
    for (i = 0; i < dim; i++) U[i * dim + i] = 1.0;
    for (sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, diag = 0.0;
        for (i = 0; i < dim; i++) {
            diag += S[i * dim + i] * S[i * dim + i];
            for (j = i + 1; j < dim; j++) off += S[i * dim + j] * S[i * dim + j];
        }
        if (off <= 1e-36 * diag || off == 0.0) {
            rc = 0;
            break;
        }
        for (p = 0; p < dim - 1; p++)
            for (q = p + 1; q < dim; q++) {
                double apq = S[p * dim + q], theta, t, c, s;
                if (apq == 0.0) continue;
                theta = (S[q * dim + q] - S[p * dim + p]) / (2.0 * apq);
                t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                c = 1.0 / sqrt(t * t + 1.0);
                s = t * c;
                for (k = 0; k < dim; k++) { /* columns p,q */
                    double a = S[k * dim + p], b = S[k * dim + q];
                    S[k * dim + p] = c * a - s * b;
                    S[k * dim + q] = s * a + c * b;
                }
                for (k = 0; k < dim; k++) { /* rows p,q */
                    double a = S[p * dim + k], b = S[q * dim + k];
                    S[p * dim + k] = c * a - s * b;
                    S[q * dim + k] = s * a + c * b;
                }
                for (k = 0; k < dim; k++) {
                    double a = U[k * dim + p], b = U[k * dim + q];
                    U[k * dim + p] = c * a - s * b;
                    U[k * dim + q] = s * a + c * b;
                }
            }
    }
    for (i = 0; i < dim; i++) lam[i] = S[i * dim + i];
    free(S);
    free(sq);
    return rc;
}

void port_pmatrix(int dim, const double *U, const double *lam, const double *pi, double t,
                  double *P)
{
    int i, j, k;
    double *ex = malloc(sizeof(double) * dim);
    for (k = 0; k < dim; k++) ex[k] = exp(lam[k] * t);
    for (i = 0; i < dim; i++) {
        double ri = 1.0 / sqrt(pi[i]);
        for (j = 0; j < dim; j++) {
            double acc = 0.0, rj = sqrt(pi[j]);
            for (k = 0; k < dim; k++) acc += U[i * dim + k] * ex[k] * U[j * dim + k];
            P[i * dim + j] = acc * ri * rj;
        }
    }
    free(ex);
}

/* ---------------------------------------------------------- data / patterns */

int port_encode(int nTax, int nChar, const char *seqs, const char *symbols, int dim,
                const char *equateSymbols, int nEquates, int *codes)
{
    int i, m, n = nTax * nChar;
    for (i = 0; i < n; i++) {
        char ch = seqs[i];
        int code = 9999;
        for (m = 0; m < dim; m++)
            if (ch == symbols[m]) { code = m; break; }
        if (code == 9999) {
            if (ch == '-') code = GAP_CODE;
            else if (ch == '?') code = QMARK_CODE;
            else
                for (m = 0; m < nEquates; m++)
                    if (ch == equateSymbols[m]) { code = EQUATES_BASE + m; break; }
        }
        if (code == 9999) return -1;
        codes[i] = code;
    }
    return 0;
}

int port_makePatterns(int nTax, int nChar, const int *codes, int *patterns, int *counts,
                      int *seqPosIdx)
{
    /* Open-addressing hash of column contents; a new column is appended at
     * the end, so pattern order is first occurrence, as in the reference. */
    size_t cap = 1;
    int *slot, nPat = 0, i, t;
    int *col = malloc(sizeof(int) * nTax);
    while (cap < (size_t)nChar * 2 + 16) cap <<= 1;
    slot = malloc(sizeof(int) * cap);
    for (size_t s = 0; s < cap; s++) slot[s] = -1;
    for (i = 0; i < nChar; i++) counts[i] = 0;
    for (i = 0; i < nChar; i++) {
        uint64_t h = 1469598103934665603ULL;
        size_t s;
        for (t = 0; t < nTax; t++) {
            col[t] = codes[(size_t)t * nChar + i];
            h = (h ^ (uint32_t)col[t]) * 1099511628211ULL;
        }
        s = (size_t)(h & (cap - 1));
        for (;;) {
            int pidx = slot[s];
            if (pidx < 0) {
                slot[s] = nPat;
                for (t = 0; t < nTax; t++) patterns[(size_t)t * nChar + nPat] = col[t];
                counts[nPat] = 1;
                seqPosIdx[i] = nPat;
                nPat++;
                break;
            }
            for (t = 0; t < nTax; t++)
                if (patterns[(size_t)t * nChar + pidx] != col[t]) break;
            if (t == nTax) {
                counts[pidx]++;
                seqPosIdx[i] = pidx;
                break;
            }
            s = (s + 1) & (cap - 1);
        }
    }
    free(slot);
    free(col);
    return nPat;
}

void port_invarSites(int nTax, int nPat, int dim, int nEquates, const int *equates,
                     const int *patterns, int *invarVec, int *invarArr)
{
    int p, t, j;
    (void)nEquates;
    for (p = 0; p < nPat; p++) {
        int sum = 0;
        for (j = 0; j < dim; j++) {
            int all = 1;
            for (t = 0; t < nTax; t++) {
                int c = patterns[(size_t)t * nPat + p], ok;
                if (c >= 0) ok = (c == j);
                else if (c == N_LIKE || c == GAP_CODE || c == QMARK_CODE) ok = 1;
                else ok = equates[(c - EQUATES_BASE) * dim + j];
                if (!ok) { all = 0; break; }
            }
            invarArr[(size_t)j * nPat + p] = all;
            sum += all;
        }
        invarVec[p] = sum;
    }
}

/* ----------------------------------------------------- FP64 reference path */

static int isNLike(const int *equates, int dim, int e)
{
    int j;
    for (j = 0; j < dim; j++)
        if (!equates[e * dim + j]) return 0;
    return 1;
}

/* contribution of a leaf child to parent state s, category c (Pf/p4_node.c:663-720) */
static double tipFactor64(const double *P, int dim, int code, const int *equates, int nEq,
                          int s)
{
    int j;
    double sum;
    if (code >= 0) return P[s * dim + code];
    if (code == GAP_CODE || code == QMARK_CODE) return 1.0;
    if (code >= EQUATES_BASE && code < EQUATES_BASE + nEq) {
        int e = code - EQUATES_BASE;
        if (isNLike(equates, dim, e)) return 1.0;
        sum = 0.0;
        for (j = 0; j < dim; j++)
            if (equates[e * dim + j]) sum += P[s * dim + j];
        return sum;
    }
    return NAN;
}

/* When set, the next port_partLogLike64 copies the root's CL
 * (nCat x dim x nPat) here and clears the pointer: the input of the
 * ancestral-state draw (Pf/p4_treeSim.c:591-845 reads t->root->cl). */
static double *g_rootCLOut = NULL;
void port_setRootCLOut(double *out) { g_rootCLOut = out; }

double port_partLogLike64(int nNodes, int root, const int *leftChild, const int *sibling,
                          const int *isLeaf, const int *seqNum, const int *postOrder,
                          int dim, int nCat, int nPat, int nEquates, const int *equates,
                          const int *patterns, const int *counts, const double *pdecks,
                          const double *rootComp, double pInvar, const int *invarVec,
                          const int *invarArr, double *patLikes, double *catWork)
{
    double **cl = calloc(nNodes, sizeof(double *));
    size_t clSize = (size_t)nCat * dim * nPat;
    size_t deck = (size_t)nCat * dim * dim;
    int k, v, c, s, p, j;
    double lnL = 0.0;

    for (k = 0; k < nNodes; k++) {
        v = postOrder[k];
        if (v < 0) continue;
        if (isLeaf[v] && v != root) continue;
        cl[v] = malloc(sizeof(double) * clSize);
        for (p = 0; p < nPat; p++)
            for (c = 0; c < nCat; c++)
                for (s = 0; s < dim; s++) {
                    int first = 1, ch;
                    double val = 0.0;
                    for (ch = leftChild[v]; ch >= 0; ch = sibling[ch]) {
                        const double *P = pdecks + ch * deck + (size_t)c * dim * dim;
                        double f;
                        if (isLeaf[ch]) {
                            f = tipFactor64(P, dim, patterns[(size_t)seqNum[ch] * nPat + p], equates,
                                            nEquates, s);
                        } else {
                            const double *x = cl[ch] + (size_t)c * dim * nPat;
                            f = 0.0;
                            for (j = 0; j < dim; j++) f = f + P[s * dim + j] * x[(size_t)j * nPat + p];
                        }
                        if (first) { val = f; first = 0; }
                        else val *= f;
                    }
                    cl[v][((size_t)c * dim + s) * nPat + p] = val;
                }
    }

    if (g_rootCLOut && cl[root]) memcpy(g_rootCLOut, cl[root], sizeof(double) * clSize);
    g_rootCLOut = NULL;
    for (p = 0; p < nPat; p++) {
        double like = 0.0;
        int rootCode = isLeaf[root] ? patterns[(size_t)seqNum[root] * nPat + p] : GAP_CODE;
        for (c = 0; c < nCat; c++)
            for (s = 0; s < dim; s++) {
                int use;
                if (rootCode >= 0) use = (s == rootCode);
                else if (rootCode == GAP_CODE || rootCode == QMARK_CODE) use = 1;
                else {
                    int e = rootCode - EQUATES_BASE;
                    use = isNLike(equates, dim, e) ? 1 : equates[e * dim + s];
                }
                if (use) like += rootComp[s] * cl[root][((size_t)c * dim + s) * nPat + p];
                if (catWork) {   /* Pf/p4_tree.c:1513-1516: per category, every state */
                    if (s == 0) catWork[(size_t)p * nCat + c] = 0.0;
                    catWork[(size_t)p * nCat + c] += rootComp[s] * cl[root][((size_t)c * dim + s) * nPat + p];
                }
            }
        if (pInvar != 0.0) {
            like *= (1.0 - pInvar) / (double)nCat;
            if (invarVec[p] > 0)
                for (s = 0; s < dim; s++)
                    if (invarArr[(size_t)s * nPat + p]) like += rootComp[s] * pInvar;
        } else if (nCat > 1) {
            like = like / (double)nCat;
        }
        if (like <= 0.0) {
            lnL = -1.0e99;
            break;
        }
        lnL = lnL + counts[p] * log(like);
        if (patLikes) patLikes[p] = like;
    }
    for (k = 0; k < nNodes; k++) free(cl[k]);
    free(cl);
    return lnL;
}

/* ---------------------------------------------- FP32 mirror of the GPU path */

typedef struct {
    int dim, nCat, nPartial, nPat;
    int root, cherries;   /* cherries: no rescale at a non-root node whose only children are two leaves */
    const int *leftChild, *sibling, *isLeaf, *seqNum;
    const float *decks, *eqTab;
    const uint8_t *ccodes;
    float *slots; /* stack of saved partial products, nCat*dim each */
    int sp;
} mirror_ctx;

static void mirror_tip(const mirror_ctx *m, int leaf, int p, float *out)
{
    int dim = m->dim, c, s;
    int code = m->ccodes[(size_t)m->seqNum[leaf] * m->nPat + p];
    for (c = 0; c < m->nCat; c++)
        for (s = 0; s < dim; s++) {
            float v;
            if (code < dim) v = m->decks[(((size_t)leaf * m->nCat + c) * dim + s) * dim + code];
            else if (code == dim) v = 1.0f;
            else v = m->eqTab[(((size_t)leaf * m->nPartial + (code - dim - 1)) * m->nCat + c) * dim + s];
            out[c * dim + s] = v;
        }
}

static void mirror_xform(const mirror_ctx *m, int node, float *acc)
{
    /* out[s] = P[s][0]*x[0], then fmaf over j = 1..dim-1 */
    int dim = m->dim, c, s, j;
    float x[64];
    for (c = 0; c < m->nCat; c++) {
        const float *P = m->decks + ((size_t)node * m->nCat + c) * dim * dim;
        for (j = 0; j < dim; j++) x[j] = acc[c * dim + j];
        for (s = 0; s < dim; s++) {
            float t = P[s * dim] * x[0];
            for (j = 1; j < dim; j++) t = fmaf(P[s * dim + j], x[j], t);
            acc[c * dim + s] = t;
        }
    }
}

static int need_slots(const mirror_ctx *m, int v, int *need)
{
    int ch, best = 0, second = 0, n;
    for (ch = m->leftChild[v]; ch >= 0; ch = m->sibling[ch]) {
        if (m->isLeaf[ch]) continue;
        n = need_slots(m, ch, need);
        if (n > best) { second = best; best = n; }
        else if (n > second) second = n;
    }
    /* first child uses its own need; every later one needs one more slot */
    n = best;
    {
        int cnt = 0;
        for (ch = m->leftChild[v]; ch >= 0; ch = m->sibling[ch])
            if (!m->isLeaf[ch]) cnt++;
        if (cnt >= 2 && second + 1 > n) n = second + 1;
    }
    need[v] = n;
    return n;
}

/* Internal children in order of decreasing need (stable in sibling order). */
static int ordered_internal(const mirror_ctx *m, int v, const int *need, int *out)
{
    int n = 0, ch, i, j;
    for (ch = m->leftChild[v]; ch >= 0; ch = m->sibling[ch])
        if (!m->isLeaf[ch]) out[n++] = ch;
    for (i = 1; i < n; i++) {
        int x = out[i];
        for (j = i - 1; j >= 0 && need[out[j]] < need[x]; j--) out[j + 1] = out[j];
        out[j + 1] = x;
    }
    return n;
}

static void mirror_scale(int n, float *acc, int *E)
{
    float mx = 0.0f;
    int i;
    for (i = 0; i < n; i++) mx = fmaxf(mx, acc[i]);
    if (mx < ldexpf(1.0f, -PORT_SCALE_LOG2) && mx > 0.0f) {
        uint32_t bits;
        int e2, k;
        float probe = mx;
        int pre = 0;
        memcpy(&bits, &probe, 4);
        if (((bits >> 23) & 0xff) == 0) { /* subnormal: lift by 2^64 first */
            probe = mx * 18446744073709551616.0f;
            memcpy(&bits, &probe, 4);
            pre = 64;
        }
        e2 = (int)((bits >> 23) & 0xff) - 126 - pre; /* mx = f * 2^e2, f in [0.5,1) */
        k = -e2;
        *E += k;
        while (k > 0) {
            int step = k > 100 ? 100 : k;
            float f = ldexpf(1.0f, step);
            for (i = 0; i < n; i++) acc[i] = acc[i] * f;
            k -= step;
        }
    }
}

static void mirror_eval(mirror_ctx *m, int v, const int *need, int p, float *acc, int *E)
{
    int nk = 0, i, ch, first = 1, n = m->nCat * m->dim;
    int *kids;
    float *tmp = malloc(sizeof(float) * n);
    for (ch = m->leftChild[v]; ch >= 0; ch = m->sibling[ch]) nk++;
    kids = malloc(sizeof(int) * (nk + 1));
    nk = ordered_internal(m, v, need, kids);
    for (i = 0; i < nk; i++) {
        float *slot = NULL;
        if (!first) {
            slot = m->slots + (size_t)(m->sp++) * n;
            memcpy(slot, acc, sizeof(float) * n);
        }
        mirror_eval(m, kids[i], need, p, acc, E);
        mirror_xform(m, kids[i], acc);
        if (!first) {
            int q;
            for (q = 0; q < n; q++) acc[q] = acc[q] * slot[q];
            m->sp--;
        }
        first = 0;
    }
    for (ch = m->leftChild[v]; ch >= 0; ch = m->sibling[ch]) {
        if (!m->isLeaf[ch]) continue;
        if (first) {
            mirror_tip(m, ch, p, acc);
            first = 0;
        } else {
            int q;
            mirror_tip(m, ch, p, tmp);
            for (q = 0; q < n; q++) acc[q] = acc[q] * tmp[q];
        }
    }
    {
        /* the GPU program reads a cherry's transformed product from a table
           computed without the rescale step (an exact power-of-two scaling,
           so only where later rescales happen differs) */
        int a = m->leftChild[v], b = a >= 0 ? m->sibling[a] : -1;
        int cherry = m->cherries && v != m->root && a >= 0 && m->isLeaf[a] && b >= 0 && m->isLeaf[b] &&
                     m->sibling[b] < 0;
        if (!cherry) mirror_scale(n, acc, E);
    }
    free(kids);
    free(tmp);
}

static float frexp32(float x, int *e)
{
    uint32_t b;
    int pre = 0;
    memcpy(&b, &x, 4);
    if (((b >> 23) & 0xffu) == 0u) {
        x = x * 18446744073709551616.0f;
        memcpy(&b, &x, 4);
        pre = 64;
    }
    *e = (int)((b >> 23) & 0xffu) - 126 - pre;
    b = (b & 0x807fffffu) | (126u << 23);
    memcpy(&x, &b, 4);
    return x;
}

double port_partPrune32(int nNodes, int root, const int *leftChild, const int *sibling,
                        const int *isLeaf, const int *seqNum, int dim, int nCat, int nPat,
                        int nPartial, const float *decks32, const float *eqTab32,
                        const uint8_t *ccodes, const double *rootComp, double pInvar,
                        const uint32_t *partialMask, const uint32_t *invMask,
                        const double *counts, float *likeScaled, int *exps, double *lnl, int cherries)
{
    mirror_ctx m;
    int *need = calloc(nNodes, sizeof(int));
    int n = nCat * dim, p, c, s, bad = 0;
    float *acc = malloc(sizeof(float) * n);
    float pi32[64];
    double total = 0.0;
    const double LN2 = 0.693147180559945309417232121458;
    const double varScale = (1.0 - pInvar) / (double)nCat;
    const double logScale = (pInvar != 0.0) ? log(varScale) : (nCat > 1 ? log(1.0 / nCat) : 0.0);
    m.dim = dim; m.nCat = nCat; m.nPartial = nPartial; m.nPat = nPat;
    m.root = root; m.cherries = cherries;
    m.leftChild = leftChild; m.sibling = sibling; m.isLeaf = isLeaf; m.seqNum = seqNum;
    m.decks = decks32; m.eqTab = eqTab32; m.ccodes = ccodes;
    m.slots = malloc(sizeof(float) * n * (nNodes + 1));
    m.sp = 0;
    for (s = 0; s < dim; s++) pi32[s] = (float)rootComp[s];
    need_slots(&m, root, need);
    for (p = 0; p < nPat; p++) {
        int E = 0;
        float like32 = 0.0f;
        double l;
        uint32_t rmask = dim >= 32 ? 0xffffffffu : ((1u << dim) - 1u);
        uint32_t im = (pInvar != 0.0) ? invMask[p] : 0u;
        mirror_eval(&m, root, need, p, acc, &E);
        if (isLeaf[root]) {
            int code = ccodes[(size_t)seqNum[root] * nPat + p];
            if (code < dim) rmask = 1u << code;
            else if (code > dim) rmask = partialMask[code - dim - 1];
        }
        for (c = 0; c < nCat; c++)
            for (s = 0; s < dim; s++)
                if ((rmask >> s) & 1u) like32 = fmaf(pi32[s], acc[c * dim + s], like32);
        if (im) {
            double lt = ldexp((double)like32, -E) * varScale;
            for (s = 0; s < dim; s++)
                if ((im >> s) & 1u) lt = lt + rootComp[s] * pInvar;
            if (!(lt > 0.0)) bad = 1;
            l = log(lt);
        } else {
            int e;
            float mm;
            if (!(like32 > 0.0f)) bad = 1;
            mm = frexp32(like32, &e);
            l = (double)logf(mm) + (double)(e - E) * LN2 + logScale;
        }
        likeScaled[p] = like32;
        exps[p] = E;
        lnl[p] = l;
        total = total + counts[p] * l;
    }
    free(m.slots);
    free(acc);
    free(need);
    return bad ? -1.0e99 : total;
}
