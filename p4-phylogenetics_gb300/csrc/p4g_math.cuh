// FP64 special functions for the discrete-gamma category rates, usable on the
// host (p4g_gdasrvCalcRates) and on the device (setPrams kernel).
//
// p4 computes the rates with Yang's DiscreteGamma (Pf/gamma.c:17-50): equal-
// probability bins of Gamma(alpha, alpha), rate = mean of the bin.  The cut
// points come from the AS91 chi-square quantile (Best & Roberts 1975) seeded
// by the AS70 normal quantile (Odeh & Evans 1974); bin means from the AS32
// incomplete gamma ratio (Bhattacharjee 1970) of alpha+1; log gamma from ACM
// algorithm 291 (Pike & Hill 1966).  AS91 iterates to a relative tolerance of
// 5e-7, so the same iteration structure is kept here: a different quantile
// method would move the rates by up to ~1e-6 and the lnL with them.
// Every iteration is capped; a non-converging input returns an error.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define P4G_HD __host__ __device__
#else
#define P4G_HD
#endif

namespace p4g {

P4G_HD inline double gm_lnGamma(double alpha)
{
    double x = alpha, f = 0.0, z;
    if (x < 7.0) {
        f = 1.0;
        z = x - 1.0;
        for (int it = 0; it < 16; it++) {
            z += 1.0;
            if (!(z < 7.0)) break;
            f *= z;
        }
        x = z;
        f = -log(f);
    }
    z = 1.0 / (x * x);
    // Stirling series: 1/12, -1/360, 1/1260, -1/1680 and ln sqrt(2 pi)
    return f + (x - 0.5) * log(x) - x + 0.918938533204673 +
           (((-0.000595238095238 * z + 0.000793650793651) * z - 0.002777777777778) * z +
            0.083333333333333) / x;
}

// The part of the regularised lower incomplete gamma P(p, x) that does not
// need its prefactor exp(p log x - x - lnGamma(p)): the power series' sum
// (kind 0, P = gin * (factor / p)) or the continued fraction's value (kind
// 1, P = 1 - factor * gin).  Kind 2: x == 0, P = 0; kind -1: an error.
P4G_HD inline int gm_incGammaCore(double x, double p, double *ginOut)
{
    const double accurate = 1e-8, overflow = 1e30;
    if (x == 0.0) return 2;
    if (x < 0 || p <= 0) return -1;
    if (!(x > 1 && x >= p)) {  // power series
        // the quotients x / rn of four consecutive terms do not depend on
        // the running product, so they are formed together (their latencies
        // overlap); the terms are then taken one at a time, in order
        double gin = 1.0, term = 1.0, rn = p;
        for (int it = 0; it < 200000; it += 4) {
            const double r1 = rn + 1.0, r2 = r1 + 1.0, r3 = r2 + 1.0, r4 = r3 + 1.0;
            const double q[4] = {x / r1, x / r2, x / r3, x / r4};
            rn = r4;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                term *= q[k];
                gin += term;
                if (!(term > accurate)) {
                    *ginOut = gin;
                    return 0;
                }
            }
        }
        return -1;
    }
    // continued fraction
    double a = 1.0 - p, b = a + x + 1.0, term = 0.0, pn[6];
    pn[0] = 1.0;
    pn[1] = x;
    pn[2] = x + 1;
    pn[3] = x * b;
    double gin = pn[2] / pn[3];
    for (int it = 0; it < 200000; it++) {
        a += 1.0;
        b += 2.0;
        term += 1.0;
        double an = a * term;
        pn[4] = b * pn[2] - an * pn[0];
        pn[5] = b * pn[3] - an * pn[1];
        if (pn[5] != 0) {
            double rn = pn[4] / pn[5];
            double dif = fabs(gin - rn);
            if (!(dif > accurate) && dif <= accurate * rn) {
                *ginOut = gin;
                return 1;
            }
            gin = rn;
        }
        pn[0] = pn[2];
        pn[1] = pn[3];
        pn[2] = pn[4];
        pn[3] = pn[5];
        if (!(fabs(pn[4]) < overflow)) {
            pn[0] /= overflow;
            pn[1] /= overflow;
            pn[2] /= overflow;
            pn[3] /= overflow;
        }
    }
    return -1;
}

// The incomplete gamma from its core and prefactor.
P4G_HD inline double gm_incGammaFinish(int kind, double gin, double factor, double p)
{
    if (kind == 2) return 0.0;
    if (kind < 0) return -1.0;
    return kind == 0 ? gin * (factor / p) : 1.0 - factor * gin;
}

// The prefactor exp(p log x - x - lnGamma(p)).
P4G_HD inline double gm_incGammaFactor(double x, double p, double lnGammaP)
{
    return exp(p * log(x) - x - lnGammaP);
}

// Regularised lower incomplete gamma P(p, x); -1 on error.
P4G_HD inline double gm_incGamma(double x, double p, double lnGammaP)
{
    double gin = 0.0;
    const int kind = gm_incGammaCore(x, p, &gin);
    if (kind == 2 || kind < 0) return gm_incGammaFinish(kind, gin, 0.0, p);
    return gm_incGammaFinish(kind, gin, gm_incGammaFactor(x, p, lnGammaP), p);
}

P4G_HD inline double gm_normalQuantile(double prob)
{
    const double a0 = -0.322232431088, a1 = -1.0, a2 = -0.342242088547,
                 a3 = -0.0204231210245, a4 = -0.453642210148e-4, b0 = 0.0993484626060,
                 b1 = 0.588581570495, b2 = 0.531103462366, b3 = 0.103537752850,
                 b4 = 0.0038560700634;
    double p1 = prob < 0.5 ? prob : 1 - prob;
    if (p1 < 1e-20) return -9999;
    double y = sqrt(log(1 / (p1 * p1)));
    double z = y + ((((y * a4 + a3) * y + a2) * y + a1) * y + a0) /
                       ((((y * b4 + b3) * y + b2) * y + b1) * y + b0);
    return prob < 0.5 ? -z : z;
}

// AS91 set-up for the chi-square quantile with v degrees of freedom: the
// starting point *ch and lnGamma(v/2).  Returns 0 (iterate from *ch), 1 (*ch
// is the quantile already) or -1 (an error).
P4G_HD inline int gm_chi2Start(double prob, double v, double *chOut, double *gOut)
{
    const double e = 0.5e-6, aa = 0.6931471805;
    double p = prob, ch, a = 0, q, p1, p2, t;
    if (p < 0.000002 || p > 0.999998 || v <= 0.0) return -1;
    double g = gm_lnGamma(v / 2.0);
    double xx = v / 2.0;
    double c = xx - 1.0;
    *gOut = g;
    if (v < -1.24 * log(p)) {
        ch = pow(p * xx * exp(g + xx * aa), 1.0 / xx);
        if (ch - e < 0) {
            *chOut = ch;
            return 1;
        }
    } else if (v <= 0.32) {
        ch = 0.4;
        a = log(1.0 - p);
        int it = 0;
        for (; it < 200000; it++) {
            q = ch;
            p1 = 1.0 + ch * (4.67 + ch);
            p2 = ch * (6.73 + ch * (6.66 + ch));
            t = -0.5 + (4.67 + 2.0 * ch) / p1 - (6.73 + ch * (13.32 + 3.0 * ch)) / p2;
            ch -= (1.0 - exp(a + g + 0.5 * ch + c * aa) * p2 / p1) / t;
            if (fabs(q / ch - 1.0) - 0.01 <= 0.0) break;
        }
        if (it == 200000) return -1;
    } else {
        double x = gm_normalQuantile(p);
        p1 = 0.222222 / v;
        ch = v * pow((x * sqrt(p1) + 1.0 - p1), 3.0);
        if (ch > 2.2 * v + 6.0) ch = -2.0 * (log(1.0 - p) - c * log(0.5 * ch) + g);
    }
    *chOut = ch;
    return 0;
}

// exp(xx ln 2 + g + ch/2 - (xx - 1) log ch), xx = v/2: the factor of one AS91
// step that does not depend on the incomplete gamma.
P4G_HD inline double gm_chi2StepFactor(double v, double g, double ch)
{
    const double aa = 0.6931471805;
    const double xx = v / 2.0, c = xx - 1.0;
    return exp(xx * aa + g + 0.5 * ch - c * log(ch));
}

// One AS91 step from *ch, given t = P(v/2, ch/2) and e2 = gm_chi2StepFactor:
// 1 when converged (*ch is the quantile), 0 to go on, -1 on an error.
P4G_HD inline int gm_chi2Step(double prob, double v, double t, double e2, double *ch)
{
    const double e = 0.5e-6;
    const double xx = v / 2.0, c = xx - 1.0;
    if (t < 0.0) return -1;
    const double q = *ch;
    const double p2 = prob - t;
    t = p2 * e2;
    double b = t / q;
    double a = 0.5 * t - b * c;
    double s1 = (210.0 + a * (140.0 + a * (105.0 + a * (84.0 + a * (70.0 + 60.0 * a))))) / 420.0;
    double s2 = (420.0 + a * (735.0 + a * (966.0 + a * (1141.0 + 1278.0 * a)))) / 2520.0;
    double s3 = (210.0 + a * (462.0 + a * (707.0 + 932.0 * a))) / 2520.0;
    double s4 = (252.0 + a * (672.0 + 1182.0 * a) + c * (294.0 + a * (889.0 + 1740.0 * a))) / 5040.0;
    double s5 = (84.0 + 264.0 * a + c * (175.0 + 606.0 * a)) / 2520.0;
    double s6 = (120.0 + c * (346.0 + 127.0 * c)) / 5040.0;
    const double nch = q + t * (1 + 0.5 * t * s1 - b * c * (s1 - b * (s2 - b * (s3 - b * (s4 - b * (s5 - b * s6))))));
    *ch = nch;
    return !(fabs(q / nch - 1.0) > e) ? 1 : 0;
}

// Chi-square quantile with v degrees of freedom; -1 on error.
P4G_HD inline double gm_chi2Quantile(double prob, double v)
{
    double ch = 0.0, g = 0.0;
    const int st = gm_chi2Start(prob, v, &ch, &g);
    if (st < 0) return -1.0;
    if (st == 1) return ch;
    const double xx = v / 2.0;
    for (int it = 0; it < 200000; it++) {
        const double t = gm_incGamma(0.5 * ch, xx, g);
        if (t < 0.0) return -1.0;
        const int r = gm_chi2Step(prob, v, t, gm_chi2StepFactor(v, g, ch), &ch);
        if (r < 0) return -1.0;
        if (r > 0) return ch;
    }
    return -1.0;
}

// K equal-probability categories of Gamma(alpha, alpha), rate = bin mean.
// cut[] is caller scratch of K entries.  Returns 0 or -1.
P4G_HD inline int gm_discreteGamma(double alpha, int K, double *rates, double *cut)
{
    if (K < 1 || !(alpha > 0)) return -1;
    if (K == 1) {
        rates[0] = 1.0;
        return 0;
    }
    double factor = alpha / alpha * K;
    double lnga1 = gm_lnGamma(alpha + 1);
    for (int i = 0; i < K - 1; i++) {
        double ch = gm_chi2Quantile((i + 1.0) / K, 2.0 * alpha);
        if (ch < 0) return -1;
        cut[i] = ch / (2.0 * alpha);
    }
    for (int i = 0; i < K - 1; i++) {
        cut[i] = gm_incGamma(cut[i] * alpha, alpha + 1, lnga1);
        if (cut[i] < 0) return -1;
    }
    rates[0] = cut[0] * factor;
    rates[K - 1] = (1 - cut[K - 2]) * factor;
    for (int i = 1; i < K - 1; i++) rates[i] = (cut[i] - cut[i - 1]) * factor;
    return 0;
}

}  // namespace p4g
