// setPrams on the GPU: discrete-gamma rates, Q and its eigensystem, and the
// P = exp(Qt) decks of every (part, node, category), with FP64-accurate
// results.
//
// Reference: p4_setPramsPart (Pf/p4_tree.c:218-541) computes the gamma rates
// with DiscreteGamma, builds Q = R.diag(pi) and normalises it
// (Pf/util.c:44-115), takes a general real eigensystem of Q
// (Pf/eig.c:63-161) and then P(t) = V exp(lambda t) V^-1 for every node and
// category (Pf/p4_node.c:296-346, Pf/eig.c:163-223).
//
// Here Q is reversible (R symmetric, pi > 0), so the eigensystem is taken of
// the symmetric S = diag(sqrt pi) Q diag(1/sqrt pi): by cyclic Jacobi in FP64
// (round-robin pair ordering, all D/2 disjoint rotations of a round applied
// together) up to 8 states, and above that by FP32 Jacobi sweeps refined to
// FP64 accuracy with FP64 matrix products (eigBlock).  P(t)_ij =
// sum_k U_ik e^{lambda_k t} U_jk sqrt(pi_j/pi_i) is formed in FP32-pair
// arithmetic (k_pdeck); the FP64 decks are its values, the FP32 decks the
// pruning kernels read are the same values rounded to FP32.  This GPU's FP64
// pipe is narrow, so FP64 is used where a result needs it and FP32 elsewhere;
// the gamma rates follow the reference's iterations in FP64 step for step.
#include <cuda_runtime.h>
#include <algorithm>
#include <cfloat>
#include "p4g_internal.h"
#include "p4g_math.cuh"
#include "p4g_pmat.cuh"
#include "p4g_prune_common.cuh"
#include "p4g_tc.cuh"

namespace p4g {

// ----------------------------------------------------------------- helpers
__device__ __forceinline__ int findDesc(const int *prefix, int n, int idx)
{
    // largest d with prefix[d] <= idx
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= idx) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ----------------------------------------------------------------- gamma
// One warp per (part, gdasrv).  Cut point k < K-1 is the chi-square quantile
// at (k+1)/K, then the incomplete gamma ratio of alpha+1 at it; lane 0 forms
// the bin means.  With K <= 11 three lanes work on each cut point (lane
// 10r + k, role r): every AS91 step needs the incomplete gamma's series or
// continued fraction (role 0), that function's prefactor (role 1) and the
// step's own exp/log factor (role 2), three chains that do not depend on one
// another, so they run side by side and role 0 combines them.  Every value is
// formed by the same operations as in the serial gm_discreteGamma.
__device__ void gammaWarp(const PmatPart &P, int g, int *status, double *cut)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int K = P.nCat;
    const double alpha = P.gval[g];
    int bad = 0;
    if (K - 1 <= 10) {
        const int role = lane / 10, k = lane % 10;
        const bool mine = role < 3 && k < K - 1;
        const double prob = (k + 1.0) / K, v = 2.0 * alpha, xx = v / 2.0;
        double ch = 0.0, lg = 0.0;
        const int st = mine ? gm_chi2Start(prob, v, &ch, &lg) : 1;   // the same on all three roles
        int done = st != 0;
        double res = st == 1 ? ch : -1.0;
        for (int it = 0; it < 200000; it++) {
            if (__all_sync(FULL, done)) break;
            double gin = 0.0, f = 0.0, e2 = 0.0;
            int kind = 0;
            if (!done) {
                if (role == 0) kind = gm_incGammaCore(0.5 * ch, xx, &gin);
                else if (role == 1) f = gm_incGammaFactor(0.5 * ch, xx, lg);
                else e2 = gm_chi2StepFactor(v, lg, ch);
            }
            f = __shfl_sync(FULL, f, (10 + k) & 31);
            e2 = __shfl_sync(FULL, e2, (20 + k) & 31);
            if (role == 0 && !done) {
                const int r = gm_chi2Step(prob, v, gm_incGammaFinish(kind, gin, f, xx), e2, &ch);
                if (r != 0) {
                    done = 1;
                    res = r > 0 ? ch : -1.0;
                }
            }
            ch = __shfl_sync(FULL, ch, k);   // roles 1 and 2 follow their role 0
            done = __shfl_sync(FULL, done, k);
            if (!mine) done = 1;
        }
        // bin means: P(alpha+1, ch/2) with the same two-lane split
        const double chq = __shfl_sync(FULL, res, k);
        const double x = (chq / (2.0 * alpha)) * alpha;
        const double lga1 = gm_lnGamma(alpha + 1);
        double gin = 0.0, f = 0.0;
        int kind = -1;
        if (mine && chq >= 0) {
            if (role == 0) kind = gm_incGammaCore(x, alpha + 1, &gin);
            else if (role == 1) f = gm_incGammaFactor(x, alpha + 1, lga1);
        }
        f = __shfl_sync(FULL, f, (10 + k) & 31);
        if (mine && role == 0) {
            const double cv = (chq < 0) ? -1.0 : gm_incGammaFinish(kind, gin, f, alpha + 1);
            cut[k] = cv;
            bad = (chq < 0) || (cv < 0);
        }
    } else if (lane < K - 1) {
        double ch = gm_chi2Quantile((lane + 1.0) / K, 2.0 * alpha);
        double c = ch / (2.0 * alpha);
        double v = (ch < 0) ? -1.0 : gm_incGamma(c * alpha, alpha + 1, gm_lnGamma(alpha + 1));
        cut[lane] = v;
        bad = (ch < 0) || (v < 0);
    }
    bad = __any_sync(FULL, bad);
    __syncwarp();
    if (lane == 0) {
        double *r = P.rates + g * K;
        if (bad || !(alpha > 0)) {
            atomicOr(status, 1);
            for (int c = 0; c < K; c++) r[c] = 0.0;
        } else if (K == 1) {
            r[0] = 1.0;
        } else {
            const double factor = alpha / alpha * K;
            r[0] = cut[0] * factor;
            r[K - 1] = (1 - cut[K - 2]) * factor;
            for (int i = 1; i < K - 1; i++) r[i] = (cut[i] - cut[i - 1]) * factor;
        }
    }
}

// ----------------------------------------------------------------- eig
// One block per (part, comp, rMatrix): one warp for dim <= 8, eight warps for
// larger dims (a sweep round's 2x2-block and (row, pair) updates one per
// thread for 20 states; measured 216 k -> 197 k cycles per protein
// eigensystem against four warps).  Shared memory: S[dim*dim], U[dim*dim], 32 rotations (c, s, p,
// q), pi, sqrt(pi), the warps' partial sums, then (larger dims) T, W and V
// [dim*dim] each for the mixed-precision start and its refinement.
constexpr int EIG_SMALL_DIM = 8;
constexpr int EIG_THREADS_LARGE = 256;
__host__ __device__ inline int eigThreads(int maxDim) { return maxDim <= EIG_SMALL_DIM ? 32 : EIG_THREADS_LARGE; }
__host__ __device__ inline size_t eigSmemDoubles(int maxDim)
{
    return (size_t)5 * maxDim * maxDim + 4 * 32 + 2 * maxDim + 64;
}

// Rotation (c, s) that zeroes S_pq of the symmetric 2x2 block [a_pp a_pq; a_pq a_qq]:
// t = sgn(d) 2 a_pq / (|d| + sqrt(d^2 + 4 a_pq^2)), d = a_qq - a_pp, the smaller
// root, as (c, s) = (u, sgn(d) 2 a_pq) / sqrt(u^2 + 4 a_pq^2) with u = |d| + sqrt(.)
// (one square root and one reciprocal square root).
__device__ __forceinline__ float absT(float x) { return fabsf(x); }
__device__ __forceinline__ double absT(double x) { return fabs(x); }
__device__ __forceinline__ float sqrtT(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrtT(double x) { return sqrt(x); }
__device__ __forceinline__ float rsqrtT(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrtT(double x) { return rsqrt(x); }

template <typename T>
__device__ __forceinline__ void jacobiRotation(T app, T aqq, T apq, T &c, T &s)
{
    const T dd = aqq - app;
    const T r2 = (T)2 * apq;
    const T u = absT(dd) + sqrtT(dd * dd + r2 * r2);
    const T inv = rsqrtT(u * u + r2 * r2);
    c = u * inv;
    s = (dd >= (T)0 ? r2 : -r2) * inv;
}

// Round r of the round-robin ordering over m (even) players: the tid-th pair.
__device__ __forceinline__ void rrPair(int r, int tid, int m, int &p, int &q)
{
    int a = (tid == 0) ? m - 1 : (r + tid) % (m - 1);
    int b = (r + m - 1 - tid) % (m - 1);
    if (tid == 0) b = r % (m - 1);
    p = a < b ? a : b;
    q = a < b ? b : a;
}

// The off-diagonal and diagonal squared masses of S, summed over the block
// (warps' partials through red[]).
template <typename T>
__device__ __forceinline__ void offDiagMass(const T *S, int n, double *red, double &off, double &dg)
{
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    double o = 0.0, g = 0.0;
    for (int k = tid; k < n * n; k += nt) {
        const int i = k / n, j = k % n;
        const double v = (double)S[k];
        if (i == j) g += v * v;
        else if (i < j) o += v * v;
    }
    for (int x = 16; x; x >>= 1) {
        o += __shfl_xor_sync(0xffffffffu, o, x);
        g += __shfl_xor_sync(0xffffffffu, g, x);
    }
    if (lane == 0) {
        red[2 * warp] = o;
        red[2 * warp + 1] = g;
    }
    __syncthreads();
    off = 0.0;
    dg = 0.0;
    for (int w = 0; w < nw; w++) {
        off += red[2 * w];
        dg += red[2 * w + 1];
    }
    __syncthreads();   // every thread has read the sums before they are written again
}

// One Jacobi sweep (m - 1 rounds of n/2 disjoint rotations) on S, accumulated
// into U.  rc, rs, rp, rq: the round's rotations.  classical: an element below
// the rounding of both diagonal entries is set to zero instead of rotated.
template <typename T>
__device__ void jacobiSweep(T *S, T *U, int n, T *rc, T *rs, int *rp, int *rq, bool classical)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int m = (n + 1) & ~1, npairs = m / 2;
    for (int r = 0; r < m - 1; r++) {
        if (tid < npairs) {
            int p, q;
            rrPair(r, tid, m, p, q);
            T c = (T)1, sn = (T)0;
            if (q < n) {
                const T apq = S[p * n + q];
                const T g = (T)100 * absT(apq);
                if (classical && apq != (T)0 && absT(S[p * n + p]) + g == absT(S[p * n + p]) &&
                    absT(S[q * n + q]) + g == absT(S[q * n + q])) {
                    S[p * n + q] = (T)0;
                    S[q * n + p] = (T)0;
                } else if (apq != (T)0) {
                    jacobiRotation<T>(S[p * n + p], S[q * n + q], apq, c, sn);
                }
            }
            rp[tid] = p;
            rq[tid] = q;
            rc[tid] = c;
            rs[tid] = sn;
        }
        __syncthreads();
        // columns p, q of S and U: one (pair, row) per thread
        for (int k = tid; k < npairs * n; k += nt) {
            const int pr = k / n, row = k - pr * n;
            const int p = rp[pr], q = rq[pr];
            if (q >= n) continue;
            const T c = rc[pr], sn = rs[pr];
            const T a = S[row * n + p], b = S[row * n + q];
            S[row * n + p] = c * a - sn * b;
            S[row * n + q] = sn * a + c * b;
            const T ua = U[row * n + p], ub = U[row * n + q];
            U[row * n + p] = c * ua - sn * ub;
            U[row * n + q] = sn * ua + c * ub;
        }
        __syncthreads();
        // rows p, q of S: one (pair, column) per thread
        for (int k = tid; k < npairs * n; k += nt) {
            const int pr = k / n, col = k - pr * n;
            const int p = rp[pr], q = rq[pr];
            if (q >= n) continue;
            const T c = rc[pr], sn = rs[pr];
            const T a = S[p * n + col], b = S[q * n + col];
            S[p * n + col] = c * a - sn * b;
            S[q * n + col] = sn * a + c * b;
        }
        __syncthreads();
    }
}

// One Jacobi sweep in FP32 over the block, S kept exactly symmetric.  sched:
// the sweep's round-robin schedule, (p | q << 8) for round r, pair k at
// [r * npairs + k].  Per round: the first n/2 threads find the round's
// rotations; then, in one phase, a thread applies both rotations of one 2x2
// block of S (row pair k <= column pair l: S_block <- J_k^T S_block J_l,
// written with its mirror) or the column rotation of one (row, pair) piece of U.
// No thread reads a block another thread writes, so a round needs two block
// barriers.  Each thread's tasks are the same in every round (only the pairs'
// indices change), so they are decoded once.
__device__ void jacobiSweepPairs(float *S, float *U, int n, float *rc, float *rs, int *rp, int *rq,
                                 const int *sched)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int m = (n + 1) & ~1, npairs = m / 2;
    const int nS = npairs * (npairs + 1) / 2, nTask = nS + n * npairs;
    // tasks tid + j nt (j < SWEEP_TASKS: n <= MAX_DIM = 32 gives at most 648 tasks for
    // the EIG_THREADS_LARGE threads of a block): t < nS an S block (k, l), else a U
    // piece (row a, pair l)
    constexpr int SWEEP_TASKS = 3;
    static_assert((MAX_DIM / 2) * (MAX_DIM / 2 + 1) / 2 + MAX_DIM * (MAX_DIM / 2) <= SWEEP_TASKS * EIG_THREADS_LARGE,
                  "every task of a sweep has a thread");
    int ta[SWEEP_TASKS], tb[SWEEP_TASKS];
    bool isS[SWEEP_TASKS], has[SWEEP_TASKS];
#pragma unroll
    for (int j = 0; j < SWEEP_TASKS; j++) {
        const int t = tid + j * nt;
        has[j] = t < nTask;
        isS[j] = t < nS;
        ta[j] = tb[j] = 0;
        if (has[j] && isS[j]) {   // t -> (k, l), k <= l, row by row of the upper triangle
            int k = 0, rem = t;
            while (rem >= npairs - k) {
                rem -= npairs - k;
                k++;
            }
            ta[j] = k;
            tb[j] = k + rem;
        } else if (has[j]) {
            ta[j] = (t - nS) / npairs;
            tb[j] = (t - nS) - ta[j] * npairs;
        }
    }
    for (int r = 0; r < m - 1; r++) {
        if (tid < npairs) {
            const int pq = sched[r * npairs + tid];
            const int p = pq & 0xff, q = pq >> 8;
            float c = 1.f, sn = 0.f;
            if (q < n) {
                const float apq = S[p * n + q];
                if (apq != 0.f) jacobiRotation<float>(S[p * n + p], S[q * n + q], apq, c, sn);
            }
            rp[tid] = p;
            rq[tid] = q;
            rc[tid] = c;
            rs[tid] = sn;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < SWEEP_TASKS; j++) {
            if (!has[j]) continue;
            const int l = tb[j];
            const int p2 = rp[l], q2 = rq[l];
            const float c2 = rc[l], s2 = rs[l];
            const bool v2 = q2 < n;
            if (isS[j]) {
                const int k = ta[j];
                const int p1 = rp[k], q1 = rq[k];
                const float c1 = rc[k], s1 = rs[k];
                const bool v1 = q1 < n;
                const float m00 = S[p1 * n + p2];
                const float m01 = v2 ? S[p1 * n + q2] : 0.f;
                const float m10 = v1 ? S[q1 * n + p2] : 0.f;
                const float m11 = (v1 && v2) ? S[q1 * n + q2] : 0.f;
                // columns (S J_l), then rows (J_k^T .)
                const float t00 = c2 * m00 - s2 * m01, t01 = s2 * m00 + c2 * m01;
                const float t10 = c2 * m10 - s2 * m11, t11 = s2 * m10 + c2 * m11;
                const float n00 = c1 * t00 - s1 * t10, n01 = c1 * t01 - s1 * t11;
                const float n10 = s1 * t00 + c1 * t10, n11 = s1 * t01 + c1 * t11;
                S[p1 * n + p2] = n00;
                S[p2 * n + p1] = n00;
                if (v2) {
                    S[p1 * n + q2] = n01;
                    S[q2 * n + p1] = n01;
                }
                if (v1) {
                    S[q1 * n + p2] = n10;
                    S[p2 * n + q1] = n10;
                }
                if (v1 && v2) {
                    S[q1 * n + q2] = n11;
                    S[q2 * n + q1] = n11;
                }
            } else if (v2) {
                const int a = ta[j];
                const float ua = U[a * n + p2], ub = U[a * n + q2];
                U[a * n + p2] = c2 * ua - s2 * ub;
                U[a * n + q2] = s2 * ua + c2 * ub;
            }
        }
        __syncthreads();
    }
}

// The off-diagonal and diagonal squared masses of an FP32 S, summed in FP32
// over the block (a convergence test needs no more).
__device__ __forceinline__ void offDiagMass32(const float *S, int n, double *red, double &off, double &dg)
{
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    float o = 0.f, g = 0.f;
    for (int k = tid; k < n * n; k += nt) {
        const int i = k / n, j = k - i * n;
        const float v = S[k];
        if (i == j) g = fmaf(v, v, g);
        else if (i < j) o = fmaf(v, v, o);
    }
    for (int x = 16; x; x >>= 1) {
        o += __shfl_xor_sync(0xffffffffu, o, x);
        g += __shfl_xor_sync(0xffffffffu, g, x);
    }
    float *rf = (float *)red;
    if (lane == 0) {
        rf[2 * warp] = o;
        rf[2 * warp + 1] = g;
    }
    __syncthreads();
    float of = 0.f, gf = 0.f;
    for (int w = 0; w < nw; w++) {
        of += rf[2 * w];
        gf += rf[2 * w + 1];
    }
    off = of;
    dg = gf;
    __syncthreads();   // every thread has read the sums before they are written again
}

// C = A^T B (transA) or A B, n x n, row-major, every thread a strided set of outputs.
__device__ __forceinline__ void matmul64(double *C, const double *A, const double *B, int n, bool transA)
{
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
        const int i = k / n, j = k % n;
        double acc = 0.0;
        for (int l = 0; l < n; l++) acc += (transA ? A[l * n + i] : A[i * n + l]) * B[l * n + j];
        C[k] = acc;
    }
}

// A float's exact FP64 value assembled with integer operations (normal numbers
// and zeros; the rest through the conversion instruction).
__device__ __forceinline__ double floatToDouble(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu, man = u & 0x7fffffu;
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    if (ex == 0u && man == 0u) return __longlong_as_double((long long)sign);
    if (ex == 0u || ex == 0xffu) return (double)f;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(ex + 896u) << 52) |
                                            ((unsigned long long)man << 29)));
}

// A double rounded toward zero to FP32 with integer operations: magnitudes
// below FP32's normal range give a signed zero, larger ones the largest float,
// NaN and infinities go through the conversion instruction.
__device__ __forceinline__ float doubleToFloatRz(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int ex11 = (int)((b >> 52) & 0x7ffu);
    if (ex11 == 0x7ff) return (float)d;
    const int ex = ex11 - 1023 + 127;
    const unsigned sign = (unsigned)(b >> 63) << 31;
    if (ex <= 0) return __uint_as_float(sign);
    if (ex >= 255) return __uint_as_float(sign | 0x7f7fffffu);
    return __uint_as_float(sign | ((unsigned)ex << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

// C = A^T B (transA) or A B, n x n row-major; a thread computes a strip of four
// adjacent outputs of one row (four independent FMA chains sharing each A value).
// upper: the product is symmetric and only the strips that reach the upper
// triangle (j >= i) are formed; read it through symAt.
template <typename T>
__device__ __forceinline__ void matmulX4(T *C, const T *A, const T *B, int n, bool transA, bool upper)
{
    const int ns = (n + 3) >> 2;
    for (int k = threadIdx.x; k < n * ns; k += blockDim.x) {
        const int i = k / ns, j0 = (k - i * ns) * 4;
        if (upper && j0 + 3 < i) continue;
        const int w = min(4, n - j0);
        T c0 = 0, c1 = 0, c2 = 0, c3 = 0;
        for (int l = 0; l < n; l++) {
            const T a = transA ? A[l * n + i] : A[i * n + l];
            const T *b = B + l * n + j0;
            c0 += a * b[0];
            if (w > 1) c1 += a * b[1];
            if (w > 2) c2 += a * b[2];
            if (w > 3) c3 += a * b[3];
        }
        T *c = C + i * n + j0;
        c[0] = c0;
        if (w > 1) c[1] = c1;
        if (w > 2) c[2] = c2;
        if (w > 3) c[3] = c3;
    }
}

__device__ __forceinline__ double symAt(const double *C, int n, int i, int j)
{
    return i <= j ? C[i * n + j] : C[j * n + i];
}

// Sums (MAX false) or maxima (MAX true) of two per-thread values over the
// block, returned to every thread (warps' partials through red[]).
template <bool MAX>
__device__ __forceinline__ void blockReduce2(double &a, double &b, double *red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int x = 16; x; x >>= 1) {
        const double oa = __shfl_xor_sync(0xffffffffu, a, x), ob = __shfl_xor_sync(0xffffffffu, b, x);
        a = MAX ? fmax(a, oa) : a + oa;
        b = MAX ? fmax(b, ob) : b + ob;
    }
    if (lane == 0) {
        red[2 * warp] = a;
        red[2 * warp + 1] = b;
    }
    __syncthreads();
    a = red[0];
    b = red[1];
    for (int w = 1; w < nw; w++) {
        a = MAX ? fmax(a, red[2 * w]) : a + red[2 * w];
        b = MAX ? fmax(b, red[2 * w + 1]) : b + red[2 * w + 1];
    }
    __syncthreads();   // every thread has read the partials before they are written again
}

// blockReduce2 in FP32.
template <bool MAX>
__device__ __forceinline__ void blockReduce2f(float &a, float &b, double *red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int x = 16; x; x >>= 1) {
        const float oa = __shfl_xor_sync(0xffffffffu, a, x), ob = __shfl_xor_sync(0xffffffffu, b, x);
        a = MAX ? fmaxf(a, oa) : a + oa;
        b = MAX ? fmaxf(b, ob) : b + ob;
    }
    float *rf = (float *)red;
    if (lane == 0) {
        rf[2 * warp] = a;
        rf[2 * warp + 1] = b;
    }
    __syncthreads();
    a = rf[0];
    b = rf[1];
    for (int w = 1; w < nw; w++) {
        a = MAX ? fmaxf(a, rf[2 * w]) : a + rf[2 * w];
        b = MAX ? fmaxf(b, rf[2 * w + 1]) : b + rf[2 * w + 1];
    }
    __syncthreads();   // every thread has read the partials before they are written again
}

// One step of the iterative refinement of a symmetric eigendecomposition by
// Ogita and Aishima (Japan J. Indust. Appl. Math. 35, 2018, Algorithm 1).
// X holds approximate eigenvectors (columns) of the symmetric A:
//   R = I - X^T X,  S = X^T A X,  lam_i = s_ii / (1 - r_ii),
//   delta = 2 (||S - diag(lam)||_F + ||A||_F ||R||_F),
//   E_ij = (s_ij + lam_j r_ij) / (lam_j - lam_i) where |lam_j - lam_i| > delta,
//   E_ij = r_ij / 2 elsewhere (the diagonal, and pairs closer than delta),
//   X <- X + X E,
// convergent quadratically for separated eigenvalues.  R and S measure the
// residual and are formed in FP64 (upper triangles: both are symmetric), and so
// are lam and, per entry of E, the numerator and the gap; E itself, its products
// X E and the threshold delta are FP32: an error of relative size 1e-7 in E
// leaves an error of 1e-7 |E| in X, far below FP64 precision after the final
// step (whose E is of the order of the error the step before left) and
// corrected by the next step otherwise.  Every FP64 instruction counts on this
// GPU (its FP64 pipe is narrow), so the rest is FP32.
// Returns, to every thread, the largest |E_ij| over the separated pairs (emax;
// the step is applied only if it is at most maxApply) and the largest |s_ij| over
// the pairs closer than delta (cmax: the coupling the step leaves unresolved).
// lam[n] receives the eigenvalue estimates.  T, W, V: n x n FP64 scratch.
__device__ void refineStep(const double *A, double *X, double *T, double *W, double *V, double *lam, int n,
                           int maxDim, double normA, double maxApply, double *red, double &emax, double &cmax)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    matmulX4<double>(T, X, X, n, true, true);      // G = X^T X  (R = I - G)
    matmulX4<double>(W, A, X, n, false, false);    // A X
    __syncthreads();
    matmulX4<double>(V, X, W, n, true, true);      // S = X^T A X
    __syncthreads();
    // the eigenvalue estimates in FP64; the residual norms that set delta in
    // FP32 (a threshold needs no more)
    float so = 0.f, ro = 0.f;
    for (int k = tid; k < n * n; k += nt) {
        const int i = k / n, j = k - i * n;
        if (i > j) continue;
        const double v = V[k], g = T[k];
        if (i == j) {
            const double l = v / g;
            lam[i] = l;
            const float dv = doubleToFloatRz(v - l), dr = doubleToFloatRz(1.0 - g);
            so = fmaf(dv, dv, so);
            ro = fmaf(dr, dr, ro);
        } else {
            const float vf = doubleToFloatRz(v), gf = doubleToFloatRz(g);
            so = fmaf(2.f * vf, vf, so);
            ro = fmaf(2.f * gf, gf, ro);
        }
    }
    blockReduce2f<false>(so, ro, red);   // also orders the lam[] writes before their reads
    const float delta = 2.f * (sqrtf(so) + (float)normA * sqrtf(ro));
    // E in FP32 from an FP64 numerator s_ij + lam_j r_ij (r_ij = -g_ij off the
    // diagonal; one FMA, where the two terms may cancel) and an FP64 gap
    float *E32 = (float *)W;            // E, then X in FP32, in W (A X is no longer needed)
    float *X32 = E32 + maxDim * maxDim;
    float em = 0.f, cm = 0.f;
    for (int k = tid; k < n * n; k += nt) {
        const int i = k / n, j = k - i * n;
        float e;
        if (i == j) {
            e = 0.5f * doubleToFloatRz(1.0 - T[k]);
        } else {
            const double g = symAt(T, n, i, j), v = symAt(V, n, i, j);
            const float gap = doubleToFloatRz(lam[j] - lam[i]);
            if (fabsf(gap) > delta) {
                e = doubleToFloatRz(fma(-lam[j], g, v)) / gap;
                em = fmaxf(em, fabsf(e));
            } else {
                e = -0.5f * doubleToFloatRz(g);
                cm = fmaxf(cm, fabsf(doubleToFloatRz(v)));
            }
        }
        E32[k] = e;
        X32[k] = doubleToFloatRz(X[k]);
    }
    blockReduce2f<true>(em, cm, red);
    emax = em;
    cmax = cm;
    if (!(em <= maxApply)) return;
    float *XE = (float *)T;
    matmulX4<float>(XE, X32, E32, n, false, false);   // X E
    __syncthreads();
    for (int k = tid; k < n * n; k += nt) X[k] += floatToDouble(XE[k]);
    __syncthreads();
}

__device__ void eigBlock(const PmatPart *parts, int d, int pair, int maxDim, int *status, double *eigSmem)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const PmatPart &P = parts[d];
    const int cNum = pair / P.nR, rNum = pair % P.nR;
    const int n = P.dim;
    double *S = eigSmem;
    double *U = S + maxDim * maxDim;
    double *rc = U + maxDim * maxDim;      // 32 cos
    double *rs = rc + 32;                  // 32 sin
    int *rp = (int *)(rs + 32);            // 32 p
    int *rq = rp + 32;                     // 32 q
    double *pi = (double *)(rq + 32);
    double *sq = pi + maxDim;
    double *red = sq + maxDim;             // 2 per warp (8), then the row sums (n <= 56)
    double *rowSum = red + 8;
    double *T = red + 64;                  // [n*n]  (larger dims; the FP32 S and U first)
    double *W = T + maxDim * maxDim;       // [n*n]
    double *V = W + maxDim * maxDim;       // [n*n]
    const double *comp = P.comps + (size_t)cNum * n;
    const double *R = P.R + (size_t)rNum * n * n;

    for (int i = tid; i < n; i += nt) {
        pi[i] = comp[i];
        sq[i] = sqrt(comp[i]);
    }
    __syncthreads();
    // Q off-diagonals R_ij pi_j and diagonal -sum_{j!=i} (Pf/util.c:44-74), row i
    // per thread; the row's share of the normalising sum sum_{j!=i} pi_i Q_ij
    for (int i = tid; i < n; i += nt) {
        double sum = 0.0, rsum = 0.0;
        for (int j = 0; j < n; j++) {
            if (j == i) continue;
            double q = R[i * n + j] * pi[j];
            S[i * n + j] = q;
            sum = sum + q;
            rsum = rsum + pi[i] * q;
        }
        S[i * n + i] = -sum;
        rowSum[i] = rsum;
    }
    __syncthreads();
    // normalise: sum_i sum_{j!=i} pi_i Q_ij = 1 (Pf/util.c:76-115)
    if (tid == 0) {
        double ode = 0.0;
        for (int i = 0; i < n; i++) ode = ode + rowSum[i];
        red[0] = 1.0 / ode;
    }
    __syncthreads();
    const double inv = red[0];
    __syncthreads();
    for (int k = tid; k < n * n; k += nt) S[k] = S[k] * inv;
    __syncthreads();
    // symmetric form; keep the upper triangle's value for both halves
    for (int k = tid; k < n * n; k += nt) {
        int i = k / n, j = k % n;
        if (i < j) {
            double v = S[k] * sq[i] / sq[j];
            S[k] = v;
        }
        U[k] = (i == j) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int k = tid; k < n * n; k += nt) {
        int i = k / n, j = k % n;
        if (i > j) S[k] = S[j * n + i];
    }
    __syncthreads();

    int converged = 0;
    if (n > EIG_SMALL_DIM) {
        // Mixed precision (the FP64 pipe is narrow on this GPU): Jacobi sweeps
        // in FP32 find an approximate eigenbasis X, which two FP64 refinement
        // steps (refineStep) take to FP64 accuracy with matrix products alone.
        // They are accepted when the second step's correction is at most 1e-7
        // (the error left after it is of the order of its square) and every
        // pair of eigenvalues too close to separate is coupled by at most
        // 256 eps ||A||; otherwise (near-degenerate spectra) two Newton-Schulz
        // steps in FP64 (X <- X (3I - X^T X) / 2) make X orthogonal, S <- X^T S X
        // is formed in FP64, and the FP64 Jacobi sweeps below finish from the
        // nearly diagonal S, deciding convergence themselves.
        float *S32 = (float *)T;                     // in T and W until the FP64 steps
        float *U32 = S32 + maxDim * maxDim;
        float *rc32 = (float *)W;                    // the FP32 rotations, in W until it is used
        float *rs32 = rc32 + 32;
        for (int k = tid; k < n * n; k += nt) {
            S32[k] = (float)S[k];
            U32[k] = (k / n == k % n) ? 1.f : 0.f;
        }
        __syncthreads();
        int *sched = (int *)V;                       // the round-robin schedule, in V until it is used
        {
            const int m = (n + 1) & ~1, npairs = m / 2;
            for (int t = tid; t < (m - 1) * npairs; t += nt) {
                int p, q;
                rrPair(t / npairs, t % npairs, m, p, q);
                sched[t] = p | (q << 8);
            }
        }
        __syncthreads();
        double normA = 0.0;
        for (int sweep = 0; sweep < 12; sweep++) {
            double off, dg;
            offDiagMass32(S32, n, red, off, dg);
            if (sweep == 0) normA = sqrt(dg + 2.0 * off);
            if (off <= 1e-13 * dg || off == 0.0) break;
            jacobiSweepPairs(S32, U32, n, rc32, rs32, rp, rq, sched);
        }
        for (int k = tid; k < n * n; k += nt) U[k] = (double)U32[k];
        __syncthreads();
        double *lam = rc;                            // n <= 32 eigenvalue estimates
        double emax = 0.0, cmax = 0.0;
        bool refined = true;
        for (int it = 0; it < 2 && refined; it++) {
            refineStep(S, U, T, W, V, lam, n, maxDim, normA, 1e-3, red, emax, cmax);
            refined = emax <= 1e-3;
        }
        refined = refined && emax <= 1e-7 && cmax <= 256.0 * DBL_EPSILON * normA;
        if (refined) {
            for (int i = tid; i < n; i += nt) S[i * n + i] = lam[i];
            __syncthreads();
            converged = 1;
        }
        for (int it = 0; it < 2 && !refined; it++) {
            matmul64(T, U, U, n, true);              // G = X^T X
            __syncthreads();
            for (int k = tid; k < n * n; k += nt) {   // W = X (3I - G) / 2
                const int i = k / n, j = k % n;
                double acc = 0.0;
                for (int l = 0; l < n; l++) acc += U[i * n + l] * ((l == j ? 3.0 : 0.0) - T[l * n + j]);
                W[k] = 0.5 * acc;
            }
            __syncthreads();
            for (int k = tid; k < n * n; k += nt) U[k] = W[k];
            __syncthreads();
        }
        if (!refined) {
            matmul64(T, S, U, n, false);             // S U
            __syncthreads();
            for (int k = tid; k < n * n; k += nt) {  // U^T (S U), upper triangle
                const int i = k / n, j = k % n;
                if (i > j) continue;
                double acc = 0.0;
                for (int l = 0; l < n; l++) acc += U[l * n + i] * T[l * n + j];
                S[k] = acc;
            }
            __syncthreads();
            for (int k = tid; k < n * n; k += nt) {
                const int i = k / n, j = k % n;
                if (i > j) S[k] = S[j * n + i];
            }
            __syncthreads();
        }
    }
    for (int sweep = 0; sweep < 60 && !converged; sweep++) {
        // convergence: off-diagonal mass vs diagonal mass
        double off, dg;
        offDiagMass<double>(S, n, red, off, dg);
        if (off <= 1e-32 * dg || off == 0.0) {
            converged = 1;
            break;
        }
        // after the first sweeps an element below the rounding of both
        // diagonal entries is set to zero instead of rotated (the classical
        // Jacobi rule): rounding noise cannot keep the sweeps going
        jacobiSweep<double>(S, U, n, rc, rs, rp, rq, sweep > 3);
    }
    if (!converged && tid == 0) atomicOr(status, 2);
    double *out = P.eig + (size_t)pair * eigRecDoubles(n);
    float *outF = (float *)(out + n * n + 2 * n);
    for (int k = tid; k < n * n; k += nt) {
        const double u = U[k];
        const float h = (float)u;
        out[k] = u;
        outF[k] = h;
        outF[n * n + k] = (float)(u - (double)h);
    }
    for (int i = tid; i < n; i += nt) {
        out[n * n + i] = S[i * n + i];
        out[n * n + n + i] = sq[i];
        const double r = 1.0 / sq[i];
        const float sh = (float)sq[i], rh = (float)r;
        outF[2 * n * n + i] = sh;
        outF[2 * n * n + n + i] = (float)(sq[i] - (double)sh);
        outF[2 * n * n + 2 * n + i] = rh;
        outF[2 * n * n + 3 * n + i] = (float)(r - (double)rh);
    }
}

// One launch for both: blocks [0, nE) take an eigensystem each (one block,
// latency bound), blocks [nE, nE+nG) a gamma each (first warp).
// Task lists hold (descriptor, pair or gdasrv) of the inputs that changed.
__global__ void __launch_bounds__(EIG_THREADS_LARGE)
k_gammaEig(const PmatPart *parts, const int2 *eigTasks, int nE, const int2 *gammaTasks, int nG,
           int maxDim, int *status, const int *counts)
{
    extern __shared__ double eigSmem[];
    const int b = blockIdx.x;
    const int capE = nE;
    if (counts) {   // launched over a capacity; the live task counts are in device memory
        nE = counts[0];
        nG = counts[1];
        if (b < capE) {
            if (b >= nE) return;
        } else if (b - capE >= nG) {
            return;
        } else {
            if (threadIdx.x < 32) gammaWarp(parts[gammaTasks[b - capE].x], gammaTasks[b - capE].y, status, eigSmem);
            return;
        }
    }
    if (b < nE) {
        const int2 t = eigTasks[b];
        eigBlock(parts, t.x, t.y, maxDim, status, eigSmem);
    } else if (b - nE < nG && threadIdx.x < 32) {
        const int2 t = gammaTasks[b - nE];
        gammaWarp(parts[t.x], t.y, status, eigSmem);
    }
}

// ----------------------------------------------------------------- P decks
// One lane group per (node, cat): lane k computes e_k = exp(lambda_k t) once.
// For dim^2 <= 32 (DNA) the group has G = next power of two >= dim^2 lanes of
// one warp, lane i*dim + j forms the single entry P_ij and the e values go
// round by shuffle.  Larger dims take a whole block of PDECK_BLOCK threads per
// (node, cat): the eigenvectors and e values in shared memory, each thread
// some entries of the upper triangle of the symmetric form
// Ps_ij = sum_k U_ik e_k U_jk, giving P_ij = Ps_ij sqrt(pi_j/pi_i) and P_ji =
// Ps_ij sqrt(pi_i/pi_j) (half the work, every dot product 20 long instead of
// a row of 400 per lane), in FP32-pair arithmetic.  Each descriptor's task
// range is padded to a multiple of the block so groups never straddle blocks.
constexpr int PDECK_BLOCK = 128;
__host__ __device__ inline int pdeckGroup(int dim)
{
    if (dim * dim > 32) return PDECK_BLOCK;
    int g = 1;
    while (g < dim * dim) g <<= 1;
    return g;
}

// The descriptors, node tables and branch lengths come from the parameter
// image (written only by host copies) or the pinned host image, so they are
// read before the wait on the previous kernel; the Gamma rates and
// eigensystems (k_gammaEig) and the decks (which the previous evaluation's
// pruning reads) only after it.
// counts (nullable): launched over a capacity; the live task and descriptor
// counts are counts[2] and counts[3] (a batch leaves unchanged parts out).
// FP32 pairs: value = h + l with |l| <= ulp(h) / 2 (error-free transformations,
// written with the _rn intrinsics so that no product is contracted into an FMA).
struct Pair2 {
    float h, l;
};

// Knuth's TwoSum: a + b = s + e exactly.
__device__ __forceinline__ Pair2 twoSum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return Pair2{s, e};
}

// Product of two pairs, renormalised (Dekker's FastTwoSum on the FMA-exact
// product and the cross terms); relative error about 2^-46.
__device__ __forceinline__ Pair2 pairMul(Pair2 a, Pair2 b)
{
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    const float s = __fadd_rn(p, e);
    return Pair2{s, __fsub_rn(e, __fsub_rn(s, p))};
}

// Sum of two pairs (TwoSum of the high parts, the low parts added to its
// error, renormalised).
__device__ __forceinline__ Pair2 pairAdd(Pair2 a, Pair2 b)
{
    const Pair2 s = twoSum(a.h, b.h);
    const float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
    const float h = __fadd_rn(s.h, e);
    return Pair2{h, __fsub_rn(e, __fsub_rn(h, s.h))};
}

// 1/j! as FP32 pairs, j = 0..13.
#define P4G_INV_FACT(j, f) (float)(1.0 / (f)), (float)(1.0 / (f) - (double)(float)(1.0 / (f)))
__constant__ float kInvFact[14][2] = {
    {P4G_INV_FACT(0, 1.0)}, {P4G_INV_FACT(1, 1.0)}, {P4G_INV_FACT(2, 2.0)}, {P4G_INV_FACT(3, 6.0)},
    {P4G_INV_FACT(4, 24.0)}, {P4G_INV_FACT(5, 120.0)}, {P4G_INV_FACT(6, 720.0)}, {P4G_INV_FACT(7, 5040.0)},
    {P4G_INV_FACT(8, 40320.0)}, {P4G_INV_FACT(9, 362880.0)}, {P4G_INV_FACT(10, 3628800.0)},
    {P4G_INV_FACT(11, 39916800.0)}, {P4G_INV_FACT(12, 479001600.0)}, {P4G_INV_FACT(13, 6227020800.0)}};
#undef P4G_INV_FACT

// e^x as an FP32 pair for an FP64 argument: x = k ln2 + r with one FP64 FMA
// (|r| <= ln2 / 2), e^r by its Taylor series to r^13 / 13! (truncation below
// 2e-16) in pair arithmetic (Horner), scaled by 2^k.  Relative error about
// 5e-15.  Arguments below -87 (results below FP32's normal range) give 0.
__device__ __forceinline__ Pair2 pairExp(double x)
{
    if (x != x) return Pair2{__int_as_float(0x7fc00000), 0.f};
    if (x < -87.0) return Pair2{0.f, 0.f};
    if (x > 88.0) return Pair2{__int_as_float(0x7f800000), 0.f};
    const float kf = rintf(__fmul_rn((float)x, 1.44269504088896341f));
    const double r = fma(-(double)kf, 0.69314718055994531, x);
    const float rh = (float)r;
    const Pair2 rp{rh, (float)(r - (double)rh)};
    Pair2 y{kInvFact[13][0], kInvFact[13][1]};
#pragma unroll
    for (int j = 12; j >= 0; j--) y = pairAdd(pairMul(y, rp), Pair2{kInvFact[j][0], kInvFact[j][1]});
    const float sc = __int_as_float((127 + (int)kf) << 23);   // 2^k exactly, k in [-126, 127]
    return Pair2{__fmul_rn(y.h, sc), __fmul_rn(y.l, sc)};
}

// Dot2 (see k_pdeck) of row i of the pair matrix A and row j of U; N: the
// state count at compile time (0: n at run time).
template <int N>
__device__ __forceinline__ Pair2 dot2Row(const float *ah, const float *al, const float *uh, const float *ul, int n)
{
    float ps = 0.f, es = 0.f;   // running sum and its error sum
#pragma unroll
    for (int k = 0; k < (N ? N : MAX_DIM); k++) {
        if (!N && k >= n) break;
        const float a = ah[k], b = uh[k];
        const float h = __fmul_rn(a, b);
        float r = __fmaf_rn(a, b, -h);   // exact: a b = h + r
        r = __fmaf_rn(a, ul[k], r);
        r = __fmaf_rn(al[k], b, r);
        const Pair2 sm = twoSum(ps, h);
        ps = sm.h;
        es = __fadd_rn(es, __fadd_rn(sm.l, r));
    }
    return twoSum(ps, es);
}

__global__ void k_pdeck(const PmatPart *parts, const int *prefix, int nDesc, int nTasks, const int *counts)
{
    if (counts) {
        nTasks = counts[2];
        nDesc = counts[3];
        if (nTasks <= 0 || nDesc <= 0) return;
    }
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool inRange = idx < nTasks;
    const int d = findDesc(prefix, nDesc, inRange ? idx : nTasks - 1);
    const PmatPart P = parts[d];   // a copy: the wait below does not make it be read again
    const int n = P.dim;
    const int G = pdeckGroup(n);
    const int local = idx - prefix[d];
    const int unit = local / G, g = local % G;
    const bool active = inRange && unit < P.nNodes * P.nCat;
    const int node = active ? unit / P.nCat : 0;
    const int cat = active ? unit % P.nCat : 0;
    double t = 0.0, bl = 0.0;
    const double *E = P.eig;
    int cNum = 0, rNum = 0, gNum = 0;
    bool leafNode = false;
    if (active) {
        const int *ni = P.nodeIdx + ((size_t)node * P.nParts + P.partIdx) * 3;
        cNum = ni[0];
        rNum = ni[1];
        gNum = ni[2];
        bl = P.brLen[node];
        leafNode = P.isLeaf[node] != 0;
    }
    pdlEnter();
    if (active) {
        // t as p4_calculateBigPDecksPart forms it (Pf/p4_node.c:318-343)
        if (P.nG) t = bl * P.rates[gNum * P.nCat + cat] * P.relRate;
        else t = bl * P.relRate;
        if (P.pInvar != 0.0) t = t / (1.0 - P.pInvar);
        E = P.eig + (size_t)(cNum * P.nR + rNum) * eigRecDoubles(n);
    }
    const double *lam = E + n * n, *sq = lam + n;
    if (n * n <= 32) {   // one entry per lane, in FP32 pairs as the block form below
        const int base = lane - (lane % G);
        const bool elem = active && g < n * n && node != P.root;
        const int i = elem ? g / n : 0, j = elem ? g % n : 0;
        const float *F = (const float *)(E + n * n + 2 * n);   // the record's FP32 pairs
        float ps = 0.f, es = 0.f;   // Dot2 of row i of A = U diag(e) and row j of U
        auto term = [&](float uh, float ul, float eh, float el, float b, float bl) {
            const Pair2 a = pairMul(Pair2{uh, ul}, Pair2{eh, el});
            const float h = __fmul_rn(a.h, b);
            float r = __fmaf_rn(a.h, b, -h);
            r = __fmaf_rn(a.h, bl, r);
            r = __fmaf_rn(a.l, b, r);
            const Pair2 sm = twoSum(ps, h);
            ps = sm.h;
            es = __fadd_rn(es, __fadd_rn(sm.l, r));
        };
        if (n == 4) {
            // DNA: rows i and j of U loaded before e is formed (the indices are in
            // the record for every lane: i = j = 0 where there is no entry)
            float uih[4], uil[4], ujh[4], ujl[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                uih[k] = F[i * 4 + k];
                uil[k] = F[16 + i * 4 + k];
                ujh[k] = F[j * 4 + k];
                ujl[k] = F[16 + j * 4 + k];
            }
            Pair2 ek{0.f, 0.f};
            if (active && g < n) ek = pairExp(lam[g] * t);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float eh = __shfl_sync(0xffffffffu, ek.h, base + k);
                const float el = __shfl_sync(0xffffffffu, ek.l, base + k);
                if (elem) term(uih[k], uil[k], eh, el, ujh[k], ujl[k]);
            }
        } else {
            Pair2 ek{0.f, 0.f};
            if (active && g < n) ek = pairExp(lam[g] * t);
            for (int k = 0; k < n; k++) {
                const float eh = __shfl_sync(0xffffffffu, ek.h, base + k);
                const float el = __shfl_sync(0xffffffffu, ek.l, base + k);
                if (elem) term(F[i * n + k], F[n * n + i * n + k], eh, el, F[j * n + k], F[n * n + j * n + k]);
            }
        }
        Pair2 v{0.f, 0.f};
        if (elem) {
            const float *sqp = F + 2 * n * n;   // sqh, sql, rqh, rql
            v = pairMul(twoSum(ps, es), pairMul(Pair2{sqp[j], sqp[n + j]}, Pair2{sqp[2 * n + i], sqp[3 * n + i]}));
        }
        const bool leaf = elem && leafNode;
        if (elem) {
            const float f = __fadd_rn(v.h, v.l);
            float *d32 = P.decks32 + ((size_t)node * P.nCat + cat) * n * n;
            if (leaf) d32[j * n + i] = f;   // leaves: column j contiguous
            else d32[i * n + j] = f;
            if (P.decks64)
                P.decks64[((size_t)node * P.nCat + cat) * n * n + i * n + j] = floatToDouble(v.h) + floatToDouble(v.l);
        }
        // partial-equate sums of a leaf's rows (j order, pair sums), gathered by
        // lane (i, 0); nPartial is the same for the whole warp (one descriptor per
        // warp), and a warp that holds no leaf deck skips them (the condition is
        // warp-uniform, so the shuffles keep every lane)
        const int nPartialW = __any_sync(0xffffffffu, leaf) ? P.nPartial : 0;
        for (int q = 0; q < nPartialW; q++) {
            const uint32_t msk = P.partialMask[q];
            Pair2 sacc{0.f, 0.f};
            for (int jj = 0; jj < n; jj++) {
                const float vh = __shfl_sync(0xffffffffu, v.h, base + i * n + jj);
                const float vl = __shfl_sync(0xffffffffu, v.l, base + i * n + jj);
                if ((msk >> jj) & 1u) sacc = pairAdd(sacc, Pair2{vh, vl});
            }
            if (leaf && j == 0)
                P.eqTab[(((size_t)node * P.nPartial + q) * P.nCat + cat) * n + i] = __fadd_rn(sacc.h, sacc.l);
        }
        return;
    }
    // a whole block for this (node, cat): the block is uniform in `active`.
    // The sums run in FP32 pairs (value = hi + lo) on the FP32 pipes, which are
    // many times wider than this GPU's FP64 pipe: with A = U diag(e^{lambda t}),
    //   M_ij = sum_k A_ik U_jk    (symmetric: the upper triangle only)
    // by the compensated dot product Dot2 of Ogita, Rump and Oishi (SIAM J. Sci.
    // Comput. 26, 2005; products split exactly with an FMA, partial sums with
    // Knuth's TwoSum), the pairs' cross terms added to the error sum, then
    // P_ij = M_ij sqrt(pi_j) / sqrt(pi_i) and P_ji = M_ij sqrt(pi_i) / sqrt(pi_j)
    // as pair products.  The result carries about 2 x 24 bits (~1e-14 of the
    // terms' magnitude); the FP64 deck is hi + lo rounded once, the FP32 deck
    // hi + lo rounded to FP32.  e^{lambda t} is a pair too (pairExp); FP64 is
    // left with its argument and range reduction and that final add.
    __shared__ __align__(16) float sUh[MAX_DIM * MAX_DIM], sUl[MAX_DIM * MAX_DIM];
    __shared__ __align__(16) float sAh[MAX_DIM * MAX_DIM], sAl[MAX_DIM * MAX_DIM];
    __shared__ float sPh[MAX_DIM * MAX_DIM], sPl[MAX_DIM * MAX_DIM];   // the deck as pairs
    __shared__ float sEh[MAX_DIM], sEl[MAX_DIM], sSq[4 * MAX_DIM];   // e pairs; sqh, sql, rqh, rql
    const int tid = threadIdx.x;
    if (active) {
        const float *F = (const float *)(E + n * n + 2 * n);   // the record's FP32 pairs
        for (int k = tid; k < n * n; k += PDECK_BLOCK) {
            sUh[k] = F[k];
            sUl[k] = F[n * n + k];
        }
        for (int k = tid; k < 4 * n; k += PDECK_BLOCK) sSq[k] = F[2 * n * n + k];
        if (tid < n) {
            const Pair2 e = pairExp(lam[tid] * t);
            sEh[tid] = e.h;
            sEl[tid] = e.l;
        }
        __syncthreads();
        for (int k = tid; k < n * n; k += PDECK_BLOCK) {   // A_ik = U_ik e_k
            const int c = k % n;
            const Pair2 a = pairMul(Pair2{sUh[k], sUl[k]}, Pair2{sEh[c], sEl[c]});
            sAh[k] = a.h;
            sAl[k] = a.l;
        }
    }
    __syncthreads();
    if (!active || node == P.root) return;
    const bool leaf = leafNode;
    float *d32 = P.decks32 + ((size_t)node * P.nCat + cat) * n * n;
    double *d64 = P.decks64 ? P.decks64 + ((size_t)node * P.nCat + cat) * n * n : nullptr;
    // tensor-core image of an internal node's P (row i = N index, column j =
    // K index) as K-major core matrices: hi at +0, lo at +768 floats
    float *tb = (P.tcB && !leaf) ? P.tcB + ((size_t)node * P.nCat + cat) * 1536 : nullptr;
    auto put = [&](int i, int j, Pair2 v) {
        const float f = __fadd_rn(v.h, v.l);
        if (leaf) d32[j * n + i] = f;   // leaves: column j contiguous
        else d32[i * n + j] = f;
        if (d64) d64[i * n + j] = floatToDouble(v.h) + floatToDouble(v.l);
        if (tb) {
            const float hi = tc::toTf32(f);
            const int off = (i >> 3) * 192 + (j >> 2) * 32 + (i & 7) * 4 + (j & 3);
            tb[off] = hi;
            tb[768 + off] = tc::toTf32(f - hi);
        }
        sPh[i * n + j] = v.h;
        sPl[i * n + j] = v.l;
    };
    const float *sqh = sSq, *sql = sSq + n, *rqh = sSq + 2 * n, *rql = sSq + 3 * n;
    for (int u = tid; u < n * n; u += PDECK_BLOCK) {
        const int i = u / n, j = u - (u / n) * n;
        if (j < i) continue;
        const Pair2 m = n == 20 ? dot2Row<20>(sAh + i * n, sAl + i * n, sUh + j * n, sUl + j * n, n)
                                : dot2Row<0>(sAh + i * n, sAl + i * n, sUh + j * n, sUl + j * n, n);
        put(i, j, pairMul(m, pairMul(Pair2{sqh[j], sql[j]}, Pair2{rqh[i], rql[i]})));
        if (j != i) put(j, i, pairMul(m, pairMul(Pair2{sqh[i], sql[i]}, Pair2{rqh[j], rql[j]})));
    }
    if (leaf && P.nPartial) {
        __syncthreads();   // leafNode is uniform over the block
        for (int w = tid; w < P.nPartial * n; w += PDECK_BLOCK) {
            const int q = w / n, i = w - q * n;
            const uint32_t msk = P.partialMask[q];
            Pair2 sacc{0.f, 0.f};
            for (int j = 0; j < n; j++)
                if ((msk >> j) & 1u) sacc = pairAdd(sacc, Pair2{sPh[i * n + j], sPl[i * n + j]});
            P.eqTab[(((size_t)node * P.nPartial + q) * P.nCat + cat) * n + i] = __fadd_rn(sacc.h, sacc.l);
        }
    }
}

// The same two launches with the eigen/gamma task counts read from device
// memory (launched over capacities capE, capG), so that the launch shape does
// not depend on which inputs changed: what a captured CUDA graph needs.
int launchPmatDev(const PmatPart *dParts, const int2 *dEigTasks, int capE, const int2 *dGammaTasks, int capG,
                  const int *dCounts, const int *dPrefixD, int nDesc, int nD, int maxDim, int *dStatus,
                  cudaStream_t s)
{
    if (capG + capE > 0) {
        size_t per = eigSmemDoubles(maxDim);
        size_t smem = std::max<size_t>(per, MAX_CAT) * sizeof(double);
        if (smem > 48 * 1024)
            P4G_CUDA(cudaFuncSetAttribute(k_gammaEig, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_gammaEig<<<capG + capE, eigThreads(maxDim), smem, s>>>(dParts, dEigTasks, capE, dGammaTasks, capG, maxDim, dStatus,
                                                  dCounts);
        P4G_CUDA(cudaGetLastError());
    }
    if (nD > 0) {
        P4G_CUDA(launchPdl(k_pdeck, dim3((nD + PDECK_BLOCK - 1) / PDECK_BLOCK), dim3(PDECK_BLOCK), 0, s, dParts,
                           dPrefixD, nDesc, nD, dCounts));
    }
    return P4G_OK;
}

int pdeckTasks(int dim, int nNodes, int nCat)
{
    int t = nNodes * nCat * pdeckGroup(dim);
    return (t + PDECK_BLOCK - 1) / PDECK_BLOCK * PDECK_BLOCK;
}

int launchPmat(const PmatPart *dParts, const int2 *dEigTasks, int nE, const int2 *dGammaTasks, int nG,
               const int *dPrefixD, int nDesc, int nD, int maxDim, int *dStatus, cudaStream_t s)
{
    if (nG + nE > 0) {
        size_t per = eigSmemDoubles(maxDim);
        size_t smem = std::max<size_t>(per, MAX_CAT) * sizeof(double);
        if (smem > 48 * 1024)
            P4G_CUDA(cudaFuncSetAttribute(k_gammaEig, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_gammaEig<<<nG + nE, eigThreads(maxDim), smem, s>>>(dParts, dEigTasks, nE, dGammaTasks, nG, maxDim, dStatus, nullptr);
        P4G_CUDA(cudaGetLastError());
    }
    if (nD > 0) {
        // one block per protein deck (several DNA decks per block): the decks spread over the SMs
        P4G_CUDA(launchPdl(k_pdeck, dim3((nD + PDECK_BLOCK - 1) / PDECK_BLOCK), dim3(PDECK_BLOCK), 0, s, dParts,
                           dPrefixD, nDesc, nD, (const int *)nullptr));
    }
    return P4G_OK;
}

}  // namespace p4g
