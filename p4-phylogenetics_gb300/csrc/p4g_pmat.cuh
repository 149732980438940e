// Descriptor of one (tree, part) unit of setPrams work, laid out in the
// tree's parameter image so that one host->device copy carries both the
// descriptors and the parameter values they point at.
#pragma once
#include <stdint.h>

namespace p4g {

// One eigensystem record per (comp, rMatrix): U [n*n], lambda [n], sqrt(pi) [n]
// as doubles, then the same values as FP32 pairs (hi + lo, |lo| <= ulp(hi)/2)
// for the pair-arithmetic P decks: Uh [n*n], Ul [n*n], sqh [n], sql [n] and the
// pairs of 1/sqrt(pi), rqh [n], rql [n] (2n^2 + 4n floats = n^2 + 2n doubles).
__host__ __device__ inline size_t eigRecDoubles(int n) { return 2 * ((size_t)n * n + 2 * n); }

struct PmatPart {
    const double *comps;     // [nComps][dim]
    const double *R;         // [nR][dim][dim] symmetric
    const double *gval;      // [nG] gamma shapes
    const double *brLen;     // [nNodes]
    const int *nodeIdx;      // [nNodes][nParts][3] comp, rMatrix, gdasrv numbers
    const int *isLeaf;       // [nNodes]
    double *rates;           // [nG][nCat]            (out)
    double *eig;             // [nComps*nR][eigRecDoubles(dim)] (out)
    float *decks32;          // [nNodes][nCat][dim][dim] (out)
    float *eqTab;            // [nNodes][nPartial][nCat][dim] (out)
    double *decks64;         // [nNodes][nCat][dim][dim] (out, nullable)
    float *tcB;              // [nNodes][nCat][2][768] split-TF32 images of the internal
                             // nodes' P for the tensor-core kernel (out, nullable)
    const uint32_t *partialMask;  // [nPartial]
    double pInvar, relRate;
    int dim, nCat, nComps, nR, nG, nNodes, root, nPartial, partIdx, nParts;
    int pad_[2];
};

int pdeckTasks(int dim, int nNodes, int nCat);
int launchPmatDev(const PmatPart *dParts, const int2 *dEigTasks, int capE, const int2 *dGammaTasks, int capG,
                  const int *dCounts, const int *dPrefixD, int nDesc, int nD, int maxDim, int *dStatus,
                  cudaStream_t s);
int launchPmat(const PmatPart *dParts, const int2 *dEigTasks, int nE, const int2 *dGammaTasks, int nG,
               const int *dPrefixD, int nDesc, int nD, int maxDim, int *dStatus, cudaStream_t s);

}  // namespace p4g
