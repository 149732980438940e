// Job descriptor of the plain FP64 path (one tree-part per launch sequence).
#pragma once
#include <stdint.h>

namespace p4g {

struct Node64Job {
    const double *decks64;    // [nNodes][nCat][dim][dim], row = parent state
    const int *patterns;      // raw p4 codes [nTax][nPat]
    const int *equates;       // [nEquates][dim]
    const int *table;         // per internal node: self, nKids, (child, kind, ref) x nKids
    const int *nodeStart;     // [nInternal] offsets into table (post-order)
    double *cl;               // [nInternal][nCat][dim][nPatPad]
    const double *rootComp;   // [dim]
    const double *counts;     // [nPat]
    const uint32_t *invMask;  // [nPat]
    double *partials;         // [root blocks]
    double *out;
    int *ticket;
    int *badFlag;
    double pInvar, varScale;
    int nPat, nPatPad, nCat, dim, nInternal, rootInternal, rootLeafRow, pad_;
};

int launchPrune64(const Node64Job *dJob, const Node64Job &h, cudaStream_t s);
// One internal node's CL (internal index nodeIdx of the job's table).
int launchNode64(const Node64Job *dJob, const Node64Job &h, int nodeIdx, cudaStream_t s);

}  // namespace p4g
