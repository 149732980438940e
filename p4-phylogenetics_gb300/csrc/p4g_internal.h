// Internal structures of libp4gpu: host objects mirroring p4's C structs
// (Pf/pftypes.h:24-240) and the device-side job descriptors of the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <functional>
#include <map>
#include <string>
#include <vector>
#include "p4gpu.h"
#include "p4g_prune64.cuh"

namespace p4g {

// p4 character codes (Pf/defines.h).
constexpr int GAP_CODE = -1;
constexpr int QMARK_CODE = -2;
constexpr int N_LIKE = -3;
constexpr int EQUATES_BASE = -64;

// Rescale a pattern's CL block when its largest entry drops below 2^-32.
constexpr int SCALE_LOG2 = 32;

constexpr int MAX_DIM = 32;     // state masks are 32-bit
constexpr int MAX_CAT = 16;

// ------------------------------------------------------------ status
int setError(int code, const char *fmt, ...);
#define P4G_CUDA(call)                                                          \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess)                                                  \
            return ::p4g::setError(P4G_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, \
                                   #call, cudaGetErrorString(e_));              \
    } while (0)

// ------------------------------------------------------------ device buffer
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t n);   // grow-only
    void release();
    ~DevBuf() { release(); }
    template <class T> T *as() const { return (T *)ptr; }
};

struct PinnedBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t n);
    void release();
    ~PinnedBuf() { release(); }
    template <class T> T *as() const { return (T *)ptr; }
};

// ------------------------------------------------------------ data
struct Part {
    int dim = 0, nTax = 0, nChar = 0, nEquates = 0;
    std::string symbols, equateSymbols;
    std::vector<int> equates;          // nEquates*dim, 0/1
    std::vector<int> sequences;        // nTax*nChar codes
    std::vector<int> patterns;         // nTax*nPatterns
    std::vector<int> counts;           // nPatterns
    std::vector<int> seqPosIdx;        // nChar
    std::vector<int> invVec;           // nPatterns
    std::vector<int> invArr;           // dim*nPatterns
    std::vector<double> siteLikes;     // nChar (after getSiteLikes evaluation)
    int nPatterns = 0;
    bool patternsMade = false, invarMade = false;
    // compact device coding
    int nPartial = 0;                  // equates that are not all-ones
    std::vector<int> partialOfEquate;  // equate index -> partial index or -1 (all-ones)
    std::vector<uint32_t> partialMask; // nPartial state masks
    // device copies
    DevBuf dCodes;     // uint8 [nTax][nPatPad]
    DevBuf dCounts;    // double [nPatterns]
    DevBuf dInvMask;   // uint32 [nPatterns]
    DevBuf dPat32;     // int32 raw patterns [nTax][nPatterns] (plain FP64 path)
    DevBuf dEqInt;     // int32 equates table [nEquates*dim] (plain FP64 path)
    DevBuf dEquates;   // uint32 state masks of the partial equates [nPartial]
    bool dev64Valid = false;
    int upload64(cudaStream_t s);
    int nPatPad = 0;
    bool devValid = false;
    unsigned long long gen = 0;   // bumped at every upload of new device data
    int upload(cudaStream_t s);
};

struct Data {
    int nTax = 0, nParts = 0;
    std::vector<Part *> parts;
};

// ------------------------------------------------------------ model
struct Comp {
    int free = 0;
    double *val = nullptr;   // caller-owned, aliased (Pf/p4_model.c:337)
};
struct RMatrix {
    int free = 0, spec = 0;
    std::vector<double> bigR; // dim*dim
    double kappa = 2.0;
};
struct Gdasrv {
    int free = 0, nCat = 0;
    double *val = nullptr, *freqs = nullptr, *rates = nullptr;  // aliased
};
struct ModelPart {
    int dim = 0, nComps = 0, nRMatrices = 0, nGdasrvs = 0, nCat = 1, pInvarFree = 0;
    double pInvar = 0.0, relRate = 1.0;
    std::vector<Comp> comps;
    std::vector<RMatrix> rMatrices;
    std::vector<Gdasrv *> gdasrvs;
    int *bQETneedsReset = nullptr;  // aliased, nComps*nRMatrices
};
struct Model {
    int nParts = 0, doRelRates = 0, relRatesAreFree = 0, nFreePrams = 0, isHet = 0;
    int *rMatrixNormalizeTo1 = nullptr;
    double *bounds[14] = {};   // PINVAR_MIN .. BRLEN_MAX pointers (caller-owned)
    std::vector<ModelPart> parts;
    double PIVEC_MIN() const { return bounds[6] ? *bounds[6] : 1e-13; }
};

// ------------------------------------------------------------ tree
struct Tree;
struct Node {
    int nodeNum = -1;
    Tree *tree = nullptr;
    int parent = -1, leftChild = -1, sibling = -1;
    int seqNum = -1, isLeaf = 0, inTree = 1;
    double brLen = -1.0;
    std::vector<int> compNums, rMatrixNums, gdasrvNums;
};

// Program opcodes of the fused pruning kernels (one instruction per int32:
// op in bits 0-3, operand a in bits 4-17, operand b in bits 18-31).
// OP_SCALE_XFORM = OP_SCALE then OP_XFORM of the same node (a = node).
// OP_CLADE (a = clade index; the k-th OP_CLADE of a program reads clade k):
// the transformed product of a whole small subtree, read from the
// per-evaluation table of its distinct leaf-code combinations (the subtree's
// own ops, run once per combination), with the combination's scale exponent
// added.
// OP_CHERRY (a = cherry index, b = first leaf's row) is followed by an
// OP_ARG word (b = second leaf's row) and then the cherry's own TIPSET,
// TIPMUL, SCALE_XFORM: a job with a cherry table reads the transformed
// product of the node's two leaves from it (a per-evaluation table of every
// (code, code) pair) and skips those three ops; a job without one skips the
// lookup.
enum Op : int { OP_TIPSET = 0, OP_TIPMUL = 1, OP_XFORM = 2, OP_PUSH = 3, OP_MULSLOT = 4,
                OP_SCALE = 5, OP_ROOT = 6, OP_CHERRY = 7, OP_ARG = 8, OP_SCALE_XFORM = 9, OP_CLADE = 10 };
inline int mkIns(int op, int a, int b) { return op | (a << 4) | (b << 18); }

// One (tree, part) unit of pruning work, read by every block of that unit.
struct PruneJob {
    const float *decks;       // [nNodes][nCat][dim][dim]; leaf decks transposed
    const float *eqTab;       // [nNodes][nPartial][nCat][dim]
    const uint8_t *codes;     // [nTax][nPatPad]
    const double *counts;     // [nPat]
    const uint32_t *invMask;  // [nPat]
    const uint32_t *partialMask; // [nPartial]
    const int *prog;          // program
    const double *rootComp;   // [dim] FP64
    double *partials;         // per-block partial sums
    double *out;              // part lnL
    int *ticket;              // last-block counter (self-resetting)
    int *badFlag;             // any non-positive like (self-resetting)
    const float *tcB;         // split-TF32 P images for k_prune_tc (nullable)
    float *cherryTab;         // [nCherry][K][K][nCat][dim] (K = dim + 1 + nPartial codes)
    const int4 *cherries;     // [nCherry] (node, first leaf, second leaf, -)
    float *catLikes;          // optional [nPat][nCat] per-category root sums, scaled like likeScaled
    float *rootCL;            // optional [nPat][nCat][dim] root partials (a leaf root's own code
                              //   applied), scaled like likeScaled
    const uint32_t *cladeIdx; // [nClade][nPatPad] table entry of each pattern's leaf-code combination
    const float *cladeTab;    // [entries][nCat][dim] transformed products
    const int *cladeExp;      // [entries] their scale exponents
    float *cladeOut;          // clade-table job: write the program's result here
    int *cladeOutExp;         //   ([nPat][nCat][dim], [nPat]) instead of the root reduction
    float *likeScaled;        // optional per-pattern outputs (nullable)
    int *exps;
    double *lnl;
    double pInvar;            // 0 => no invariant term
    double varScale;          // (1-pInvar)/nCat
    double logScale;          // log of the factor applied to the variable-site like
    int nPat, nPatPad, nPartial, nProg, nNodes, nTax, nBlocks, nSlots;
    int rootLeafRow;          // seqNum of a leaf root, -1 otherwise
    int dim, nCat;
    int nCherry;              // cherries in the program (0: none)
    int nClade;               // clade-table rows staged per tile (0: none), in the program's read order
    // Staging maps of a whole-tree program that reads clade tables (nullable:
    // every deck and code row staged): deckMap = [nNodes] shared-memory deck of
    // each node, then [nDeck] node of each deck; rowMap = [nTax] staged code
    // row of each taxon, then [nRow] taxon of each row.  Decks are remapped in
    // the shared-memory deck shapes only.
    const int *deckMap;
    const int *rowMap;
    int nDeck, nRow;
    int nCladeEntries;        // entries of cladeTab / cladeExp: an index at or past it is refused
                              //   (badFlag bit 4, lnL NaN) instead of read
};
struct BlockDesc {
    int job;
    int p0;
    int blk;   // index of this block within its job
    int pad_;
};

// Per-tree device state.  One pinned parameter image per tree carries the
// setPrams descriptors, the pruning jobs, the program and every parameter
// value; a single host->device copy refreshes all of it.
struct PruneGroup {
    int dim, nCat, blk0, nBlk, smem, shape;
};
// Captured launch sequences, each with the signature it was captured for.
// A few are kept (least recently used goes first), so that calls which
// alternate between shapes (e.g. setPrams with and without eigensystems to
// recompute, as MCMC proposals do) replay instead of capturing again.
struct GraphSlot {
    static constexpr int WAYS = 4;
    struct Entry {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        std::vector<long long> sig;
        unsigned long long used = 0;
    };
    Entry e[WAYS];
    unsigned long long clock = 0;
    int run(const std::vector<long long> &sig, cudaStream_t s, const std::function<int()> &enqueue);
    void release();
};

struct TreeDev {
    bool allocated = false;
    PinnedBuf hImg;
    DevBuf dImg;
    size_t imgBytes = 0;
    size_t oPmat = 0, oJobs = 0, oPrefix = 0, oBrLen = 0, oNodeIdx = 0, oIsLeaf = 0;
    size_t oProg = 0, oBlocks = 0, oMaps = 0;
    int progCap = 0;
    int nDeck = 0, nRow = 0;   // decks and code rows a whole-tree tile stages
    std::vector<size_t> oComps, oR, oG;
    DevBuf dRates, dEig, dDecks32, dEqTab, dDecks64, dPartials, dOut, dTicket, dBad, dTcB;
    std::vector<size_t> oRates, oEig, oDecks, oEqTab, oPartials, oTcB;  // element offsets
    DevBuf dLike, dExp, dLnl, dCatLike, dRootCL;
    std::vector<size_t> oPat, oCatLike, oRootCL;
    bool rootCLOn = false, jobsRootCL = false;   // root partials wanted / in the jobs
    PinnedBuf hOut;   // nParts doubles, then the status int
    cudaEvent_t imgFree = nullptr;   // last H2D of the image done
    // The branch lengths are read by the P-deck kernel straight from the
    // pinned host image (hImgDev: its device-side address), so that an
    // evaluation whose other inputs are unchanged needs no image copy;
    // shadow = the host image as last copied to the device (empty: unknown).
    const void *hImgDev = nullptr;
    std::vector<char> shadow;
    // the stream's last kernel may be this tree's clade numbering (which
    // writes the clade jobs, tiles and codes): the next clade launch must not
    // read them before its wait; cleared once another operation follows
    bool cladeFresh = false;
    unsigned long long devGen = 0;   // unique per allocation of the tree's device state
    std::vector<int> prog;
    int nProg = 0, nSlots = 0;
    std::vector<int4> cherryList;     // (node, leaf, leaf, -) of the current program
    // clade tables (p4g_clades.cu); trees evaluated in a batch use none
    int cladeSize = 6;                // largest clade in leaves (< 2: off)
    bool cladeOff = false;            // switched off by the first evaluation's timing
    bool cladeChecked = false;        // that timing was done, or the caller set the size
    bool inBatch = false;
    int nClade = 0;
    std::vector<int> cladeOf;         // per node: clade index or -1
    DevBuf dCladeKeys, dCladeVals, dCladeIdx, dCladeTab, dCladeExp, dCladeCodes, dCladeMisc, dCladeMeta, dCladeBlocks;
    PinnedBuf hClade;                 // staging of the clade jobs, tasks and programs
    cudaEvent_t cladeUp = nullptr;    // their last upload
    std::vector<PruneGroup> cladeGroups;
    std::vector<const int *> cladeTileCount;   // per clade group: its device tile count
    std::map<int, int> cladeShape;    // (dim * 64 + nCat) -> tile shape of the clade-table launches
    long long cladeVersion = 0;       // counts clade builds (a captured batch graph follows it)
    DevBuf dCherryTab;
    std::vector<size_t> oCherryTab;   // per part, floats
    size_t oCherries = 0;             // image offset of the cherry list
    int capCherry = 0;
    long long cherryWork = 0;         // cherry-table blocks: nCherry x the largest nCat of the parts with tables
    std::vector<BlockDesc> blocks;
    std::vector<PruneGroup> groups;
    // setPrams input cache: eigensystems / gamma rates are recomputed only
    // for the (comp, R) pairs and gdasrvs whose values changed
    std::vector<std::vector<double>> cComps, cR, cG;
    bool cacheValid = false;
    int lastLaunches = 0;   // setPrams kernels enqueued by the last setPrams
    size_t oEigTasks = 0, oGammaTasks = 0;
    bool progDirty = true;
    bool tuned = false;
    int blockCap = 0;
    bool haveParams = false;
    bool siteOutputs = false;
    bool jobsSiteOutputs = false;
    // CUDA graphs of the setPrams and pruning launch sequences (p4g_setGraphs)
    bool useGraphs = true;
    GraphSlot setPramsGraph, pruneGraph;
    // plain FP64 path (precision mode 1)
    int precision = 0;
    bool table64Dirty = true;
    std::vector<int> table64, nodeStart64;
    DevBuf dTable64, dCl64, dJobs64, dPartials64;
    std::vector<Node64Job> jobs64;    // host copy of the last FP64 evaluation's jobs
    DevBuf dCl2, dNewtP, dNewtSums;   // Newton branch-length optimisation (p4g_newt.cu)
    std::vector<size_t> oCl64, oPartials64;
    int nInternal64 = 0;
};

struct Tree {
    int nNodes = 0, nLeaves = 0, nParts = 0;
    int *preOrder = nullptr, *postOrder = nullptr;  // aliased
    double *partLikes = nullptr;                    // aliased
    int *passLimit = nullptr;                       // aliased: ML optimisation pass limit
    Data *data = nullptr;
    Model *model = nullptr;
    std::vector<Node *> nodes;
    int root = -1;
    bool topoDirty = true;
    double logLike = 0.0;
    TreeDev dev;
};

// ------------------------------------------------------------ launches
struct Ctx {
    int device = -1;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    int nSM = 0;
};
Ctx &ctx();
int ensureCtx();

// Programmatic dependent launch (on by default, p4g_setProgrammaticLaunch):
// the kernels launched through launchPdl start with griddepcontrol.wait, so
// they read nothing before the previous kernel in the stream has completed,
// and may themselves be launched while that kernel drains.
extern bool g_pdl;
template <typename... KArgs, typename... Args>
inline cudaError_t launchPdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                             Args... args)
{
    if (!g_pdl) {
        k<<<grid, block, smem, s>>>(args...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// p4g_prune.cu
// Bits of a pruning launch's `early` argument: what the kernel may read
// before its wait on the stream's previous kernel, because that kernel does
// not write it (host code knows the launch order; 0 = wait first, the safe
// default).  Anything written before that kernel is complete by then: a
// kernel launched this way starts only once every block of the previous one
// has passed its own wait.
//   PDL_EARLY_JOBS  : jobs, block list, tile count, program, tip codes,
//                     clade-table index rows, pattern weights and masks
//   PDL_EARLY_DECKS : the P decks and partial-equate tables as well
constexpr int PDL_EARLY_JOBS = 1, PDL_EARLY_DECKS = 2;
// nTilesDev (nullable): a device-side tile count; the launch covers
// min(nTiles, *nTilesDev) tiles (sized on the host for nTiles).
// early: PDL_EARLY_* bits (p4g_prune_common.cuh) -- what the stream's previous
// kernel does not write, so that the kernel may stage it before its wait.
int launchPrune(const PruneJob *dJobs, const BlockDesc *dBlocks, int nTiles, int dim, int nCat,
                int smemBytes, int shape, cudaStream_t s, const int *nTilesDev = nullptr, int early = 0);
int pruneNumShapes(int dim);
int pruneTile(int dim, int shape);
int pruneShapeValid(int dim, int nCat, int shape);
int pruneKernelExists(int dim, int nCat, int shape);
// cherryBlocks: cherry-list length (or capacity) x the largest nCat of the parts with tables
int launchCherry(const PruneJob *dJobs, int nJobs, long long cherryBlocks, cudaStream_t s);
// p4g_prune_tc.cu
int pruneTcSmemBytes(int nProg, int nTax, int nSlots, int nClade);
int launchPruneTc(const PruneJob *dJobs, const BlockDesc *dBlocks, int nTiles, int smemBytes, cudaStream_t s,
                  const int *nTilesDev = nullptr, int early = 0);
int pruneSmemBytes(int dim, int nCat, int nProg, int nNodes, int nTax, int nSlots, int shape, int nClade = 0,
                   int nDeck = -1, int nRow = -1);

// host math shared with device code (p4g_math.cuh)
int discreteGammaHost(double alpha, int K, double *rates);

}  // namespace p4g

// Host helpers defined in p4g_api.cu and reused by p4g_noalloc.cu.
int buildProgram(p4g::Tree *t, std::vector<int> &prog, int &nSlots, std::vector<int4> *cherries = nullptr);
int computeNeed(p4g::Tree *t, std::vector<int> &need, std::vector<int> &order);
// p4g_api.cu, for p4g_sim.cu
int treeLogLikeSites(p4g::Tree *t, double *lnL);
int setPramsForDraws(p4g::Tree *t);
int resetTreeDev(p4g::Tree *t);
int fp64Evaluate(p4g::Tree *t, bool doSetPrams, double *lnL);

int cladeSelect(p4g::Tree *t, const std::vector<int> &order, std::vector<int> &cladeOf);
int cladeBuild(p4g::Tree *t, const std::vector<int> &need, const std::vector<int> &cladeOf);
// early: PDL_EARLY_* bits for the first clade launch (later ones follow a
// clade launch and stage their jobs and decks early)
int cladeLaunch(p4g::Tree *t, cudaStream_t s, int early = 0);
// The clade-table work of several trees as one launch per (dim, nCat) group:
// every tree's clade jobs copied into dJobs, their tile lists merged on the
// device into dBlocks with the totals in dCounts (groups: one per group,
// blk0 / nBlk the merged list's region and capacity).  Returns P4G_OK with
// groups empty when the trees' clade groups differ (then each tree launches
// its own).
int cladeMerge(const std::vector<p4g::Tree *> &trees, p4g::DevBuf &dJobs, p4g::DevBuf &dBlocks,
               p4g::DevBuf &dCounts, p4g::DevBuf &dSrc, std::vector<p4g::PruneGroup> &groups, cudaStream_t s);
int emitProgram(p4g::Tree *t, int r, const std::vector<int> &need, std::vector<int> &prog,
                std::vector<int4> *cherries, const std::vector<int> *cladeOf, const std::vector<int> *rowOf);
void buildCompact(p4g::Part *p);
int compactCode(const p4g::Part *p, int c);
int validateModel(p4g::Tree *t, int pNum);
int defaultShape(int dim);
