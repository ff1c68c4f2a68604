// Device state of one mesh: inputs, CSR pattern, colouring, assembly plans and
// results, all resident in HBM for the lifetime of the context.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "tiles.cuh"

namespace mfem {

// Gather plan ("units").  A unit is one CSR entry (r, c) with c >= r in node
// order; its transpose (c, r) receives the transposed block, which is bitwise
// the same sum because block(k,j) = block(j,k)^T exactly and both entries see
// the same elements in the same ascending order.  contrib lists every
// (element, j, k) adding to the unit, ascending element id, packed
// e << 4 | j << 2 | k.
struct GatherPlan {
    bool built = false;
    int nUnits = 0;
    long long nContrib = 0;
    DevBuf unitStart;   // int [nUnits + 1]  offsets into contrib (in unit order)
    DevBuf unitPos;     // int2[nUnits]      (pos(r,c), pos(c,r)), by first element, then count
    DevBuf contrib;     // u32 [nContrib]
    int nDiagUnits = 0; // units [0, nDiagUnits) are diagonal entries
    DevBuf diagNode;    // int [nDiagUnits]  nodes by first incident element, then valence
};

// FP32 spatial-tile plan (tiles.cu): rows in Morton order cut into tiles of at
// most maxRows rows touching at most maxElem elements.
struct TilePlan {
    bool built = false;
    bool unfit = false;         // built, but the mesh does not fit the tiles
    int maxRows = 48, maxElem = 512;
    int nTiles = 0;
    long long nTileElems = 0;   // sum over tiles of their element counts
    long long nUnits = 0;       // off-diagonal units (an intra-tile pair counts once)
    long long nContrib = 0;     // contributions summed per coefficient set
    SmemLayout layout{};
    int planMax[5] = {1, 0, 0, 0, 0};   // largest tile: elements, contributions, off entries, rows, nodes
    DevBuf desc, elems, lconn, nodes, offEnt, diagEnt, contrib;
    DevBuf w32;                 // per-element weights of the current coefficients
};

// Interface-node sum of the preconditioner blocks between sub-domains (halo.cu),
// the device form of src/halo.cc:39-122.  Entry j of the interface lists is
// node[j]; the distinct interface nodes and, for each, its entries in
// interface order (the order the reference adds the received blocks in).
struct HaloPlan {
    bool built = false;
    int nbIntf = 0, nbIntfNodes = 0, nUniq = 0;
    DevBuf node;        // int [nbIntfNodes]  0-based local node of each entry
    DevBuf uniqNode;    // int [nUniq]
    DevBuf uniqStart;   // int [nUniq + 1]    into uniqEntry
    DevBuf uniqEntry;   // int [nbIntfNodes]  entry indices, interface order per node
};

struct Coloring {
    bool built = false;
    int nbColors = 0;
    std::vector<int> hOffsets;   // nbColors + 1, into colorElems
    DevBuf color;                // int [E]
    DevBuf colorElems;           // int [E] elements sorted by colour (stable)
    DevBuf perm;                 // int [E] new position of each element (colorPerm)
};

// Optional per-kernel CUDA-event timing (mfem_profile): each named launch
// region is bracketed by two events on the context stream.
struct KernelTimer {
    bool on = false;
    struct Rec { const char *name; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    size_t used = 0;
    void begin(const char *name, cudaStream_t s);
    void end(cudaStream_t s);
    void reset() { used = 0; }
    ~KernelTimer();
};

// Pipelined end-to-end steps (context.cu: mfem_step_async / mfem_wait): two result slots, so that the
// copy-out of step k (on its own stream) overlaps the inputs and the assembly
// of step k+1.  The slot of step k is k & 1; Context::values/prec always hold
// the slot of the latest step.
struct Pipeline {
    cudaStream_t copy = nullptr;
    cudaEvent_t computed = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr};   // copy-out of the slot finished
    bool recorded[2] = {false, false};
    DevBuf spareValues, sparePrec;                // the other slot
    int cur = 0;                                  // slot now in Context::values
    int *hostStatus = nullptr;                    // pinned int[2][8]: status per slot
    long long next = 0;                           // ticket of the next step
    ~Pipeline();
};

// An instantiated CUDA graph with the arguments it was captured with; a
// launch whose arguments differ re-captures it.
struct CachedGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<long long> key;
    CachedGraph() = default;
    CachedGraph(const CachedGraph &) = delete;
    CachedGraph &operator=(const CachedGraph &) = delete;
    ~CachedGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

struct Context {
    int device = 0;
    KernelTimer timer;
    cudaStream_t stream = nullptr;
    // second stream for independent kernels of one step (the FP64 gather's
    // diagonal and off-diagonal units), forked from and joined to `stream`
    // by the two events; made on first use, destroyed with the context
    cudaStream_t side = nullptr;
    cudaEvent_t sideFork = nullptr, sideJoin = nullptr;
    std::string lastError;

    // mesh
    int nbElem = 0, nbNodes = 0;
    bool hasCoords = false;
    DevBuf coord;      // double [N*3]
    DevBuf e2n;        // int    [E*4], 0-based
    const void *hostE2n = nullptr;   // identity of the caller's elemToNode
    unsigned long long hostE2nSig = 0;   // and a fingerprint of its contents

    // pattern
    bool hasPattern = false;
    int nnz = 0, order = MFEM_ORDER_SORTED;
    DevBuf rowPtr, col, diagPos;      // col 0-based
    DevBuf nodeElemPtr, nodeElem;     // incidence, ascending element per node
    bool hasIncidence = false;
    DevBuf elemPos;                   // int [E*16]
    bool hasElemPos = false;
    const void *hostRow = nullptr, *hostCol = nullptr;  // identity of caller's CSR

    GatherPlan gather;
    TilePlan tiles;
    Coloring coloring;
    int fp32Kernel = 1;               // 0: gradient records + unit gather, 1: tiles

    // coefficients
    int coefOp = -1;                  // -1: reference constants
    DevBuf coef;                      // double [E] or [E*2]
    DevBuf lame;                      // double [E*3]: (A, B, mu) of the ela coefficients
    bool lameValid = false;           //   made from coef by the FP64 gather when stale

    // Dirichlet mask, one byte per node: bit k = DOF k constrained
    DevBuf mask;
    bool hasMask = false;

    // results
    int lastOp = -1, lastPrecision = MFEM_FP64;
    DevBuf values;                    // double or float [nnz * opDim]
    DevBuf prec;                      // double [N * opDim]
    bool precIsInit = false;
    bool precBlocks = false;          // prec holds the diagonal blocks of the latest
                                      // assembly, not yet inverted (mfem_prec_init)
    HaloPlan halo;

    // FP32 path: elements whose quality |6V| / (|a||b||c|) is below this
    // threshold get their Jacobian in FP64; the count of the last assembly is
    // kept in status[5].
    float sliverThreshold = 0.1f;
    bool flaggedPending = false;
    // bounded device waits (tile kernel): polls before giving up, and bytes the
    // barrier expects on top of the real copies (testing the limit only)
    unsigned waitLimit = 1u << 22, testExtraTx = 0;

    // scratch
    DevBuf grad;                      // per-element gradient records
    DevBuf solver;                    // CG work vectors (solve.cu)
    DevBuf xsplit;                    // float2 [N*d]: hi/lo split of an SpMV operand (FP32 values)
    DevBuf scratch, scratch2, scanTmp;
    DevBuf status;                    // int[8] device-side error flags
    CachedGraph scatterGraph;         // the colour-ordered scatter (asm64.cu)

    // last member: destroyed first, so that its copies finish before the
    // buffers they read are freed
    std::unique_ptr<Pipeline> pipe;
};

// pattern.cu
void build_incidence(Context &c);
void build_pattern(Context &c, int order);
void build_pattern_from_incidence(Context &c, const int *hIndex, const int *hValue);
void adopt_pattern(Context &c, const int *hRow, const int *hCol, int nnz);
void build_elem_pos(Context &c);
void build_gather_plan(Context &c);

// tiles.cu, tileplan.cu
void build_tile_plan(Context &c);
void build_tile_plan_device(Context &c);
void assemble_tiles32(Context &c, int op, bool fusePrec);
void split_and_weights(Context &c, int op, float4 *hl, float2 *w);
TilePlanView plan_view(const TilePlan &tp);
void split_coords(const Context &c, float4 *hl, cudaStream_t s);
void weights32_all(int op, const double *coef, long long n, float2 *w, cudaStream_t s);

// coloring.cu
void build_coloring(Context &c, unsigned long long seed);

// asm64.cu
void assemble_fp64(Context &c, int op, int strategy, bool fusePrec);
void prec_init_fp64(Context &c, int op);
int  prec_invert(Context &c, int op);

// context.cu
void pipeline_guard(Context &c);

// solve.cu
int op_dim_of(const Context &c);
void spmv_device(Context &c, const double *x, double *y, int constrainedFlag);
void prec_apply_device(Context &c, const double *r, double *z);
void pcg(Context &c, const double *b, double *x, double rtol, int maxIter, int constrainedFlag,
         int *iters, double *relres);

// helpers in context.cu
int *status_ptr(Context &c);
void read_status(Context &c, int *h, int n);

}  // namespace mfem

// The opaque handle of the C ABI.
struct mfem_context {
    mfem::Context c;
};

namespace mfem {

// Runs f on the context with its device current and turns internal errors into
// the status code (message kept for mfem_last_error).
template <class F>
int run_guarded(mfem_context *ctx, F &&f) {
    if (!ctx) return MFEM_ERR_INVALID_ARG;
    try {
        MFEM_CUDA(cudaSetDevice(ctx->c.device));
        f(ctx->c);
        ctx->c.lastError.clear();
        return MFEM_OK;
    } catch (const Error &e) {
        ctx->c.lastError = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        ctx->c.lastError = "host allocation failed";
        return MFEM_ERR_CAPACITY;
    }
}

}  // namespace mfem
