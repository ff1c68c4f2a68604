// Batched assembly: many meshes of uneven size, each with several coefficient
// sets, assembled per iteration by one replay of a CUDA graph.
//
// FP32: the graph holds the coordinate splits and ONE persistent launch of the
// tile kernel over a cross-mesh work list (every tile of every mesh; meshes
// largest first, tiles in plan order); CTAs take work items from an atomic
// counter; each item computes the
// tile's gradients once and its entries and preconditioner blocks for every
// coefficient set of its mesh.
// FP64: the graph holds, per mesh and set, the bit-exact gather launches:
// gradient records (for the first set of a mesh; later sets rewrite only the
// records' weights), diagonal units + preconditioner, off-diagonal units.
// Results equal the single-mesh entry points' bit for bit (same plans, same
// arithmetic).  No counterpart in the reference, which assembles one mesh per
// rank (src/FEM.cc:177-257).
#include <algorithm>
#include <string>
#include <vector>

#include "context.h"
#include "elem32.cuh"
#include "tiles.cuh"
#include "tile_body.cuh"

namespace mfem {

struct BatchMesh {
    TileMesh geo;
    TileSets sets;
    TilePlanView plan;
    int op;
};

void gather_fp64_sets(const Context &c, int op, const double *coef, double *rec, double *values,
                      double *prec, const unsigned char *mask, int *singular, cudaStream_t s,
                      bool gradientsReady);

}  // namespace mfem

// FP64 batch: meshes are spread over this many concurrent branches of the
// graph (each with its own gradient-record buffer), so that small meshes that
// cannot fill the GPU alone run side by side
constexpr int kBatchBranches = 4;

struct mfem_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side[kBatchBranches - 1] = {};   // the other branches while capturing
    cudaEvent_t fork = nullptr, join[kBatchBranches - 1] = {};
    size_t maxRec = 0;                            // doubles of one branch's record buffer
    std::string lastError;
    struct Item {
        mfem_context *ctx;
        int op, nSets;
        mfem::DevBuf coef;            // nSets x per-element coefficients (empty: constants)
        mfem::DevBuf w32;             // nSets x per-element FP32 weights
        bool hasCoef = false;
        size_t valOff = 0, precOff = 0, nodeOff = 0;
    };
    std::vector<Item *> items;
    mfem::DevBuf hilo, values32, values64, prec, recs, meshTable, desc, order, counters;
    size_t totalVal = 0, totalPrec = 0, totalNodes = 0;
    mfem::SmemLayout layout{};
    int nWork = 0, gridPersistent = 0;
    bool prepared = false;
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};   // [precision][prec]
    ~mfem_batch() {
        for (auto &g : graph)
            for (auto &h : g)
                if (h) cudaGraphExecDestroy(h);
        for (Item *it : items) delete it;
        for (auto &x : side)
            if (x) cudaStreamDestroy(x);
        if (fork) cudaEventDestroy(fork);
        for (auto &e : join)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace mfem {

namespace {

template <bool PREC>
__global__ void __launch_bounds__(kTileThreads, 4)
k_batch_tile32(const BatchMesh *__restrict__ meshes, const TileDesc *__restrict__ desc,
               const int *__restrict__ order, int nWork, SmemLayout L, float qthr2, int *counters,
               int *workCounter, TileCtl ctl) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int sWork;
    for (;;) {
        if (threadIdx.x == 0) sWork = atomicAdd(workCounter, 1);
        __syncthreads();
        const int w = sWork;
        __syncthreads();
        if (w >= nWork) return;
        const TileDesc T = desc[order[w]];
        const BatchMesh &B = meshes[T.mesh];
        bool ok;
        if (B.op == MFEM_OP_LAP)
            ok = tilek::tile_body<MFEM_OP_LAP, PREC>(T, B.geo, B.sets, B.plan, L, qthr2, sm, counters, ctl);
        else
            ok = tilek::tile_body<MFEM_OP_ELA, PREC>(T, B.geo, B.sets, B.plan, L, qthr2, sm, counters, ctl);
        if (!ok) return;
        __syncthreads();   // shared memory is reused by the next item
    }
}

int op_dim(int op) { return op == MFEM_OP_LAP ? 1 : 9; }

void prepare(mfem_batch &b) {
    if (b.prepared) return;
    MFEM_REQUIRE(!b.items.empty(), MFEM_ERR_STATE, "empty batch");
    // sizes and offsets
    b.totalVal = b.totalPrec = b.totalNodes = 0;
    int pm[5] = {1, 0, 0, 0, 0};   // plan maxima over the meshes (smem_layout's arguments)
    std::vector<TileDesc> all;
    std::vector<long long> cost;
    size_t maxRec = 0;
    for (size_t m = 0; m < b.items.size(); m++) {
        auto *it = b.items[m];
        Context &c = it->ctx->c;
        build_tile_plan(c);
        MFEM_REQUIRE(!c.tiles.unfit, MFEM_ERR_CAPACITY,
                     "batch: a mesh does not fit the tiles (a node touching more elements than a tile holds)");
        build_gather_plan(c);
        it->valOff = b.totalVal;
        it->precOff = b.totalPrec;
        it->nodeOff = b.totalNodes;
        b.totalVal += (size_t)c.nnz * op_dim(it->op) * it->nSets;
        b.totalPrec += (size_t)c.nbNodes * op_dim(it->op) * it->nSets;
        b.totalNodes += (size_t)c.nbNodes;
        maxRec = std::max(maxRec, (size_t)c.nbElem * 16);
        for (int k = 0; k < 5; k++) pm[k] = std::max(pm[k], c.tiles.planMax[k]);
        std::vector<TileDesc> d(c.tiles.nTiles);
        MFEM_CUDA(cudaMemcpy(d.data(), c.tiles.desc.ptr, sizeof(TileDesc) * d.size(), cudaMemcpyDeviceToHost));
        for (auto &t : d) {
            t.mesh = (int)m;
            all.push_back(t);
            cost.push_back((long long)t.nElem * 4 + (long long)t.nContrib * it->nSets);
        }
    }
    // shared-memory layout holding any tile of any mesh
    const SmemLayout L = smem_layout(pm[0], pm[1], pm[2], pm[3], pm[4]);
    b.layout = L;
    MFEM_REQUIRE(L.bytes <= 227 * 1024, MFEM_ERR_CAPACITY, "batch: tiles need more than 227 KB");
    // work list
    std::vector<int> ord(all.size());
    for (size_t i = 0; i < ord.size(); i++) ord[i] = (int)i;
    // meshes by total cost, largest first; a mesh's tiles stay in plan (Morton)
    // order, which keeps neighbouring tiles' reads and writes close in L2
    std::vector<long long> meshCost(b.items.size(), 0);
    for (size_t i = 0; i < all.size(); i++) meshCost[all[i].mesh] += cost[i];
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int x, int y) { return meshCost[all[x].mesh] > meshCost[all[y].mesh]; });
    b.nWork = (int)all.size();
    b.desc.reserve(sizeof(TileDesc) * all.size());
    MFEM_CUDA(cudaMemcpy(b.desc.ptr, all.data(), sizeof(TileDesc) * all.size(), cudaMemcpyHostToDevice));
    b.order.reserve(sizeof(int) * ord.size());
    MFEM_CUDA(cudaMemcpy(b.order.ptr, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice));
    b.hilo.reserve(sizeof(float4) * 2 * b.totalNodes);
    b.prec.reserve(sizeof(double) * b.totalPrec);
    b.maxRec = maxRec;
    b.recs.reserve(sizeof(double) * maxRec * kBatchBranches);
    b.counters.reserve(sizeof(int) * 8);
    // mesh table
    std::vector<BatchMesh> tab(b.items.size());
    float4 *hi = b.hilo.as<float4>();
    for (size_t m = 0; m < b.items.size(); m++) {
        auto *it = b.items[m];
        Context &c = it->ctx->c;
        BatchMesh &B = tab[m];
        B.geo.hl = hi + 2 * it->nodeOff;
        B.geo.coord = c.coord.as<double>();
        B.geo.e2n = c.e2n.as<int4>();
        B.geo.diagPos = c.diagPos.as<int>();
        B.geo.mask = c.hasMask ? c.mask.as<unsigned char>() : nullptr;
        B.sets.w = (const float2 *)it->w32.reserve(sizeof(float2) * (size_t)c.nbElem * it->nSets);
        B.sets.wStride = (size_t)c.nbElem;
        B.sets.values = nullptr;          // filled per precision below
        B.sets.valuesStride = (size_t)c.nnz * op_dim(it->op);
        B.sets.prec = b.prec.as<double>() + it->precOff;
        B.sets.precStride = (size_t)c.nbNodes * op_dim(it->op);
        B.sets.nSets = it->nSets;
        B.plan = plan_view(c.tiles);
        B.op = it->op;
    }
    b.meshTable.reserve(sizeof(BatchMesh) * tab.size() * 2);
    // two tables: one without and one with the preconditioner output
    for (auto &B : tab) B.sets.prec = nullptr;
    std::vector<BatchMesh> withPrec = tab;
    for (size_t m = 0; m < tab.size(); m++)
        withPrec[m].sets.prec = b.prec.as<double>() + b.items[m]->precOff;
    b.values32.reserve(sizeof(float) * b.totalVal);
    for (size_t m = 0; m < tab.size(); m++) {
        tab[m].sets.values = b.values32.as<float>() + b.items[m]->valOff;
        withPrec[m].sets.values = tab[m].sets.values;
    }
    MFEM_CUDA(cudaMemcpy(b.meshTable.ptr, tab.data(), sizeof(BatchMesh) * tab.size(), cudaMemcpyHostToDevice));
    MFEM_CUDA(cudaMemcpy(b.meshTable.as<BatchMesh>() + tab.size(), withPrec.data(),
                         sizeof(BatchMesh) * tab.size(), cudaMemcpyHostToDevice));
    // persistent grid: as many CTAs as fit on the device at once
    int sms = 0, perSM = 0;
    MFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b.device));
    MFEM_CUDA(cudaFuncSetAttribute(k_batch_tile32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes));
    MFEM_CUDA(cudaFuncSetAttribute(k_batch_tile32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes));
    MFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_batch_tile32<true>, kTileThreads, L.bytes));
    b.gridPersistent = std::max(1, std::min(b.nWork, sms * std::max(perSM, 1)));
    b.prepared = true;
}

void record32(mfem_batch &b, bool withPrec) {
    // the per-mesh coordinate splits and weights (two small launches a mesh)
    // over the concurrent branches, joined before the persistent kernel
    float4 *hi = b.hilo.as<float4>();
    MFEM_CUDA(cudaEventRecord(b.fork, b.stream));
    for (auto &x : b.side) MFEM_CUDA(cudaStreamWaitEvent(x, b.fork, 0));
    for (size_t m = 0; m < b.items.size(); m++) {
        auto *it = b.items[m];
        Context &c = it->ctx->c;
        const int k = (int)(m % kBatchBranches);
        cudaStream_t st = k == 0 ? b.stream : b.side[k - 1];
        split_coords(c, hi + 2 * it->nodeOff, st);
        const long long n = (long long)c.nbElem * (it->hasCoef ? it->nSets : 1);
        weights32_all(it->op, it->hasCoef ? it->coef.as<double>() : nullptr, n, it->w32.as<float2>(), st);
    }
    for (int j = 0; j < kBatchBranches - 1; j++) {
        MFEM_CUDA(cudaEventRecord(b.join[j], b.side[j]));
        MFEM_CUDA(cudaStreamWaitEvent(b.stream, b.join[j], 0));
    }
    int *cnt = b.counters.as<int>();
    MFEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * 8, b.stream));
    const BatchMesh *tab = b.meshTable.as<BatchMesh>() + (withPrec ? b.items.size() : 0);
    // flag thresholds: all contexts of a batch use the first one's
    const float q = b.items[0]->ctx->c.sliverThreshold;
    if (withPrec)
        k_batch_tile32<true><<<b.gridPersistent, kTileThreads, b.layout.bytes, b.stream>>>(
            tab, b.desc.as<TileDesc>(), b.order.as<int>(), b.nWork, b.layout, q * q, cnt, cnt + 4, TileCtl{1u << 22, 0u});
    else
        k_batch_tile32<false><<<b.gridPersistent, kTileThreads, b.layout.bytes, b.stream>>>(
            tab, b.desc.as<TileDesc>(), b.order.as<int>(), b.nWork, b.layout, q * q, cnt, cnt + 4, TileCtl{1u << 22, 0u});
    check_launch("k_batch_tile32");
}

// The FP64 batch as kBatchBranches concurrent branches forked from and joined
// to b.stream: each mesh (all its coefficient sets, which share its gradient
// records) goes to the branch with the least work so far (elements x sets),
// with that branch's record buffer.  The meshes write disjoint outputs; the
// singular-block counter is an integer sum.
void record64(mfem_batch &b, bool withPrec) {
    int *cnt = b.counters.as<int>();
    MFEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * 8, b.stream));
    MFEM_CUDA(cudaEventRecord(b.fork, b.stream));
    for (auto &x : b.side) MFEM_CUDA(cudaStreamWaitEvent(x, b.fork, 0));
    long long load[kBatchBranches] = {};
    for (auto *it : b.items) {
        Context &c = it->ctx->c;
        const int dim = op_dim(it->op);
        int k = 0;
        for (int j = 1; j < kBatchBranches; j++)
            if (load[j] < load[k]) k = j;
        load[k] += (long long)c.nbElem * it->nSets;
        cudaStream_t st = k == 0 ? b.stream : b.side[k - 1];
        double *rec = b.recs.as<double>() + (size_t)k * b.maxRec;
        for (int s = 0; s < it->nSets; s++) {
            const double *coef = it->hasCoef
                ? it->coef.as<double>() + (size_t)s * c.nbElem * (it->op == MFEM_OP_LAP ? 1 : 2)
                : nullptr;
            double *vals = b.values64.as<double>() + it->valOff + (size_t)s * c.nnz * dim;
            double *prec = withPrec ? b.prec.as<double>() + it->precOff + (size_t)s * c.nbNodes * dim
                                    : nullptr;
            gather_fp64_sets(c, it->op, coef, rec, vals, prec,
                             c.hasMask ? c.mask.as<unsigned char>() : nullptr, cnt, st, s > 0);
        }
    }
    for (int j = 0; j < kBatchBranches - 1; j++) {
        MFEM_CUDA(cudaEventRecord(b.join[j], b.side[j]));
        MFEM_CUDA(cudaStreamWaitEvent(b.stream, b.join[j], 0));
    }
}

cudaGraphExec_t graph_for(mfem_batch &b, int precision, bool withPrec) {
    cudaGraphExec_t &g = b.graph[precision][withPrec ? 1 : 0];
    if (g) return g;
    if (precision == MFEM_FP64) b.values64.reserve(sizeof(double) * b.totalVal);
    cudaGraph_t graph;
    MFEM_CUDA(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal));
    try {
        if (precision == MFEM_FP32) record32(b, withPrec);
        else record64(b, withPrec);
    } catch (...) {
        cudaStreamEndCapture(b.stream, &graph);
        throw;
    }
    MFEM_CUDA(cudaStreamEndCapture(b.stream, &graph));
    MFEM_CUDA(cudaGraphInstantiate(&g, graph, 0));
    cudaGraphDestroy(graph);
    return g;
}

template <class F>
int guarded(mfem_batch *b, F &&f) {
    if (!b) return MFEM_ERR_INVALID_ARG;
    try {
        MFEM_CUDA(cudaSetDevice(b->device));
        f(*b);
        b->lastError.clear();
        return MFEM_OK;
    } catch (const Error &e) {
        b->lastError = e.what();
        return e.code;
    }
}

}  // namespace
}  // namespace mfem

extern "C" {

int mfem_batch_create(mfem_batch **out, int device) {
    if (!out) return MFEM_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return MFEM_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return MFEM_ERR_INVALID_ARG;
    mfem_batch *b = new mfem_batch;
    b->device = device;
    const int rc = mfem::guarded(b, [](mfem_batch &bb) {
        MFEM_CUDA(cudaStreamCreateWithFlags(&bb.stream, cudaStreamNonBlocking));
        for (auto &x : bb.side) MFEM_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        MFEM_CUDA(cudaEventCreateWithFlags(&bb.fork, cudaEventDisableTiming));
        for (auto &e : bb.join) MFEM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    });
    if (rc != MFEM_OK) {
        delete b;
        return rc;
    }
    *out = b;
    return MFEM_OK;
}

int mfem_batch_destroy(mfem_batch *b) {
    if (!b) return MFEM_ERR_INVALID_ARG;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    delete b;
    return MFEM_OK;
}

const char *mfem_batch_last_error(const mfem_batch *b) {
    return b ? b->lastError.c_str() : "null batch";
}

int mfem_batch_get_stream(mfem_batch *b, void **stream) {
    if (!b || !stream) return MFEM_ERR_INVALID_ARG;
    *stream = (void *)b->stream;
    return MFEM_OK;
}

int mfem_batch_add(mfem_batch *b, mfem_context *ctx, int operatorID, int nbSets,
                   const double *coefSets) {
    return mfem::guarded(b, [&](mfem_batch &bb) {
        MFEM_REQUIRE(ctx, MFEM_ERR_INVALID_ARG, "null context");
        MFEM_REQUIRE(ctx->c.device == bb.device, MFEM_ERR_INVALID_ARG, "context on another device");
        MFEM_REQUIRE(ctx->c.hasPattern && ctx->c.hasCoords, MFEM_ERR_STATE,
                     "context needs a mesh with coordinates and a pattern");
        MFEM_REQUIRE(operatorID == MFEM_OP_LAP || operatorID == MFEM_OP_ELA, MFEM_ERR_INVALID_ARG,
                     "operatorID must be 0 or 1");
        MFEM_REQUIRE(nbSets >= 1 && (coefSets || nbSets == 1), MFEM_ERR_INVALID_ARG,
                     "nbSets >= 1, and coefficients for more than one set");
        auto *it = new mfem_batch::Item;
        it->ctx = ctx;
        it->op = operatorID;
        it->nSets = nbSets;
        if (coefSets) {
            const size_t n = (size_t)ctx->c.nbElem * (operatorID == MFEM_OP_LAP ? 1 : 2) * nbSets;
            it->coef.reserve(sizeof(double) * n);
            MFEM_CUDA(cudaMemcpy(it->coef.ptr, coefSets, sizeof(double) * n, cudaMemcpyHostToDevice));
            it->hasCoef = true;
        }
        bb.items.push_back(it);
        bb.prepared = false;
        for (auto &g : bb.graph)
            for (auto &h : g)
                if (h) {
                    cudaGraphExecDestroy(h);
                    h = nullptr;
                }
    });
}

int mfem_batch_set_coefficients(mfem_batch *b, int item, const double *coefSets) {
    return mfem::guarded(b, [&](mfem_batch &bb) {
        MFEM_REQUIRE(item >= 0 && item < (int)bb.items.size(), MFEM_ERR_INVALID_ARG, "no such item");
        auto *it = bb.items[item];
        MFEM_REQUIRE(it->hasCoef && coefSets, MFEM_ERR_STATE, "item was added without coefficients");
        const size_t n = (size_t)it->ctx->c.nbElem * (it->op == MFEM_OP_LAP ? 1 : 2) * it->nSets;
        MFEM_CUDA(cudaMemcpyAsync(it->coef.ptr, coefSets, sizeof(double) * n, cudaMemcpyHostToDevice,
                                  bb.stream));
    });
}

int mfem_batch_assemble(mfem_batch *b, int precision, int withPrec) {
    return mfem::guarded(b, [&](mfem_batch &bb) {
        MFEM_REQUIRE(precision == MFEM_FP32 || precision == MFEM_FP64, MFEM_ERR_INVALID_ARG,
                     "unknown precision");
        mfem::prepare(bb);
        cudaGraphExec_t g = mfem::graph_for(bb, precision, withPrec != 0);
        MFEM_CUDA(cudaGraphLaunch(g, bb.stream));
    });
}

int mfem_batch_synchronize(mfem_batch *b) {
    return mfem::guarded(b, [&](mfem_batch &bb) {
        MFEM_CUDA(cudaStreamSynchronize(bb.stream));
        int h[8];
        MFEM_CUDA(cudaMemcpy(h, bb.counters.ptr, sizeof(h), cudaMemcpyDeviceToHost));
        MFEM_REQUIRE(h[2] == 0, MFEM_ERR_TIMEOUT, "batch: a staged copy did not arrive in time");
    });
}

int mfem_batch_get_values(mfem_batch *b, int item, int set, int precision, void *values) {
    return mfem::guarded(b, [&](mfem_batch &bb) {
        MFEM_REQUIRE(bb.prepared && item >= 0 && item < (int)bb.items.size(), MFEM_ERR_INVALID_ARG,
                     "no such item");
        auto *it = bb.items[item];
        MFEM_REQUIRE(set >= 0 && set < it->nSets && values, MFEM_ERR_INVALID_ARG, "no such set");
        const size_t n = (size_t)it->ctx->c.nnz * mfem::op_dim(it->op);
        const size_t off = it->valOff + (size_t)set * n;
        MFEM_CUDA(cudaStreamSynchronize(bb.stream));
        if (precision == MFEM_FP32)
            MFEM_CUDA(cudaMemcpy(values, bb.values32.as<float>() + off, sizeof(float) * n, cudaMemcpyDeviceToHost));
        else
            MFEM_CUDA(cudaMemcpy(values, bb.values64.as<double>() + off, sizeof(double) * n, cudaMemcpyDeviceToHost));
    });
}

int mfem_batch_get_prec(mfem_batch *b, int item, int set, double *prec) {
    return mfem::guarded(b, [&](mfem_batch &bb) {
        MFEM_REQUIRE(bb.prepared && item >= 0 && item < (int)bb.items.size(), MFEM_ERR_INVALID_ARG,
                     "no such item");
        auto *it = bb.items[item];
        MFEM_REQUIRE(set >= 0 && set < it->nSets && prec, MFEM_ERR_INVALID_ARG, "no such set");
        const size_t n = (size_t)it->ctx->c.nbNodes * mfem::op_dim(it->op);
        MFEM_CUDA(cudaStreamSynchronize(bb.stream));
        MFEM_CUDA(cudaMemcpy(prec, bb.prec.as<double>() + it->precOff + (size_t)set * n,
                             sizeof(double) * n, cudaMemcpyDeviceToHost));
    });
}

int mfem_batch_info(mfem_batch *b, int *nbItems, long long *nbElemTotal, long long *nbAssemblies,
                    int *nbWork, int *grid) {
    return mfem::guarded(b, [&](mfem_batch &bb) {
        mfem::prepare(bb);
        long long e = 0, a = 0;
        for (auto *it : bb.items) {
            e += it->ctx->c.nbElem;
            a += (long long)it->ctx->c.nbElem * it->nSets;
        }
        if (nbItems) *nbItems = (int)bb.items.size();
        if (nbElemTotal) *nbElemTotal = e;
        if (nbAssemblies) *nbAssemblies = a;
        if (nbWork) *nbWork = bb.nWork;
        if (grid) *grid = bb.gridPersistent;
    });
}

}  // extern "C"
