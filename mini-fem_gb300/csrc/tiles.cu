// FP32 assembly by spatial tiles of rows (owner computes, one CTA per tile).
//
// The rows (nodes) are put in Morton order of their coordinates and cut into
// tiles of at most maxRows rows whose incident elements number at most maxElem.
// One CTA per tile (about four per SM):
//   -. one thread prefetches into L2 (cp.async.bulk.prefetch) the plan
//      segments of the tile that starts about one wave later, when this CTA's
//      slot frees (blockIdx + 4 x SMs); CTA 0 prefetches every tile descriptor;
//   0. one thread starts TMA bulk copies (cp.async.bulk, completion on an
//      mbarrier) of the tile's contribution lists and diagonal table;
//   1. meanwhile the CTA gathers the coordinates of the tile's nodes (one
//      32-byte sector per node) into the shared-memory region that the
//      off-diagonal table fills later, then computes the FP32 gradients of the
//      elements incident to the tile's rows (ascending element id,
//      connectivity as indices into the tile's node list) into shared memory:
//      each element once per tile that needs it, no records in HBM; elements
//      below the quality threshold are queued and get FP64 gradients in a
//      second pass by consecutive threads; the off-diagonal table is then
//      copied (second mbarrier) over the coordinates, and each warp waits for
//      it only when it reaches phase 2;
//   3a. four lanes per diagonal entry sum a quarter of its contributions each
//      and combine them with error-free additions; the first of the four writes
//      the block and keeps the compensated sums.  Only the warps these lanes
//      fill take part; the others start phase 2 at once;
//   3b. one thread per row (the first warps) masks the block and inverts it in
//      FP64 into the preconditioner, while the other warps run phase 2;
//   2. one thread per off-diagonal entry sums its contributions with Kahan
//      compensation (ela: two contributions per compensated addition, their
//      sum formed by an FMA) and writes the 3x3 block (or scalar) to the CSR
//      values;
//      warps take 32 entries at a time from a shared counter, so that the warps
//      of 3a and 3b join when their work is done.
// The plan is built once per mesh and pattern on the device (tileplan.cu).
// Every contribution list is in node -> element incidence order and every
// combination order is fixed, so results are deterministic.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "context.h"
#include "elem32.cuh"
#include "tiles.cuh"
#include "tile_body.cuh"

namespace mfem {

namespace {

// L2 prefetch of [base + off, + len) widened to 16-byte boundaries (the plan
// arrays are allocated with 16 bytes of slack, so the range stays inside them)
__device__ __forceinline__ void prefetch_range(const void *base, size_t off, size_t len) {
    if (!len) return;
    const uintptr_t a = reinterpret_cast<uintptr_t>(base) + off, b = a + len;
    const uintptr_t a16 = a & ~(uintptr_t)15, b16 = (b + 15) & ~(uintptr_t)15;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a16), "r"((unsigned)(b16 - a16))
                 : "memory");
}

template <int OP, bool PREC>
__global__ void __launch_bounds__(kTileThreads, 4)
k_tile32(TilePlanView P, TileMesh M, TileSets S, SmemLayout L, float qthr2, int *counters,
         TileCtl ctl) {
    extern __shared__ __align__(16) unsigned char sm[];
    if (threadIdx.x == 32) {
        // the descriptors of every tile, then the plan segments of the tile that
        // starts about one wave later (when this CTA's slot frees), into L2
        if (blockIdx.x == 0) prefetch_range(P.desc, 0, (size_t)ctl.nTiles * sizeof(TileDesc));
        const int nt = (int)blockIdx.x + ctl.pfDist;
        if (ctl.pfDist > 0 && nt < ctl.nTiles) {
            const TileDesc N = P.desc[nt];
            prefetch_range(P.contrib, (size_t)N.contribBegin * 2, (size_t)N.nContribPad * 2);
            prefetch_range(P.diagEnt, (size_t)N.diagBegin * 16, (size_t)N.nRowsPad * 16);
            prefetch_range(P.offEnt, (size_t)N.offBegin * 16, (size_t)N.nOffPad * 16);
            prefetch_range(P.lconn, (size_t)N.elemBegin * 8, (size_t)N.nElem * 8);
            prefetch_range(P.elems, (size_t)N.elemBegin * 4, (size_t)N.nElem * 4);
            prefetch_range(P.nodes, (size_t)N.nodeBegin * 4, (size_t)N.nNodes * 4);
        }
    }
    const TileDesc T = P.desc[blockIdx.x];
    tilek::tile_body<OP, PREC>(T, M, S, P, L, qthr2, sm, counters, ctl);
}

// Per-element weights of the FP32 blocks for n = E * nSets elements (sets laid
// out one after the other, as the coefficient arrays are).
template <int OP>
__global__ void k_weights32(const double *__restrict__ coef, long long n, float2 *__restrict__ w) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = weights32<OP>(coef, (int)i);
}

// hi and lo parts of node i side by side (hl[2i], hl[2i+1]): one 32-byte sector
__global__ void k_split_coords_t(const double *__restrict__ coord, int nbNodes,
                                 float4 *__restrict__ hl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbNodes) return;
    const double x = coord[3 * i], y = coord[3 * i + 1], z = coord[3 * i + 2];
    float xh, yh, zh, xl, yl, zl;
    split_hilo(x, xh, xl);
    split_hilo(y, yh, yl);
    split_hilo(z, zh, zl);
    hl[2 * i] = make_float4(xh, yh, zh, 0.f);
    hl[2 * i + 1] = make_float4(xl, yl, zl, 0.f);
}

// The FP32 step's two inputs in one launch: threads [0, nbNodes) split one
// node's coordinates, the next threads form one element's weights.
template <int OP>
__global__ void k_split_and_weights(const double *__restrict__ coord, int nbNodes,
                                    float4 *__restrict__ hl, const double *__restrict__ coef,
                                    long long nbElem, float2 *__restrict__ w) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nbNodes) {
        const int i = (int)t;
        const double x = coord[3 * (size_t)i], y = coord[3 * (size_t)i + 1], z = coord[3 * (size_t)i + 2];
        float xh, yh, zh, xl, yl, zl;
        split_hilo(x, xh, xl);
        split_hilo(y, yh, yl);
        split_hilo(z, zh, zl);
        hl[2 * (size_t)i] = make_float4(xh, yh, zh, 0.f);
        hl[2 * (size_t)i + 1] = make_float4(xl, yl, zl, 0.f);
    } else if (t - nbNodes < nbElem) {
        w[t - nbNodes] = weights32<OP>(coef, (int)(t - nbNodes));
    }
}

int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

SmemLayout smem_layout(int maxElem, int maxContribPad, int maxOffPad, int maxRowsPad, int maxNodes) {
    SmemLayout L;
    L.w = maxElem * 64;                                 // gradients: 4 float4 per element
    L.contrib = L.w + round_up(maxElem * 8, 16);        // weights: float2 per element
    L.diag = L.contrib + round_up(maxContribPad * 2, 16);
    L.off = L.diag + maxRowsPad * 16;                   // after phase 1: off-diagonal table,
    L.res = L.off + maxOffPad * 16;                     //   then the row results
    L.x = L.off;                                        // during phase 1: coordinates,
    L.q = L.x + maxNodes * 32;                          //   then the flagged-element queue
    const int lateEnd = std::max(L.res + maxRowsPad * 4 * kResStride, L.q + maxElem * 2);
    L.bar = round_up(lateEnd, 16);
    L.bytes = L.bar + 16;                               // two mbarriers
    return L;
}

// A mesh the tiles cannot hold (a node touching more elements than a tile,
// an entry with more than 255 contributions, a layout beyond shared memory) is
// marked unfit: the FP32 path then uses the record kernel, which has no such
// limit.
void build_tile_plan(Context &c) {
    TilePlan &tp = c.tiles;
    if (tp.built) return;
    tp.unfit = false;
    try {
        build_tile_plan_device(c);
    } catch (const Error &e) {
        if (e.code != MFEM_ERR_CAPACITY) throw;
        tp.unfit = true;
        tp.built = true;
    }
}


TilePlanView plan_view(const TilePlan &tp) {
    TilePlanView P;
    P.desc = tp.desc.as<TileDesc>();
    P.elems = tp.elems.as<int>();
    P.lconn = tp.lconn.as<ushort4>();
    P.nodes = tp.nodes.as<int>();
    P.offEnt = tp.offEnt.as<int4>();
    P.diagEnt = tp.diagEnt.as<int4>();
    P.contrib = tp.contrib.as<unsigned short>();
    return P;
}

void weights32_all(int op, const double *coef, long long n, float2 *w, cudaStream_t s) {
    if (op == MFEM_OP_LAP) k_weights32<MFEM_OP_LAP><<<blocks_for(n, 256), 256, 0, s>>>(coef, n, w);
    else k_weights32<MFEM_OP_ELA><<<blocks_for(n, 256), 256, 0, s>>>(coef, n, w);
    check_launch("k_weights32");
}

void split_coords(const Context &c, float4 *hl, cudaStream_t s) {
    k_split_coords_t<<<blocks_for(c.nbNodes, 256), 256, 0, s>>>(c.coord.as<double>(), c.nbNodes, hl);
    check_launch("k_split_coords_t");
}

// The FP32 step's inputs: coordinates split into hi + lo floats and the
// per-element weights of the current coefficients, one launch.
void split_and_weights(Context &c, int op, float4 *hl, float2 *w) {
    const int N = c.nbNodes;
    c.timer.begin("split_coords+weights", c.stream);
    const double *coef = c.coefOp == op ? c.coef.as<double>() : nullptr;
    const unsigned g = blocks_for((long long)N + c.nbElem, 256);
    if (op == MFEM_OP_LAP)
        k_split_and_weights<MFEM_OP_LAP><<<g, 256, 0, c.stream>>>(c.coord.as<double>(), N, hl, coef, c.nbElem, w);
    else
        k_split_and_weights<MFEM_OP_ELA><<<g, 256, 0, c.stream>>>(c.coord.as<double>(), N, hl, coef, c.nbElem, w);
    check_launch("k_split_and_weights");
    c.timer.end(c.stream);
}

void assemble_tiles32(Context &c, int op, bool fusePrec) {
    build_tile_plan(c);
    const TilePlan &tp = c.tiles;
    const int N = c.nbNodes;
    const int dim = op == MFEM_OP_LAP ? 1 : 9;
    c.values.reserve(sizeof(float) * (size_t)c.nnz * dim);
    double *prec = fusePrec ? (double *)c.prec.reserve(sizeof(double) * (size_t)N * dim) : nullptr;
    float4 *hl = (float4 *)c.scratch.reserve(sizeof(float4) * 2 * (size_t)N);
    float2 *w = (float2 *)c.tiles.w32.reserve(sizeof(float2) * (size_t)c.nbElem);
    split_and_weights(c, op, hl, w);
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st + 4, 0, sizeof(int) * 3, c.stream));
    TileMesh M;
    M.hl = hl;
    M.coord = c.coord.as<double>();
    M.e2n = c.e2n.as<int4>();
    M.diagPos = c.diagPos.as<int>();
    M.mask = c.hasMask ? c.mask.as<unsigned char>() : nullptr;
    TileSets S;
    S.w = w;
    S.wStride = 0;
    S.values = c.values.as<float>();
    S.valuesStride = 0;
    S.prec = prec;
    S.precStride = 0;
    S.nSets = 1;
    const TilePlanView P = plan_view(tp);
    const SmemLayout L = tp.layout;
    const float q = c.sliverThreshold;
    int sms = 0;
    MFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    c.timer.begin(fusePrec ? "tile32+prec" : "tile32", c.stream);
    auto launch = [&](auto kern) {
        MFEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes));
        kern<<<tp.nTiles, kTileThreads, L.bytes, c.stream>>>(P, M, S, L, q * q, st + 4,
                                                             TileCtl{c.waitLimit, c.testExtraTx, tp.nTiles,
                                                                     4 * sms});
    };
    if (op == MFEM_OP_LAP) {
        if (fusePrec) launch(k_tile32<MFEM_OP_LAP, true>);
        else launch(k_tile32<MFEM_OP_LAP, false>);
    } else {
        if (fusePrec) launch(k_tile32<MFEM_OP_ELA, true>);
        else launch(k_tile32<MFEM_OP_ELA, false>);
    }
    check_launch("k_tile32");
    c.timer.end(c.stream);
    c.flaggedPending = true;
    c.lastOp = op;
    c.lastPrecision = MFEM_FP32;
    c.precIsInit = fusePrec;
}

}  // namespace mfem

extern "C" int mfem_tile_info(mfem_context *ctx, int *nbTiles, long long *nbTileElems,
                              long long *nbUnits, long long *nbContrib, int *smemBytes) {
    if (!ctx) return MFEM_ERR_INVALID_ARG;
    try {
        MFEM_CUDA(cudaSetDevice(ctx->c.device));
        MFEM_REQUIRE(ctx->c.hasPattern, MFEM_ERR_STATE, "no CSR pattern");
        mfem::build_tile_plan(ctx->c);
        const mfem::TilePlan &tp = ctx->c.tiles;
        MFEM_REQUIRE(!tp.unfit, MFEM_ERR_CAPACITY,
                     "tile plan: the mesh does not fit the tiles (the FP32 path uses the record kernel)");
        if (nbTiles) *nbTiles = tp.nTiles;
        if (nbTileElems) *nbTileElems = tp.nTileElems;
        if (nbUnits) *nbUnits = tp.nUnits;
        if (nbContrib) *nbContrib = tp.nContrib;
        if (smemBytes) *smemBytes = tp.layout.bytes;
        return MFEM_OK;
    } catch (const mfem::Error &e) {
        ctx->c.lastError = e.what();
        return e.code;
    }
}
