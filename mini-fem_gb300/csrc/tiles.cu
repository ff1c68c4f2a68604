// FP32 assembly by spatial tiles of rows (owner computes, one CTA per tile).
//
// The rows (nodes) are put in Morton order of their coordinates and cut into
// tiles of at most maxRows rows whose incident elements number at most maxElem.
// One CTA per tile:
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
//      compensation and writes the 3x3 block (or scalar) to the CSR values;
//      warps take 32 entries at a time from a shared counter, so that the warps
//      of 3a and 3b join when their work is done.
// The plan is built once per mesh on the host from the device pattern.  Every
// contribution list is in ascending element order and every combination order
// is fixed, so results are deterministic.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <exception>
#include <numeric>
#include <thread>
#include <vector>

#include "context.h"
#include "elem32.cuh"
#include "tiles.cuh"
#include "tile_body.cuh"

namespace mfem {

namespace {

template <int OP, bool PREC>
__global__ void __launch_bounds__(kTileThreads, 4)
k_tile32(TilePlanView P, TileMesh M, TileSets S, SmemLayout L, float qthr2, int *counters,
         TileCtl ctl) {
    extern __shared__ __align__(16) unsigned char sm[];
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

uint32_t spread3(uint32_t v) {   // 10 bits -> every third bit
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}

int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Contribution code: local element l, and the gradient slots of its nodes j and
// k as the tile kernel lays them out (slot of node j = (j + l / 2) mod 4, see
// gslot), so that the kernel finds gradient j at slot index code >> 2.
unsigned short contrib_code(int l, int j, int k) {
    const int r = l >> 1;
    return (unsigned short)((l << 4) | (((j + r) & 3) << 2) | ((k + r) & 3));
}

}  // namespace

SmemLayout smem_layout(int maxElem, int maxContribPad, int maxOffPad, int maxRowsPad, int maxNodes) {
    SmemLayout L;
    L.w = maxElem * 64;                                 // gradients: 4 float4 per element
    L.contrib = L.w + round_up(maxElem * 8, 16);        // weights: float2 per element
    L.diag = L.contrib + round_up(maxContribPad * 2, 16);
    L.off = L.diag + maxRowsPad * 8;                    // after phase 1: off-diagonal table,
    L.res = L.off + maxOffPad * 16;                     //   then the row results
    L.x = L.off;                                        // during phase 1: coordinates,
    L.q = L.x + maxNodes * 32;                          //   then the flagged-element queue
    const int lateEnd = std::max(L.res + maxRowsPad * 4 * kResStride, L.q + maxElem * 2);
    L.bar = round_up(lateEnd, 16);
    L.bytes = L.bar + 16;                               // two mbarriers
    return L;
}

// Host-side plan construction (once per mesh and pattern).
namespace {
void build_tile_plan_impl(Context &c);
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
        build_tile_plan_impl(c);
    } catch (const Error &e) {
        if (e.code != MFEM_ERR_CAPACITY) throw;
        tp.unfit = true;
        tp.built = true;
    }
}

namespace {

// The plan is built in three passes: the rows in Morton order are cut into
// tiles (sequential: a tile grows while its rows' elements fit), every tile's
// lists are then built independently on all host threads, and the per-tile
// lists are finally laid end to end with the padding the bulk copies need.
struct TileLists {
    std::vector<int> elems, nodes;
    std::vector<ushort4> lconn;
    std::vector<unsigned short> contrib;
    std::vector<int2> diag;
    std::vector<int4> off;
};

void build_tile_plan_impl(Context &c) {
    TilePlan &tp = c.tiles;
    build_incidence(c);
    const int N = c.nbNodes, E = c.nbElem, nnz = c.nnz;
    std::vector<double> coord((size_t)N * 3);
    std::vector<int> e2n((size_t)E * 4), nptr(N + 1), nelem((size_t)E * 4), rowPtr(N + 1),
        col((size_t)nnz);
    MFEM_CUDA(cudaMemcpyAsync(coord.data(), c.coord.ptr, coord.size() * 8, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(e2n.data(), c.e2n.ptr, e2n.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(nptr.data(), c.nodeElemPtr.ptr, nptr.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(nelem.data(), c.nodeElem.ptr, nelem.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(rowPtr.data(), c.rowPtr.ptr, rowPtr.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(col.data(), c.col.ptr, col.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));

    // Morton order of the nodes (10 bits per axis over the bounding box)
    double lo3[3] = {1e300, 1e300, 1e300}, hi3[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < N; i++)
        for (int d = 0; d < 3; d++) {
            lo3[d] = std::min(lo3[d], coord[3 * (size_t)i + d]);
            hi3[d] = std::max(hi3[d], coord[3 * (size_t)i + d]);
        }
    std::vector<uint64_t> key(N);
    for (int i = 0; i < N; i++) {
        uint32_t q[3];
        for (int d = 0; d < 3; d++) {
            const double span = hi3[d] > lo3[d] ? hi3[d] - lo3[d] : 1.0;
            const double f = (coord[3 * (size_t)i + d] - lo3[d]) / span;
            q[d] = (uint32_t)std::min(1023.0, std::max(0.0, f * 1023.0));
        }
        const uint64_t m = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
        key[i] = (m << 32) | (uint32_t)i;
    }
    std::sort(key.begin(), key.end());

    // 1. the cut: consecutive rows while the tile's incident elements fit
    std::vector<int> tileRowBegin, rowOrder(N), rowTile(N, -1), rowLocal(N, 0), mark(E, -1);
    {
        int i = 0, elemCount = 0;
        while (i < N) {
            const int t = (int)tileRowBegin.size();
            tileRowBegin.push_back(i);
            elemCount = 0;
            int nr = 0;
            while (i < N && nr < tp.maxRows) {
                const int r = (int)(key[i] & 0xffffffffu);
                int add = 0;
                for (int q = nptr[r]; q < nptr[r + 1]; q++)
                    if (mark[nelem[q] >> 2] != t) add++;
                if (nr > 0 && elemCount + add > tp.maxElem) break;
                MFEM_REQUIRE(elemCount + add <= tp.maxElem, MFEM_ERR_CAPACITY,
                             "tile plan: one row touches more elements than a tile holds");
                for (int q = nptr[r]; q < nptr[r + 1]; q++) mark[nelem[q] >> 2] = t;
                elemCount += add;
                rowOrder[i] = r;
                rowTile[r] = t;
                rowLocal[r] = nr++;
                i++;
            }
        }
        tileRowBegin.push_back(N);
    }
    MFEM_REQUIRE(tp.maxElem <= 4096, MFEM_ERR_CAPACITY, "tile plan: local index overflow");
    const int nTiles = (int)tileRowBegin.size() - 1;

    // 2. every tile's lists, tiles spread over the host threads
    std::vector<TileLists> lists(nTiles);
    auto buildTile = [&](int t, std::vector<int> &posInRow) {
        TileLists &L = lists[t];
        const int r0 = tileRowBegin[t], nRows = tileRowBegin[t + 1] - r0;
        for (int lr = 0; lr < nRows; lr++) {
            const int r = rowOrder[r0 + lr];
            for (int q = nptr[r]; q < nptr[r + 1]; q++) L.elems.push_back(nelem[q] >> 2);
        }
        std::sort(L.elems.begin(), L.elems.end());
        L.elems.erase(std::unique(L.elems.begin(), L.elems.end()), L.elems.end());
        for (int e : L.elems)
            for (int k = 0; k < 4; k++) L.nodes.push_back(e2n[4 * (size_t)e + k]);
        std::sort(L.nodes.begin(), L.nodes.end());
        L.nodes.erase(std::unique(L.nodes.begin(), L.nodes.end()), L.nodes.end());
        auto nodeLocal = [&](int n) {
            return (unsigned short)(std::lower_bound(L.nodes.begin(), L.nodes.end(), n) - L.nodes.begin());
        };
        auto elemLocal = [&](int e) {
            return (int)(std::lower_bound(L.elems.begin(), L.elems.end(), e) - L.elems.begin());
        };
        L.lconn.reserve(L.elems.size());
        for (int e : L.elems) {
            const size_t b4 = 4 * (size_t)e;
            L.lconn.push_back(make_ushort4(nodeLocal(e2n[b4]), nodeLocal(e2n[b4 + 1]),
                                           nodeLocal(e2n[b4 + 2]), nodeLocal(e2n[b4 + 3])));
        }
        std::vector<int> cnt, start, fill;
        std::vector<char> keep;
        for (int lr = 0; lr < nRows; lr++) {
            const int r = rowOrder[r0 + lr];
            const int b = rowPtr[r], len = rowPtr[r + 1] - b;
            // position of each column of row r in the row (node-indexed, reset below)
            for (int m = 0; m < len; m++) posInRow[col[b + m]] = m;
            // which entries of the row this tile computes: the diagonal, entries to
            // rows outside the tile, and (r, c) with c a later row of the tile,
            // which also yields (c, r) transposed
            keep.assign(len, 0);
            for (int m = 0; m < len; m++) {
                const int cc = col[b + m];
                keep[m] = cc == r || rowTile[cc] != t || rowLocal[cc] > lr;
            }
            cnt.assign(len, 0);
            for (int q = nptr[r]; q < nptr[r + 1]; q++) {
                const int e = nelem[q] >> 2;
                for (int k = 0; k < 4; k++) {
                    const int m = posInRow[e2n[4 * (size_t)e + k]];
                    MFEM_REQUIRE(m >= 0, MFEM_ERR_PATTERN, "tile plan: pattern misses an element pair");
                    cnt[m]++;
                }
            }
            start.assign(len + 1, 0);
            for (int m = 0; m < len; m++) start[m + 1] = start[m] + (keep[m] ? cnt[m] : 0);
            const int base = (int)L.contrib.size();
            L.contrib.resize(L.contrib.size() + start[len]);
            fill.assign(len, 0);
            for (int q = nptr[r]; q < nptr[r + 1]; q++) {
                const int e = nelem[q] >> 2, j = nelem[q] & 3;
                for (int k = 0; k < 4; k++) {
                    const int m = posInRow[e2n[4 * (size_t)e + k]];
                    if (!keep[m]) continue;
                    L.contrib[base + start[m] + fill[m]++] = contrib_code(elemLocal(e), j, k);
                }
            }
            bool hasDiag = false;
            for (int m = 0; m < len; m++) {
                if (!keep[m]) continue;
                MFEM_REQUIRE(cnt[m] <= 255 && base + start[m] < (1 << 23), MFEM_ERR_CAPACITY,
                             "tile plan: too many contributions for one entry");
                const int meta = ((base + start[m]) << 8) | cnt[m];
                const int cc = col[b + m];
                if (cc == r) {
                    L.diag.push_back(make_int2(r, meta));
                    hasDiag = true;
                } else {
                    int tpos = -1;
                    if (rowTile[cc] == t) {
                        const int cb = rowPtr[cc], clen = rowPtr[cc + 1] - cb;
                        for (int mm = 0; mm < clen; mm++)
                            if (col[cb + mm] == r) { tpos = cb + mm; break; }
                        MFEM_REQUIRE(tpos >= 0, MFEM_ERR_PATTERN, "tile plan: pattern is not symmetric");
                    }
                    L.off.push_back(make_int4(b + m, tpos, meta, 0));
                }
            }
            if (!hasDiag) L.diag.push_back(make_int2(r, 0));
            for (int m = 0; m < len; m++) posInRow[col[b + m]] = -1;
        }
    };
    {
        const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        const int nThreads = (int)std::min<long long>(hw, std::max(1, nTiles / 16));
        std::atomic<int> nextTile(0);
        std::vector<std::exception_ptr> errs(nThreads);
        auto worker = [&](int w) {
            try {
                std::vector<int> posInRow(N, -1);
                for (int t; (t = nextTile.fetch_add(1)) < nTiles;) buildTile(t, posInRow);
            } catch (...) {
                errs[w] = std::current_exception();
                nextTile.store(nTiles);
            }
        };
        std::vector<std::thread> pool;
        for (int w = 1; w < nThreads; w++) pool.emplace_back(worker, w);
        worker(0);
        for (auto &th : pool) th.join();
        for (auto &e : errs)
            if (e) std::rethrow_exception(e);
    }

    // 3. the lists end to end; every segment starts 16-byte aligned and is padded
    // to whole 16-byte units that lie inside the arrays (one bulk copy each)
    std::vector<TileDesc> tiles(nTiles);
    size_t nE = 0, nN = 0, nC = 0, nD = 0, nO = 0;
    for (const TileLists &L : lists) {
        nE += L.elems.size();
        nN += L.nodes.size();
        nC += L.contrib.size() + 8;
        nD += L.diag.size() + 1;
        nO += L.off.size();
    }
    std::vector<int> tileElems, tileNodes;
    std::vector<ushort4> lconn;
    std::vector<unsigned short> contrib;
    std::vector<int2> diagEnt;
    std::vector<int4> offEnt;
    tileElems.reserve(nE);
    lconn.reserve(nE);
    tileNodes.reserve(nN);
    contrib.reserve(nC);
    diagEnt.reserve(nD);
    offEnt.reserve(nO);
    int maxElem = 0, maxContrib = 0, maxOff = 0, maxRows = 0, maxNodes = 0;
    for (int t = 0; t < nTiles; t++) {
        TileLists &L = lists[t];
        TileDesc &T = tiles[t];
        T.elemBegin = (int)tileElems.size();
        T.nElem = (int)L.elems.size();
        tileElems.insert(tileElems.end(), L.elems.begin(), L.elems.end());
        lconn.insert(lconn.end(), L.lconn.begin(), L.lconn.end());
        T.nodeBegin = (int)tileNodes.size();
        T.nNodes = (int)L.nodes.size();
        tileNodes.insert(tileNodes.end(), L.nodes.begin(), L.nodes.end());
        T.offBegin = (int)offEnt.size();
        T.diagBegin = (int)diagEnt.size();
        T.contribBegin = (int)contrib.size();
        T.nRows = tileRowBegin[t + 1] - tileRowBegin[t];
        offEnt.insert(offEnt.end(), L.off.begin(), L.off.end());
        diagEnt.insert(diagEnt.end(), L.diag.begin(), L.diag.end());
        contrib.insert(contrib.end(), L.contrib.begin(), L.contrib.end());
        T.nOff = (int)L.off.size();
        T.nContrib = (int)L.contrib.size();
        while (diagEnt.size() % 2) diagEnt.push_back(make_int2(0, 0));
        while (contrib.size() % 8) contrib.push_back(0);
        T.nOffPad = (int)offEnt.size() - T.offBegin;
        T.nRowsPad = (int)diagEnt.size() - T.diagBegin;
        T.nContribPad = (int)contrib.size() - T.contribBegin;
        maxElem = std::max(maxElem, T.nElem);
        maxContrib = std::max(maxContrib, T.nContribPad);
        maxOff = std::max(maxOff, T.nOffPad);
        maxRows = std::max(maxRows, T.nRowsPad);
        maxNodes = std::max(maxNodes, T.nNodes);
        L = TileLists();   // release as we go
    }

    tp.nTiles = (int)tiles.size();
    tp.layout = smem_layout(std::max(maxElem, 1), maxContrib, maxOff, maxRows, maxNodes);
    tp.planMax[0] = std::max(maxElem, 1);
    tp.planMax[1] = maxContrib;
    tp.planMax[2] = maxOff;
    tp.planMax[3] = maxRows;
    tp.planMax[4] = maxNodes;
    MFEM_REQUIRE(tp.layout.bytes <= 227 * 1024, MFEM_ERR_CAPACITY,
                 "tile plan: a tile needs more than 227 KB of shared memory");
    auto up = [&](DevBuf &d, const void *src, size_t bytes) {
        d.reserve(std::max<size_t>(bytes, 16));
        if (bytes) MFEM_CUDA(cudaMemcpyAsync(d.ptr, src, bytes, cudaMemcpyHostToDevice, c.stream));
    };
    up(tp.desc, tiles.data(), tiles.size() * sizeof(TileDesc));
    up(tp.elems, tileElems.data(), tileElems.size() * 4);
    up(tp.lconn, lconn.data(), lconn.size() * sizeof(ushort4));
    up(tp.nodes, tileNodes.data(), tileNodes.size() * 4);
    up(tp.offEnt, offEnt.data(), offEnt.size() * sizeof(int4));
    up(tp.diagEnt, diagEnt.data(), diagEnt.size() * sizeof(int2));
    up(tp.contrib, contrib.data(), contrib.size() * 2);
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    tp.nTileElems = 0;
    tp.nUnits = 0;
    tp.nContrib = 0;
    for (const TileDesc &T : tiles) {
        tp.nTileElems += T.nElem;
        tp.nUnits += T.nOff;
        tp.nContrib += T.nContrib;
    }
    tp.built = true;
}

}  // namespace

TilePlanView plan_view(const TilePlan &tp) {
    TilePlanView P;
    P.desc = tp.desc.as<TileDesc>();
    P.elems = tp.elems.as<int>();
    P.lconn = tp.lconn.as<ushort4>();
    P.nodes = tp.nodes.as<int>();
    P.offEnt = tp.offEnt.as<int4>();
    P.diagEnt = tp.diagEnt.as<int2>();
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
    c.timer.begin(fusePrec ? "tile32+prec" : "tile32", c.stream);
    auto launch = [&](auto kern) {
        MFEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes));
        kern<<<tp.nTiles, kTileThreads, L.bytes, c.stream>>>(P, M, S, L, q * q, st + 4,
                                                             TileCtl{c.waitLimit, c.testExtraTx});
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
