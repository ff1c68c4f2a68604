// FP32 assembly by spatial tiles of rows (owner computes, one CTA per tile).
//
// The rows (nodes) are put in Morton order of their coordinates and cut into
// tiles of at most kTileRows rows whose incident elements number at most
// tileMaxElem.  One CTA per tile:
//   1. computes the FP32 gradients and weights of every element incident to its
//      rows (ascending element id) into shared memory -- each element once per
//      tile that needs it, no gradient records in HBM;
//   2. sums every off-diagonal entry of its rows from those gradients with Kahan
//      compensation, one thread per entry, and writes it to the CSR values;
//   3. sums the diagonal entries, writes them, and -- on the FP64 pipe, which
//      runs beside the other warps' FP32 and memory work -- masks and inverts the
//      3x3 (or 1x1) diagonal blocks into the preconditioner.
// The plan (tile rows, tile elements, per-entry contribution lists as 16-bit
// tile-local references) is built once per mesh on the host from the device
// pattern; every list is in ascending element order, so results are
// deterministic.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "context.h"
#include "elem32.cuh"

namespace mfem {

namespace {

constexpr int kTileThreads = 256;

struct TileDesc {
    int rowBegin, nRows;      // into tileRows
    int elemBegin, nElem;     // into tileElems
    int offBegin, nOff;       // into offPos / offMeta
    int contribBegin, pad;    // into contrib16
};

uint32_t spread3(uint32_t v) {   // 10 bits -> every third bit
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}

template <int OP, bool PREC>
__global__ void __launch_bounds__(kTileThreads)
k_tile32(const TileDesc *__restrict__ tiles, const int *__restrict__ tileRows,
         const int *__restrict__ tileElems, const int *__restrict__ offPos,
         const unsigned *__restrict__ offMeta, const unsigned *__restrict__ diagMeta,
         const unsigned short *__restrict__ contrib, const float4 *__restrict__ hi,
         const float4 *__restrict__ lo, const double *__restrict__ coord,
         const int4 *__restrict__ e2n, const double *__restrict__ coef,
         const int *__restrict__ diagPos, const unsigned char *__restrict__ mask, float qthr2,
         float *__restrict__ values, double *__restrict__ prec, int *counters) {
    extern __shared__ float4 sm[];
    const TileDesc T = tiles[blockIdx.x];
    float4 *G = sm;                    // 4 per element: g_j.xyz
    float4 *W = sm + 4 * T.nElem;      // 1 per element: (A, B, mu) or (kappa)
    const int tid = threadIdx.x;

    // 1. gradients of the tile's elements
    int flagged = 0;
    for (int i = tid; i < T.nElem; i += kTileThreads) {
        const int e = tileElems[T.elemBegin + i];
        float g[12];
        flagged += grad32(hi, lo, coord, e2n[e], qthr2, g);
#pragma unroll
        for (int j = 0; j < 4; j++) G[4 * i + j] = make_float4(g[3 * j], g[3 * j + 1], g[3 * j + 2], 0.f);
        W[i] = weights32<OP>(coef, e);
    }
    if (flagged) atomicAdd(counters + 1, flagged);
    __syncthreads();

    const unsigned short *cl = contrib + T.contribBegin;
    // 2. off-diagonal entries
    for (int t = tid; t < T.nOff; t += kTileThreads) {
        const unsigned meta = offMeta[T.offBegin + t];
        const int b = meta >> 8, n = meta & 0xff;
        const int pos = offPos[T.offBegin + t];
        if (OP == MFEM_OP_LAP) {
            Kahan acc;
            for (int q = b; q < b + n; q++) {
                const unsigned u = cl[q];
                const int l = u >> 4;
                const float4 gj = G[4 * l + ((u >> 2) & 3)], gk = G[4 * l + (u & 3)];
                acc.add(W[l].x * fmaf(gj.x, gk.x, fmaf(gj.y, gk.y, gj.z * gk.z)));
            }
            values[pos] = acc.value();
        } else {
            Kahan acc[9];
            for (int q = b; q < b + n; q++) {
                const unsigned u = cl[q];
                const int l = u >> 4;
                const float4 gj = G[4 * l + ((u >> 2) & 3)], gk = G[4 * l + (u & 3)];
                const float4 w = W[l];
                const float p00 = gj.x * gk.x, p11 = gj.y * gk.y, p22 = gj.z * gk.z;
                acc[0].add(fmaf(p00, w.x, (p11 + p22) * w.z));
                acc[4].add(fmaf(p11, w.x, (p00 + p22) * w.z));
                acc[8].add(fmaf(p22, w.x, (p00 + p11) * w.z));
                acc[1].add(gj.x * gk.y * w.y);
                acc[2].add(gj.x * gk.z * w.y);
                acc[3].add(gj.y * gk.x * w.y);
                acc[5].add(gj.y * gk.z * w.y);
                acc[6].add(gj.z * gk.x * w.y);
                acc[7].add(gj.z * gk.y * w.y);
            }
            float *v = values + (size_t)pos * 9;
#pragma unroll
            for (int m = 0; m < 9; m++) v[m] = acc[m].value();
        }
    }

    // 3. diagonal entries + preconditioner
    for (int t = tid; t < T.nRows; t += kTileThreads) {
        const int r = tileRows[T.rowBegin + t];
        const unsigned meta = diagMeta[T.rowBegin + t];
        const int b = meta >> 8, n = meta & 0xff;
        const int p = diagPos[r];
        if (OP == MFEM_OP_LAP) {
            Kahan acc;
            for (int q = b; q < b + n; q++) {
                const unsigned u = cl[q];
                const int l = u >> 4;
                const float4 g = G[4 * l + ((u >> 2) & 3)];
                acc.add(W[l].x * fmaf(g.x, g.x, fmaf(g.y, g.y, g.z * g.z)));
            }
            if (p >= 0) values[p] = acc.value();
            if (PREC) prec[r] = 1.0 / ((double)acc.s - (double)acc.c);
        } else {
            Kahan acc[6];
            for (int q = b; q < b + n; q++) {
                const unsigned u = cl[q];
                const int l = u >> 4;
                const float4 g = G[4 * l + ((u >> 2) & 3)];
                const float4 w = W[l];
                const float p00 = g.x * g.x, p11 = g.y * g.y, p22 = g.z * g.z;
                acc[0].add(fmaf(p00, w.x, (p11 + p22) * w.z));
                acc[1].add(fmaf(p11, w.x, (p00 + p22) * w.z));
                acc[2].add(fmaf(p22, w.x, (p00 + p11) * w.z));
                acc[3].add(g.x * g.y * w.y);
                acc[4].add(g.x * g.z * w.y);
                acc[5].add(g.y * g.z * w.y);
            }
            if (p >= 0) {
                float *v = values + (size_t)p * 9;
                const float d0 = acc[0].value(), d4 = acc[1].value(), d8 = acc[2].value();
                const float o1 = acc[3].value(), o2 = acc[4].value(), o5 = acc[5].value();
                v[0] = d0; v[1] = o1; v[2] = o2;
                v[3] = o1; v[4] = d4; v[5] = o5;
                v[6] = o2; v[7] = o5; v[8] = d8;
            }
            if (PREC) {
                double s[6];
#pragma unroll
                for (int m = 0; m < 6; m++) s[m] = (double)acc[m].s - (double)acc[m].c;
                double a[9] = {s[0], s[3], s[4], s[3], s[1], s[5], s[4], s[5], s[2]};
                if (mask) dirichlet_mask3(a, mask[r]);
                if (p >= 0 && !inv3_cofactor(a)) atomicAdd(counters, 1);
                double *o = prec + (size_t)r * 9;   // 72-byte blocks: 8-byte aligned only
#pragma unroll
                for (int m = 0; m < 9; m++) o[m] = a[m];
            }
        }
    }
}

__global__ void k_split_coords_t(const double *__restrict__ coord, int nbNodes,
                                 float4 *__restrict__ hi, float4 *__restrict__ lo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbNodes) return;
    const double x = coord[3 * i], y = coord[3 * i + 1], z = coord[3 * i + 2];
    const float xh = __double2float_rn(x), yh = __double2float_rn(y), zh = __double2float_rn(z);
    hi[i] = make_float4(xh, yh, zh, 0.f);
    lo[i] = make_float4(__double2float_rn(x - (double)xh), __double2float_rn(y - (double)yh),
                        __double2float_rn(z - (double)zh), 0.f);
}

}  // namespace

// Host-side plan construction (once per mesh and pattern).
void build_tile_plan(Context &c) {
    TilePlan &tp = c.tiles;
    if (tp.built) return;
    build_incidence(c);
    const int N = c.nbNodes, E = c.nbElem, nnz = c.nnz;
    std::vector<double> coord((size_t)N * 3);
    std::vector<int> e2n((size_t)E * 4), nptr(N + 1), nelem((size_t)E * 4), rowPtr(N + 1),
        col((size_t)nnz), diagPos(N);
    MFEM_CUDA(cudaMemcpyAsync(coord.data(), c.coord.ptr, coord.size() * 8, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(e2n.data(), c.e2n.ptr, e2n.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(nptr.data(), c.nodeElemPtr.ptr, nptr.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(nelem.data(), c.nodeElem.ptr, nelem.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(rowPtr.data(), c.rowPtr.ptr, rowPtr.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(col.data(), c.col.ptr, col.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(diagPos.data(), c.diagPos.ptr, diagPos.size() * 4, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));

    // Morton order of the nodes
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
            double f = (coord[3 * (size_t)i + d] - lo3[d]) / span;
            q[d] = (uint32_t)std::min(1023.0, std::max(0.0, f * 1023.0));
        }
        const uint64_t m = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
        key[i] = (m << 32) | (uint32_t)i;
    }
    std::sort(key.begin(), key.end());

    std::vector<TileDesc> tiles;
    std::vector<int> tileRows, tileElems, offPos;
    std::vector<unsigned> offMeta, diagMeta;
    std::vector<unsigned short> contrib;
    tileRows.reserve(N);
    offPos.reserve((size_t)nnz);
    offMeta.reserve((size_t)nnz);
    diagMeta.reserve(N);
    contrib.reserve((size_t)E * 16 + 1024);
    std::vector<int> mark(E, -1), local(E, 0);
    std::vector<int> elems;
    std::vector<int> cnt, fill;

    const int maxElem = tp.maxElem;
    int i = 0;
    while (i < N) {
        const int tIndex = (int)tiles.size();
        TileDesc T{};
        T.rowBegin = (int)tileRows.size();
        elems.clear();
        int nRows = 0;
        // grow the tile
        while (i < N && nRows < tp.maxRows) {
            const int r = (int)(key[i] & 0xffffffffu);
            int add = 0;
            for (int q = nptr[r]; q < nptr[r + 1]; q++)
                if (mark[nelem[q] >> 2] != tIndex) add++;
            if (nRows > 0 && (int)elems.size() + add > maxElem) break;
            MFEM_REQUIRE((int)elems.size() + add <= maxElem, MFEM_ERR_CAPACITY,
                         "tile plan: one row touches more elements than a tile holds");
            for (int q = nptr[r]; q < nptr[r + 1]; q++) {
                const int e = nelem[q] >> 2;
                if (mark[e] != tIndex) {
                    mark[e] = tIndex;
                    elems.push_back(e);
                }
            }
            tileRows.push_back(r);
            nRows++;
            i++;
        }
        std::sort(elems.begin(), elems.end());
        for (int k = 0; k < (int)elems.size(); k++) local[elems[k]] = k;
        T.nRows = nRows;
        T.elemBegin = (int)tileElems.size();
        T.nElem = (int)elems.size();
        tileElems.insert(tileElems.end(), elems.begin(), elems.end());
        T.offBegin = (int)offPos.size();
        T.contribBegin = (int)contrib.size();
        // contribution lists, row by row
        for (int t = 0; t < nRows; t++) {
            const int r = tileRows[T.rowBegin + t];
            const int b = rowPtr[r], len = rowPtr[r + 1] - b;
            cnt.assign(len, 0);
            auto where = [&](int cc) {
                for (int m = 0; m < len; m++)
                    if (col[b + m] == cc) return m;
                return -1;
            };
            for (int q = nptr[r]; q < nptr[r + 1]; q++) {
                const int e = nelem[q] >> 2;
                for (int k = 0; k < 4; k++) {
                    const int m = where(e2n[4 * (size_t)e + k]);
                    MFEM_REQUIRE(m >= 0, MFEM_ERR_PATTERN, "tile plan: pattern misses an element pair");
                    cnt[m]++;
                }
            }
            std::vector<int> start(len + 1, 0);
            for (int m = 0; m < len; m++) start[m + 1] = start[m] + cnt[m];
            const int base = (int)contrib.size() - T.contribBegin;
            contrib.resize(contrib.size() + start[len]);
            fill.assign(len, 0);
            for (int q = nptr[r]; q < nptr[r + 1]; q++) {
                const int e = nelem[q] >> 2, j = nelem[q] & 3;
                for (int k = 0; k < 4; k++) {
                    const int m = where(e2n[4 * (size_t)e + k]);
                    contrib[T.contribBegin + base + start[m] + fill[m]++] =
                        (unsigned short)((local[e] << 4) | (j << 2) | k);
                }
            }
            for (int m = 0; m < len; m++) {
                MFEM_REQUIRE(cnt[m] <= 255 && base + start[m] < (1 << 24), MFEM_ERR_CAPACITY,
                             "tile plan: too many contributions for one entry");
                const unsigned meta = ((unsigned)(base + start[m]) << 8) | (unsigned)cnt[m];
                if (col[b + m] == r) {
                    diagMeta.push_back(meta);
                } else {
                    offPos.push_back(b + m);
                    offMeta.push_back(meta);
                }
            }
            if (diagPos[r] < 0) diagMeta.push_back(0u);
        }
        T.nOff = (int)offPos.size() - T.offBegin;
        tiles.push_back(T);
    }
    MFEM_REQUIRE(tp.maxElem * 16 <= (1 << 16), MFEM_ERR_CAPACITY, "tile plan: local index overflow");

    tp.nTiles = (int)tiles.size();
    auto up = [&](DevBuf &d, const void *src, size_t bytes) {
        d.reserve(bytes);
        MFEM_CUDA(cudaMemcpyAsync(d.ptr, src, bytes, cudaMemcpyHostToDevice, c.stream));
    };
    up(tp.desc, tiles.data(), tiles.size() * sizeof(TileDesc));
    up(tp.rows, tileRows.data(), tileRows.size() * 4);
    up(tp.elems, tileElems.data(), tileElems.size() * 4);
    up(tp.offPos, offPos.data(), std::max<size_t>(offPos.size(), 1) * 4);
    up(tp.offMeta, offMeta.data(), std::max<size_t>(offMeta.size(), 1) * 4);
    up(tp.diagMeta, diagMeta.data(), diagMeta.size() * 4);
    up(tp.contrib, contrib.data(), std::max<size_t>(contrib.size(), 1) * 2);
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    tp.nTileElems = (long long)tileElems.size();
    tp.built = true;
}

void assemble_tiles32(Context &c, int op, bool fusePrec) {
    build_tile_plan(c);
    const TilePlan &tp = c.tiles;
    const int N = c.nbNodes;
    const int dim = op == MFEM_OP_LAP ? 1 : 9;
    c.values.reserve(sizeof(float) * (size_t)c.nnz * dim);
    double *prec = fusePrec ? (double *)c.prec.reserve(sizeof(double) * (size_t)N * dim) : nullptr;
    float4 *hi = (float4 *)c.scratch.reserve(sizeof(float4) * 2 * (size_t)N);
    float4 *lo = hi + N;
    c.timer.begin("split_coords", c.stream);
    k_split_coords_t<<<blocks_for(N, 256), 256, 0, c.stream>>>(c.coord.as<double>(), N, hi, lo);
    check_launch("k_split_coords_t");
    c.timer.end(c.stream);
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st + 4, 0, sizeof(int) * 2, c.stream));
    const size_t smem = (size_t)tp.maxElem * 5 * sizeof(float4);
    const double *coef = c.coefOp == op ? c.coef.as<double>() : nullptr;
    const unsigned char *mask = c.hasMask ? c.mask.as<unsigned char>() : nullptr;
    const float q = c.sliverThreshold;
    c.timer.begin(fusePrec ? "tile32+prec" : "tile32", c.stream);
    auto launch = [&](auto kern) {
        MFEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<tp.nTiles, kTileThreads, smem, c.stream>>>(
            tp.desc.as<TileDesc>(), tp.rows.as<int>(), tp.elems.as<int>(), tp.offPos.as<int>(),
            tp.offMeta.as<unsigned>(), tp.diagMeta.as<unsigned>(), tp.contrib.as<unsigned short>(),
            hi, lo, c.coord.as<double>(), c.e2n.as<int4>(), coef, c.diagPos.as<int>(), mask, q * q,
            c.values.as<float>(), prec, st + 4);
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
