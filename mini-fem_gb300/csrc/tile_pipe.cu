// FP32 tile assembly, persistent and software-pipelined (fp32_kernel 2).
//
// The same tiles, plan and arithmetic as the one-CTA-per-tile kernel
// (tiles.cu, tile_body.cuh), reorganised so that a tile's inputs arrive while
// the previous tile computes.  In the one-CTA-per-tile form every tile starts
// with two dependent rounds of global loads (the tile's node and element ids,
// then the coordinates and weights they point at) before any arithmetic can
// begin, and that latency is paid tile after tile.  Here each CTA walks a
// strided list of tiles (blockIdx.x, + gridDim.x, ...) with two input buffers
// in shared memory:
//
//   top of tile i      one thread starts the TMA bulk copies of tile i+1's plan
//                      segments (contribution lists, diagonal and off-diagonal
//                      tables, element ids, connectivity, node ids) into the
//                      other buffer (completion on that buffer's mbarrier);
//   phase 1            the gradients of tile i (its coordinates and weights
//                      were gathered during tile i-1), the FP64 pass for
//                      flagged elements;
//   gathers of i+1     every thread waits (bounded) for tile i+1's segments and
//                      issues cp.async gathers of its node coordinates and
//                      element weights into the other buffer;
//   phases 3a, 3b, 2   tile i's diagonal rows, their FP64 block inversion and
//                      the off-diagonal entries, while those gathers fly.
//
// Results are bitwise those of the one-CTA-per-tile kernel: the same
// contribution order, the same arithmetic.
#include <algorithm>
#include <cstdint>

#include "context.h"
#include "elem32.cuh"
#include "tile_body.cuh"
#include "tiles.cuh"

namespace mfem {

namespace {

using namespace tilek;

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// Bounded wait on an mbarrier phase; the CTA agrees on the outcome.
__device__ __forceinline__ bool cta_wait(uint64_t *bar, unsigned parity, unsigned limit) {
    bool ok = false;
    for (unsigned it = 0; it < limit && !ok; it++) ok = mbar_try_wait(bar, parity);
    return !__syncthreads_or(!ok);
}

struct Buf {
    unsigned short *contrib;
    int2 *diag;
    int4 *off;
    int *elems;
    ushort4 *lconn;
    int *nodes;
    float4 *xh, *xl;
    float2 *w;
};

__device__ __forceinline__ Buf buffer(unsigned char *sm, const PipeLayout &L, int k) {
    unsigned char *b = sm + L.buf + k * L.bufBytes;
    Buf B;
    B.contrib = reinterpret_cast<unsigned short *>(b + L.contrib);
    B.diag = reinterpret_cast<int2 *>(b + L.diag);
    B.off = reinterpret_cast<int4 *>(b + L.off);
    B.elems = reinterpret_cast<int *>(b + L.elems);
    B.lconn = reinterpret_cast<ushort4 *>(b + L.lconn);
    B.nodes = reinterpret_cast<int *>(b + L.nodes);
    B.xh = reinterpret_cast<float4 *>(b + L.x);
    B.xl = B.xh + L.maxNodes;
    B.w = reinterpret_cast<float2 *>(b + L.w);
    return B;
}

__device__ __forceinline__ unsigned round4(int n) { return (unsigned)((n + 3) & ~3); }

// One thread: the TMA bulk copies of tile T's plan segments into buffer B (the
// plan starts every segment on a 16-byte boundary and pads it to whole 16-byte
// units that lie inside the arrays).
__device__ __forceinline__ void issue_segments(const TilePlanView &P, const TileDesc &T, const Buf &B,
                                               uint64_t *bar, unsigned extraTx) {
    const unsigned bc = (unsigned)T.nContribPad * 2u, bd = (unsigned)T.nRowsPad * 8u,
                   bo = (unsigned)T.nOffPad * 16u, be = round4(T.nElem) * 4u,
                   bl = round4(T.nElem) * 8u, bn = round4(T.nNodes) * 4u;
    // earlier generic-proxy reads of this buffer before the async-proxy writes
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, bc + bd + bo + be + bl + bn + extraTx);
    if (bc) bulk_g2s(B.contrib, P.contrib + T.contribBegin, bc, bar);
    if (bd) bulk_g2s(B.diag, P.diagEnt + T.diagBegin, bd, bar);
    if (bo) bulk_g2s(B.off, P.offEnt + T.offBegin, bo, bar);
    if (be) bulk_g2s(B.elems, P.elems + T.elemBegin, be, bar);
    if (bl) bulk_g2s(B.lconn, P.lconn + T.elemBegin, bl, bar);
    if (bn) bulk_g2s(B.nodes, P.nodes + T.nodeBegin, bn, bar);
}

// All threads: the coordinates (hi, lo) of the tile's nodes and the weights of
// its elements, gathered by cp.async from the ids already in buffer B.
__device__ __forceinline__ void issue_gathers(const TileDesc &T, const Buf &B, const TileMesh &M,
                                              const float2 *w) {
    for (int i = threadIdx.x; i < T.nNodes; i += kTileThreads) {
        const int n = B.nodes[i];
        cp_async16(B.xh + i, M.hl + 2 * (size_t)n);
        cp_async16(B.xl + i, M.hl + 2 * (size_t)n + 1);
    }
    for (int i = threadIdx.x; i < T.nElem; i += kTileThreads) cp_async8(B.w + i, w + B.elems[i]);
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int OP, bool PREC>
__global__ void __launch_bounds__(kTileThreads, 2)
k_tile32_pipe(TilePlanView P, TileMesh M, TileSets S, PipeLayout L, int nTiles, float qthr2,
              int *counters, TileCtl ctl) {
    extern __shared__ __align__(16) unsigned char sm[];
    float4 *G = reinterpret_cast<float4 *>(sm + L.g);
    float *sRes = reinterpret_cast<float *>(sm + L.res);
    unsigned short *sFlag = reinterpret_cast<unsigned short *>(sm + L.q);
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + L.bar);
    const int tid = threadIdx.x, lane = tid & 31;
    __shared__ int sNext, sFlagged;
    float *values = S.values;
    double *precOut = S.prec;

    int tile = blockIdx.x;
    if (tile >= nTiles) return;
    if (tid == 0) {
        mbar_init(bars, 1);
        mbar_init(bars + 1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        issue_segments(P, P.desc[tile], buffer(sm, L, 0), bars, ctl.extraTx);
    }
    __syncthreads();
    // the segment copy that a failed wait leaves pending: its barrier and phase
    uint64_t *failBar = bars;
    unsigned failParity = 0u;
    bool ok = cta_wait(bars, 0u, ctl.waitLimit);
    // prologue: the first tile's gathers
    if (ok) issue_gathers(P.desc[tile], buffer(sm, L, 0), M, S.w);

    for (int it = 0; ok; it++) {
        const TileDesc T = P.desc[tile];
        const int b = it & 1;
        const Buf B = buffer(sm, L, b), Bn = buffer(sm, L, b ^ 1);
        const int next = tile + gridDim.x;
        // the next tile's plan segments into the other buffer, free since the
        // end of the previous tile
        if (next < nTiles && tid == 0) issue_segments(P, P.desc[next], Bn, bars + (b ^ 1), ctl.extraTx);
        if (tid == 0) {
            sFlagged = 0;
            sNext = 0;
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();

        // 1. gradients of the tile's elements; flagged elements queued for FP64
        for (int i = tid; i < T.nElem; i += kTileThreads) {
            const ushort4 lc = B.lconn[i];
            ElemCoords C;
            C.h0 = B.xh[lc.x]; C.h1 = B.xh[lc.y]; C.h2 = B.xh[lc.z]; C.h3 = B.xh[lc.w];
            C.l0 = B.xl[lc.x]; C.l1 = B.xl[lc.y]; C.l2 = B.xl[lc.z]; C.l3 = B.xl[lc.w];
            float g[12];
            if (grad32_core(C, qthr2, g)) sFlag[atomicAdd(&sFlagged, 1)] = (unsigned short)i;
#pragma unroll
            for (int j = 0; j < 4; j++) G[gslot(i, j)] = make_float4(g[3 * j], g[3 * j + 1], g[3 * j + 2], 0.f);
        }
        __syncthreads();
        const int nFlagged = sFlagged;
        if (nFlagged) {
            for (int k = tid; k < nFlagged; k += kTileThreads) {
                const int i = sFlag[k];
                const ushort4 lc = B.lconn[i];
                float g[12];
                grad32_fp64(M.coord, make_int4(B.nodes[lc.x], B.nodes[lc.y], B.nodes[lc.z], B.nodes[lc.w]), g);
#pragma unroll
                for (int j = 0; j < 4; j++) G[gslot(i, j)] = make_float4(g[3 * j], g[3 * j + 1], g[3 * j + 2], 0.f);
            }
            if (tid == 0) atomicAdd(counters + 1, nFlagged);
            __syncthreads();
        }

        // the next tile's gathers (its segments have had phase 1 to arrive)
        if (next < nTiles) {
            const unsigned parity = (unsigned)((it + 1) >> 1) & 1u;
            if (!cta_wait(bars + (b ^ 1), parity, ctl.waitLimit)) {
                ok = false;
                failBar = bars + (b ^ 1);
                failParity = parity;
                break;
            }
            issue_gathers(P.desc[next], Bn, M, S.w);
        }

        // 3a. diagonal rows: four lanes per row, error-free merge (tile_body.cuh)
        const int diagThreads = min(kTileThreads, (T.nRows * 4 + 31) & ~31);
        if (tid < diagThreads) {
            const int part = tid & 3;
            for (int base = 0; base < T.nRows; base += diagThreads / 4) {
                const int rl = base + (tid >> 2);
                const bool active = rl < T.nRows;
                const int2 de = active ? B.diag[rl] : make_int2(0, 0);
                const int bq = (unsigned)de.y >> 8, n = de.y & 0xff;
                const bool writer = active && part == 0;
                const int p = writer ? M.diagPos[de.x] : -1;
                if (OP == MFEM_OP_LAP) {
                    Kahan acc;
                    for (int q = bq + part; q < bq + n; q += 4) {
                        const unsigned u = B.contrib[q];
                        const float4 g = G[slot_j(u)];
                        acc.add(B.w[u >> 4].x * fmaf(g.x, g.x, fmaf(g.y, g.y, g.z * g.z)));
                    }
                    quad_combine(acc);
                    if (writer) {
                        if (p >= 0) values[p] = acc.value();
                        if (PREC) {
                            sRes[kResStride * rl] = acc.s;
                            sRes[kResStride * rl + 1] = acc.c;
                        }
                    }
                } else {
                    Kahan acc[6];
                    for (int q = bq + part; q < bq + n; q += 4) {
                        const unsigned u = B.contrib[q];
                        const float2 w = B.w[u >> 4];
                        ela_diag_accumulate(acc, G[slot_j(u)], w.x, w.y);
                    }
#pragma unroll
                    for (int m = 0; m < 6; m++) quad_combine(acc[m]);
                    if (writer) {
                        float sv[6];
#pragma unroll
                        for (int m = 0; m < 6; m++) sv[m] = acc[m].value();
                        if (p >= 0) {
                            const float v[9] = {sv[0], sv[3], sv[4], sv[3], sv[1], sv[5], sv[4], sv[5], sv[2]};
                            store_block9(values, (size_t)p, v);
                        }
                        if (PREC) {
#pragma unroll
                            for (int m = 0; m < 6; m++) {
                                sRes[kResStride * rl + 2 * m] = acc[m].s;
                                sRes[kResStride * rl + 2 * m + 1] = acc[m].c;
                            }
                            sRes[kResStride * rl + 12] = __int_as_float(p);
                        }
                    }
                }
            }
            asm volatile("bar.sync 1, %0;" ::"r"(diagThreads) : "memory");
            if (PREC) {
                // 3b. FP64 preconditioner blocks from the compensated sums
                for (int rl = tid; rl < T.nRows; rl += diagThreads) {
                    const int r = B.diag[rl].x;
                    const float *res = sRes + kResStride * rl;
                    if (OP == MFEM_OP_LAP) {
                        precOut[r] = rcp64(f32_to_f64(res[0]) - f32_to_f64(res[1]));
                    } else {
                        double d[6];
#pragma unroll
                        for (int m = 0; m < 6; m++) d[m] = f32_to_f64(res[2 * m]) - f32_to_f64(res[2 * m + 1]);
                        if (M.mask) {
                            // src/Fortran/elasclpr.f:19-27
                            const unsigned mk = M.mask[r];
                            if (mk & 1u) { d[0] = 1.0; d[3] = 0.0; d[4] = 0.0; }
                            if (mk & 2u) { d[1] = 1.0; d[3] = 0.0; d[5] = 0.0; }
                            if (mk & 4u) { d[2] = 1.0; d[4] = 0.0; d[5] = 0.0; }
                        }
                        if (__float_as_int(res[12]) >= 0 && !inv3_sym(d)) atomicAdd(counters, 1);
                        const double o[9] = {d[0], d[3], d[4], d[3], d[1], d[5], d[4], d[5], d[2]};
                        store_block9(precOut, (size_t)r, o);
                    }
                }
            }
        }

        // 2. off-diagonal units, 32 at a time from a shared counter
        for (;;) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&sNext, 32);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= T.nOff) break;
            const int t = base + lane;
            if (t >= T.nOff) continue;
            const int4 ent = B.off[t];
            const int bq = (unsigned)ent.z >> 8, n = ent.z & 0xff;
            if (OP == MFEM_OP_LAP) {
                Kahan acc;
                for (int q = bq; q < bq + n; q++) {
                    const unsigned u = B.contrib[q];
                    const float4 gj = G[slot_j(u)], gk = G[slot_k(u)];
                    const float x = B.w[u >> 4].x * fmaf(gj.x, gk.x, fmaf(gj.y, gk.y, gj.z * gk.z));
                    if (q == bq) { acc.s = x; acc.c = 0.f; } else acc.add(x);
                }
                const float v = acc.value();
                values[ent.x] = v;
                if (ent.y >= 0) values[ent.y] = v;
            } else {
                Kahan acc[9];
                int q = bq;
                for (; q + 1 < bq + n; q += 2) {
                    const unsigned u0 = B.contrib[q], u1 = B.contrib[q + 1];
                    const float4 gj0 = G[slot_j(u0)], gk0 = G[slot_k(u0)];
                    const float4 gj1 = G[slot_j(u1)], gk1 = G[slot_k(u1)];
                    const float2 w0 = B.w[u0 >> 4], w1 = B.w[u1 >> 4];
                    ela_accumulate(acc, gj0, gk0, w0.x, w0.y, q == bq);
                    ela_accumulate(acc, gj1, gk1, w1.x, w1.y, false);
                }
                if (q < bq + n) {
                    const unsigned u = B.contrib[q];
                    const float2 w = B.w[u >> 4];
                    ela_accumulate(acc, G[slot_j(u)], G[slot_k(u)], w.x, w.y, q == bq);
                }
                float v[9];
#pragma unroll
                for (int m = 0; m < 9; m++) v[m] = n ? acc[m].value() : 0.f;
                store_block9(values, (size_t)ent.x, v);
                if (ent.y >= 0) {
                    const float tr[9] = {v[0], v[3], v[6], v[1], v[4], v[7], v[2], v[5], v[8]};
                    store_block9(values, (size_t)ent.y, tr);
                }
            }
        }
        __syncthreads();   // G, sRes and this buffer are free for the next tiles
        if (next >= nTiles) break;
        tile = next;
    }
    if (!ok) {
        // a staged copy did not arrive in time: flag, let the copy in flight
        // land (bounded), and stop
        if (tid == 0) {
            atomicOr(counters + 2, 1);
            for (unsigned w = 0; w < ctl.waitLimit && !mbar_try_wait(failBar, failParity); w++) {
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        return;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (tid == 0) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bars)) : "memory");
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bars + 1)) : "memory");
    }
}

int round_up16(int x) { return (x + 15) / 16 * 16; }

}  // namespace

PipeLayout pipe_layout(int maxElem, int maxContribPad, int maxOffPad, int maxRowsPad, int maxNodes) {
    PipeLayout L{};
    const int me = (maxElem + 3) & ~3, mn = (maxNodes + 3) & ~3;
    L.maxNodes = mn;
    L.g = 0;
    L.res = L.g + me * 64;
    L.q = L.res + round_up16(maxRowsPad * 4 * kResStride);
    L.bar = L.q + round_up16(me * 2);
    L.buf = L.bar + 16;
    int o = 0;
    L.contrib = o; o += round_up16(maxContribPad * 2);
    L.diag = o;    o += round_up16(maxRowsPad * 8);
    L.off = o;     o += maxOffPad * 16;
    L.elems = o;   o += me * 4;
    L.lconn = o;   o += me * 8;
    L.nodes = o;   o += mn * 4;
    L.x = o;       o += mn * 32;
    L.w = o;       o += me * 8;
    L.bufBytes = round_up16(o);
    L.bytes = L.buf + 2 * L.bufBytes;
    return L;
}

void assemble_tiles32_pipe(Context &c, int op, bool fusePrec) {
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
    const PipeLayout L = pipe_layout(tp.planMax[0], tp.planMax[1], tp.planMax[2], tp.planMax[3],
                                     tp.planMax[4]);
    MFEM_REQUIRE(L.bytes <= 227 * 1024, MFEM_ERR_CAPACITY,
                 "pipelined tiles need more than 227 KB of shared memory");
    const float q = c.sliverThreshold;
    int sms = 0;
    MFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    c.timer.begin(fusePrec ? "tile32+prec" : "tile32", c.stream);
    auto launch = [&](auto kern) {
        MFEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes));
        int perSM = 0;
        MFEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, kTileThreads, L.bytes));
        const int grid = std::max(1, std::min(tp.nTiles, sms * std::max(perSM, 1)));
        kern<<<grid, kTileThreads, L.bytes, c.stream>>>(P, M, S, L, tp.nTiles, q * q, st + 4,
                                                        TileCtl{c.waitLimit, c.testExtraTx});
    };
    if (op == MFEM_OP_LAP) {
        if (fusePrec) launch(k_tile32_pipe<MFEM_OP_LAP, true>);
        else launch(k_tile32_pipe<MFEM_OP_LAP, false>);
    } else {
        if (fusePrec) launch(k_tile32_pipe<MFEM_OP_ELA, true>);
        else launch(k_tile32_pipe<MFEM_OP_ELA, false>);
    }
    check_launch("k_tile32_pipe");
    c.timer.end(c.stream);
    c.flaggedPending = true;
    c.lastOp = op;
    c.lastPrecision = MFEM_FP32;
    c.precIsInit = fusePrec;
}

}  // namespace mfem
