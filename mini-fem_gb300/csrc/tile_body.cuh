// Device body of the FP32 tile kernel, shared by the single-mesh launch
// (tiles.cu) and the persistent cross-mesh launch (batch.cu).  See tiles.cu for
// the phases.
#pragma once

#include <cstdint>

#include "elem32.cuh"
#include "grad_df.cuh"
#include "tiles.cuh"

namespace mfem {
namespace tilek {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// 1D TMA bulk copy global -> shared; 16-byte aligned addresses, size % 16 == 0.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// A node's split coordinates (hi float4, lo float4: one 32-byte sector, 32-byte
// aligned, read-only in this kernel) by one 256-bit load.
__device__ __forceinline__ void ld_node_hl(const float4 *p, float4 &h, float4 &l) {
    double a, b, c, d;
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(a), "=d"(b), "=d"(c), "=d"(d) : "l"(p));
    h = make_float4(__int_as_float(__double2loint(a)), __int_as_float(__double2hiint(a)),
                    __int_as_float(__double2loint(b)), __int_as_float(__double2hiint(b)));
    l = make_float4(__int_as_float(__double2loint(c)), __int_as_float(__double2hiint(c)),
                    __int_as_float(__double2loint(d)), __int_as_float(__double2hiint(d)));
}

// 8-byte asynchronous global -> shared copy (both addresses 8-byte aligned)
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// Slot of gradient j of tile element l in the gradient array (four 16-byte
// slots per element, rotated by l / 2): the eight lanes of a quarter warp that
// store gradient j of eight consecutive elements hit eight distinct bank
// groups instead of two.
__device__ __forceinline__ int gslot(int l, int j) { return 4 * l + ((j + (l >> 1)) & 3); }

// The gradient slots a contribution code (local element << 4 | rotated slot of
// node j << 2 | rotated slot of node k, made by the plan) refers to.
__device__ __forceinline__ int slot_j(unsigned u) { return (int)(u >> 2); }
__device__ __forceinline__ int slot_k(unsigned u) { return (int)(((u >> 2) & ~3u) | (u & 3u)); }

// error-free sum of two Kahan partials (value = s - c)
__device__ __forceinline__ void kahan_merge(Kahan &a, float s2, float c2) {
    const float s = a.s + s2;
    const float bb = s - a.s;
    const float err = (a.s - (s - bb)) + (s2 - bb);
    a.c = (a.c + c2) - err;
    a.s = s;
}

__device__ __forceinline__ void quad_combine(Kahan &k) {
#pragma unroll
    for (int off = 1; off <= 2; off <<= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, k.s, off);
        const float c2 = __shfl_xor_sync(0xffffffffu, k.c, off);
        kahan_merge(k, s2, c2);
    }
}

// One elasticity contribution (j, k) in the FP32 form
//   c(a,b) = B gj_a gk_b + delta_ab mu (gj . gk)
// which is the reference's ((p_aa A + p_bb mu) + p_cc mu), p_ab B with
// A = B + mu, regrouped.  `first` assigns instead of accumulating (exact).
__device__ __forceinline__ void ela_accumulate(Kahan *acc, float4 gj, float4 gk, float B, float mu,
                                               bool first) {
    const float bx = gk.x * B, by = gk.y * B, bz = gk.z * B;
    const float md = mu * fmaf(gj.x, gk.x, fmaf(gj.y, gk.y, gj.z * gk.z));
    const float c[9] = {fmaf(gj.x, bx, md), gj.x * by, gj.x * bz,
                        gj.y * bx, fmaf(gj.y, by, md), gj.y * bz,
                        gj.z * bx, gj.z * by, fmaf(gj.z, bz, md)};
    if (first) {
#pragma unroll
        for (int m = 0; m < 9; m++) { acc[m].s = c[m]; acc[m].c = 0.f; }
    } else {
#pragma unroll
        for (int m = 0; m < 9; m++) acc[m].add(c[m]);
    }
}

// Two elasticity contributions (j0, k0), (j1, k1) added to the block as one
// term per entry: the pair's sum is formed by an FMA on the first
// contribution's value (one rounding at the pair's magnitude where the single
// form rounds each product), then added with compensation, so that the pair
// costs one compensated addition per entry instead of two.
__device__ __forceinline__ void ela_accumulate2(Kahan *acc, float4 gj0, float4 gk0, float2 w0,
                                                float4 gj1, float4 gk1, float2 w1, bool first) {
    const float bx0 = gk0.x * w0.x, by0 = gk0.y * w0.x, bz0 = gk0.z * w0.x;
    const float bx1 = gk1.x * w1.x, by1 = gk1.y * w1.x, bz1 = gk1.z * w1.x;
    const float md0 = w0.y * fmaf(gj0.x, gk0.x, fmaf(gj0.y, gk0.y, gj0.z * gk0.z));
    const float md = fmaf(w1.y, fmaf(gj1.x, gk1.x, fmaf(gj1.y, gk1.y, gj1.z * gk1.z)), md0);
    const float c[9] = {fmaf(gj1.x, bx1, fmaf(gj0.x, bx0, md)), fmaf(gj1.x, by1, gj0.x * by0),
                        fmaf(gj1.x, bz1, gj0.x * bz0),
                        fmaf(gj1.y, bx1, gj0.y * bx0), fmaf(gj1.y, by1, fmaf(gj0.y, by0, md)),
                        fmaf(gj1.y, bz1, gj0.y * bz0),
                        fmaf(gj1.z, bx1, gj0.z * bx0), fmaf(gj1.z, by1, gj0.z * by0),
                        fmaf(gj1.z, bz1, fmaf(gj0.z, bz0, md))};
    if (first) {
#pragma unroll
        for (int m = 0; m < 9; m++) { acc[m].s = c[m]; acc[m].c = 0.f; }
    } else {
#pragma unroll
        for (int m = 0; m < 9; m++) acc[m].add(c[m]);
    }
}

// One 3x3 FP32 block to base[9p .. 9p+8] with three or four 16-, 8- and
// 4-byte stores chosen by the block's address modulo 16, instead of nine 4-byte
// stores: fewer memory transactions per block.  The stores are streaming
// (st.global.cs, evict first): the values are written once, and the L2 keeps
// the coordinates and weights that neighbouring tiles gather again (0.608 ->
// 0.592 ms at 100^3).
__device__ __forceinline__ void store_block9(float *base, size_t p, const float v[9]) {
    float *o = base + p * 9;
    const unsigned mis = (unsigned)(reinterpret_cast<uintptr_t>(o) >> 2) & 3u;
    if (mis == 0u) {
        __stcs(reinterpret_cast<float4 *>(o), make_float4(v[0], v[1], v[2], v[3]));
        __stcs(reinterpret_cast<float4 *>(o + 4), make_float4(v[4], v[5], v[6], v[7]));
        __stcs(o + 8, v[8]);
    } else if (mis == 1u) {
        __stcs(o + 0, v[0]);
        __stcs(reinterpret_cast<float2 *>(o + 1), make_float2(v[1], v[2]));
        __stcs(reinterpret_cast<float4 *>(o + 3), make_float4(v[3], v[4], v[5], v[6]));
        __stcs(reinterpret_cast<float2 *>(o + 7), make_float2(v[7], v[8]));
    } else if (mis == 2u) {
        __stcs(reinterpret_cast<float2 *>(o), make_float2(v[0], v[1]));
        __stcs(reinterpret_cast<float4 *>(o + 2), make_float4(v[2], v[3], v[4], v[5]));
        __stcs(reinterpret_cast<float2 *>(o + 6), make_float2(v[6], v[7]));
        __stcs(o + 8, v[8]);
    } else {
        __stcs(o + 0, v[0]);
        __stcs(reinterpret_cast<float4 *>(o + 1), make_float4(v[1], v[2], v[3], v[4]));
        __stcs(reinterpret_cast<float4 *>(o + 5), make_float4(v[5], v[6], v[7], v[8]));
    }
}

// The same for a 3x3 FP64 block (72 bytes, 8-byte aligned): four 16-byte
// stores and one 8-byte store, streaming.
__device__ __forceinline__ void store_block9(double *base, size_t p, const double v[9]) {
    double *o = base + p * 9;
    if (reinterpret_cast<uintptr_t>(o) & 15u) {
        __stcs(o + 0, v[0]);
        __stcs(reinterpret_cast<double2 *>(o + 1), make_double2(v[1], v[2]));
        __stcs(reinterpret_cast<double2 *>(o + 3), make_double2(v[3], v[4]));
        __stcs(reinterpret_cast<double2 *>(o + 5), make_double2(v[5], v[6]));
        __stcs(reinterpret_cast<double2 *>(o + 7), make_double2(v[7], v[8]));
    } else {
        __stcs(reinterpret_cast<double2 *>(o), make_double2(v[0], v[1]));
        __stcs(reinterpret_cast<double2 *>(o + 2), make_double2(v[2], v[3]));
        __stcs(reinterpret_cast<double2 *>(o + 4), make_double2(v[4], v[5]));
        __stcs(reinterpret_cast<double2 *>(o + 6), make_double2(v[6], v[7]));
        __stcs(o + 8, v[8]);
    }
}

// Symmetric diagonal block (j, j): six distinct values d00, d11, d22, d01, d02, d12.
__device__ __forceinline__ void ela_diag_accumulate(Kahan *acc, float4 g, float B, float mu) {
    const float bx = g.x * B, by = g.y * B, bz = g.z * B;
    const float md = mu * fmaf(g.x, g.x, fmaf(g.y, g.y, g.z * g.z));
    acc[0].add(fmaf(g.x, bx, md));
    acc[1].add(fmaf(g.y, by, md));
    acc[2].add(fmaf(g.z, bz, md));
    acc[3].add(g.x * by);
    acc[4].add(g.x * bz);
    acc[5].add(g.y * bz);
}

// Two contributions to a diagonal block as one term per entry (as
// ela_accumulate2).
__device__ __forceinline__ void ela_diag_accumulate2(Kahan *acc, float4 g0, float2 w0, float4 g1,
                                                     float2 w1) {
    const float bx0 = g0.x * w0.x, by0 = g0.y * w0.x, bz0 = g0.z * w0.x;
    const float bx1 = g1.x * w1.x, by1 = g1.y * w1.x, bz1 = g1.z * w1.x;
    const float md0 = w0.y * fmaf(g0.x, g0.x, fmaf(g0.y, g0.y, g0.z * g0.z));
    const float md = fmaf(w1.y, fmaf(g1.x, g1.x, fmaf(g1.y, g1.y, g1.z * g1.z)), md0);
    acc[0].add(fmaf(g1.x, bx1, fmaf(g0.x, bx0, md)));
    acc[1].add(fmaf(g1.y, by1, fmaf(g0.y, by0, md)));
    acc[2].add(fmaf(g1.z, bz1, fmaf(g0.z, bz0, md)));
    acc[3].add(fmaf(g1.x, by1, g0.x * by0));
    acc[4].add(fmaf(g1.x, bz1, g0.x * bz0));
    acc[5].add(fmaf(g1.y, bz1, g0.y * bz0));
}

// 1 / x in FP64: the FP32 reciprocal of x (relative error below 2^-23) refined by
// two Newton-Raphson steps r <- r + r (1 - x r), each squaring the relative
// error (2^-46, then below the FP64 rounding): within an ulp or so of the
// correctly rounded reciprocal, in four FMAs instead of a division.  Values
// whose FP32 form is not a normal float with a normal reciprocal take the
// division.
__device__ __forceinline__ double rcp64(double x) {
    const double ax = fabs(x);
    if (!(ax > 0x1.0p-120 && ax < 0x1.0p120)) return 1.0 / x;
    double r = f32_to_f64(1.0f / f64_to_f32(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// Inverse of a symmetric 3x3 block in FP64 by its six distinct cofactors;
// d = (d00, d11, d22, d01, d02, d12).  The block is first scaled by the power
// of two 2^-k that brings its largest diagonal entry near 1 (exact, on the
// integer pipe) so that the determinant's reciprocal can start from FP32; the
// inverse of the scaled block times 2^-k is the inverse.  Returns false for an
// exactly singular block, which is then left as it is.
__device__ __forceinline__ bool inv3_sym(double d[6]) {
    const double mx = fmax(fabs(d[0]), fmax(fabs(d[1]), fabs(d[2])));
    if (!(mx > 0.0) || !(mx < INFINITY)) return false;   // zero, NaN or infinite diagonal
    const int k = (int)((__double_as_longlong(mx) >> 52) & 0x7ff) - 1023;
    const double a = scale_pow2(d[0], -k), e = scale_pow2(d[1], -k), i = scale_pow2(d[2], -k),
                 b = scale_pow2(d[3], -k), c = scale_pow2(d[4], -k), f = scale_pow2(d[5], -k);
    const double c00 = fma(e, i, -f * f);
    const double c01 = fma(c, f, -b * i);
    const double c02 = fma(b, f, -c * e);
    const double det = fma(a, c00, fma(b, c01, c * c02));
    if (det == 0.0) return false;
    const double r = rcp64(det);
    const double c11 = fma(a, i, -c * c);
    const double c12 = fma(b, c, -a * f);
    const double c22 = fma(a, e, -b * b);
    d[0] = scale_pow2(c00 * r, -k); d[1] = scale_pow2(c11 * r, -k); d[2] = scale_pow2(c22 * r, -k);
    d[3] = scale_pow2(c01 * r, -k); d[4] = scale_pow2(c02 * r, -k); d[5] = scale_pow2(c12 * r, -k);
    return true;
}

// One tile for nSets coefficient sets: the gradients are computed once, the
// weights, entries and preconditioner blocks once per set.  Returns false when
// the staged plan segments did not arrive within the bounded wait (error flag
// counters[2] set; the caller stops).
template <int OP, bool PREC>
__device__ __forceinline__ bool tile_body(const TileDesc &T, const TileMesh &M, const TileSets &S,
                                          const TilePlanView &P, const SmemLayout &L, float qthr2,
                                          unsigned char *sm, int *counters, TileCtl ctl) {
    float4 *G = reinterpret_cast<float4 *>(sm);                       // 4 per element
    float2 *W = reinterpret_cast<float2 *>(sm + L.w);                 // (B, mu) or (kappa, -)
    float *sRes = reinterpret_cast<float *>(sm + L.res);              // kResStride floats per row
    unsigned short *sC = reinterpret_cast<unsigned short *>(sm + L.contrib);
    int4 *sOff = reinterpret_cast<int4 *>(sm + L.off);
    int4 *sDiag = reinterpret_cast<int4 *>(sm + L.diag);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + L.bar);           // two barriers
    const int tid = threadIdx.x, lane = tid & 31;
    __shared__ int sNext;      // next off-diagonal unit of phase 2
    __shared__ int sFlagged;   // elements of phase 1b queued for the FP64 gradients
    if (tid == 0) sFlagged = 0;

    // 0. stage the contribution lists and the diagonal table with the TMA
    //    engine (barrier 0)
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        // make the initialised barriers visible to the TMA (async) proxy
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned bc = (unsigned)T.nContribPad * 2u, bd = (unsigned)T.nRowsPad * 16u;
        mbar_expect_tx(bar, bc + bd + ctl.extraTx);
        if (bc) bulk_g2s(sC, P.contrib + T.contribBegin, bc, bar);
        if (bd) bulk_g2s(sDiag, P.diagEnt + T.diagBegin, bd, bar);
    }

    // 1a. the weights of set 0 go to shared memory by asynchronous copies
    //     (cp.async, no register round trip); the connectivity of a thread's
    //     first two elements is loaded into registers; meanwhile the tile's node
    //     coordinates (hi parts, then lo parts) are gathered into the region
    //     that the off-diagonal table fills after phase 1
    const int i0 = tid, i1 = tid + kTileThreads;
    ushort4 lc0 = make_ushort4(0, 0, 0, 0), lc1 = lc0;
    if (i0 < T.nElem) {
        lc0 = P.lconn[T.elemBegin + i0];
        cp_async8(W + i0, S.w + P.elems[T.elemBegin + i0]);
    }
    if (i1 < T.nElem) {
        lc1 = P.lconn[T.elemBegin + i1];
        cp_async8(W + i1, S.w + P.elems[T.elemBegin + i1]);
    }
    for (int i = i1 + kTileThreads; i < T.nElem; i += kTileThreads)
        cp_async8(W + i, S.w + P.elems[T.elemBegin + i]);
    float4 *Xh = reinterpret_cast<float4 *>(sm + L.x);
    float4 *Xl = Xh + T.nNodes;
    for (int i = tid; i < T.nNodes; i += kTileThreads) {
        const int n = P.nodes[T.nodeBegin + i];
        float4 h, l;
        ld_node_hl(M.hl + 2 * n, h, l);
        Xh[i] = h;
        Xl[i] = l;
    }
    cp_async_wait_all();
    __syncthreads();

    // 1b. gradients of the tile's elements; flagged elements are queued (after
    //     the coordinates) and get their double-float gradients (grad_df.cuh)
    //     in a second pass by consecutive threads, so that the extra work is
    //     spread over full warps instead of stalling every warp that holds one
    //     flagged element
    unsigned short *sFlag = reinterpret_cast<unsigned short *>(sm + L.q);
    for (int i = tid; i < T.nElem; i += kTileThreads) {
        const ushort4 lc = i == i0 ? lc0 : i == i1 ? lc1 : P.lconn[T.elemBegin + i];
        ElemCoords C;
        C.h0 = Xh[lc.x]; C.h1 = Xh[lc.y]; C.h2 = Xh[lc.z]; C.h3 = Xh[lc.w];
        C.l0 = Xl[lc.x]; C.l1 = Xl[lc.y]; C.l2 = Xl[lc.z]; C.l3 = Xl[lc.w];
        float g[12];
        // a flagged element's slots are overwritten by the second pass
        if (grad32_core(C, qthr2, g)) sFlag[atomicAdd(&sFlagged, 1)] = (unsigned short)i;
#pragma unroll
        for (int j = 0; j < 4; j++) G[gslot(i, j)] = make_float4(g[3 * j], g[3 * j + 1], g[3 * j + 2], 0.f);
    }
    __syncthreads();
    const int nFlagged = sFlagged;
    if (nFlagged) {
        const int *nb = P.nodes + T.nodeBegin;
        for (int k = tid; k < nFlagged; k += kTileThreads) {
            const int i = sFlag[k];
            const ushort4 lc = P.lconn[T.elemBegin + i];
            const unsigned short ln[4] = {lc.x, lc.y, lc.z, lc.w};
            float hi[4][3], lo[4][3], g[12];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float4 h = Xh[ln[j]], l = Xl[ln[j]];
                hi[j][0] = h.x; hi[j][1] = h.y; hi[j][2] = h.z;
                lo[j][0] = l.x; lo[j][1] = l.y; lo[j][2] = l.z;
            }
            // double-float from the staged coordinates; a zero volume takes the
            // FP64 formula and its infinities
            if (!grad_df(hi, lo, g))
                grad32_fp64(M.coord, make_int4(nb[lc.x], nb[lc.y], nb[lc.z], nb[lc.w]), g);
#pragma unroll
            for (int j = 0; j < 4; j++) G[gslot(i, j)] = make_float4(g[3 * j], g[3 * j + 1], g[3 * j + 2], 0.f);
        }
        if (tid == 0) atomicAdd(counters + 1, nFlagged);
        __syncthreads();
    }

    // the off-diagonal table (barrier 1), over the node coordinates: the
    // generic-proxy reads above are ordered before the async-proxy writes.
    // Only phase 2 reads it; each warp waits for it just before its phase 2.
    if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned bo = (unsigned)T.nOffPad * 16u;
        mbar_expect_tx(bar + 1, bo);
        if (bo) bulk_g2s(sOff, P.offEnt + T.offBegin, bo, bar + 1);
    }
    // bounded wait for the contribution lists and the diagonal table (the CTA
    // agrees on the outcome)
    if (tid == 0) sNext = 0;   // phase 2's unit counter, set 0
    bool ok = false;
    for (unsigned it = 0; it < ctl.waitLimit && !ok; it++) ok = mbar_try_wait(bar, 0);
    if (__syncthreads_or(!ok)) {
        if (tid == 0) {
            atomicOr(counters + 2, 1);
            // let the off-diagonal copy land (bounded) before the CTA exits
            for (unsigned it = 0; it < ctl.waitLimit && !mbar_try_wait(bar + 1, 0); it++) {
            }
        }
        return false;
    }
    bool offMissing = false;   // this warp gave up waiting for the off-diagonal table

    for (int set = 0; set < S.nSets; set++) {
        float *values = S.values + (size_t)set * S.valuesStride;
        double *precOut = S.prec ? S.prec + (size_t)set * S.precStride : nullptr;
        if (set > 0) {
            // weights of this set (every thread is done with the previous set's)
            __syncthreads();
            const float2 *w = S.w + (size_t)set * S.wStride;
            for (int i = tid; i < T.nElem; i += kTileThreads) W[i] = w[P.elems[T.elemBegin + i]];
            if (tid == 0) sNext = 0;
            __syncthreads();
        }

        // 3a. diagonal entries: four lanes per row sum a quarter of the row's
        //     contributions each and combine them without error; the first lane
        //     writes the block and keeps the compensated sums for 3b.  Only the
        //     warps these lanes need take part; the others go straight to phase
        //     2, which does not depend on 3a.
        const int diagThreads = min(kTileThreads, (T.nRows * 4 + 31) & ~31);
        if (tid < diagThreads) {
        const int part = tid & 3;
        for (int base = 0; base < T.nRows; base += diagThreads / 4) {
            const int rl = base + (tid >> 2);
            const bool active = rl < T.nRows;
            const int4 de = active ? sDiag[rl] : make_int4(0, 0, -1, 0);
            const int b = (unsigned)de.y >> 8, n = de.y & 0xff;
            const bool writer = active && part == 0;
            const int p = writer ? de.z : -1;
            if (OP == MFEM_OP_LAP) {
                Kahan acc;
                for (int q = b + part; q < b + n; q += 4) {
                    const unsigned u = sC[q];
                    const int l = u >> 4;
                    const float4 g = G[slot_j(u)];
                    acc.add(W[l].x * fmaf(g.x, g.x, fmaf(g.y, g.y, g.z * g.z)));
                }
                quad_combine(acc);
                if (writer) {
                    if (p >= 0) __stcs(values + p, acc.value());
                    if (PREC) {
                        sRes[kResStride * rl] = acc.s;
                        sRes[kResStride * rl + 1] = acc.c;
                    }
                }
            } else {
                Kahan acc[6];
                // this lane's contributions two at a time, each pair one term
                int q = b + part;
                for (; q + 4 < b + n; q += 8) {
                    const unsigned u0 = sC[q], u1 = sC[q + 4];
                    ela_diag_accumulate2(acc, G[slot_j(u0)], W[u0 >> 4], G[slot_j(u1)], W[u1 >> 4]);
                }
                if (q < b + n) {
                    const unsigned u = sC[q];
                    const float2 w = W[u >> 4];
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
        // the row sums of 3a are ready for the diagonal warps (named barrier 1)
        asm volatile("bar.sync 1, %0;" ::"r"(diagThreads) : "memory");
        if (PREC) {
            // 3b. one thread per row (full warps on the FP64 pipe): the FP64
            //     preconditioner block from the compensated sums, while the
            //     other warps work on phase 2
            for (int rl = tid; rl < T.nRows; rl += diagThreads) {
                const int r = sDiag[rl].x;
                const float *res = sRes + kResStride * rl;
                if (OP == MFEM_OP_LAP) {
                    __stcs(precOut + r, rcp64(f32_to_f64(res[0]) - f32_to_f64(res[1])));
                } else {
                    double d[6];
#pragma unroll
                    for (int m = 0; m < 6; m++) d[m] = f32_to_f64(res[2 * m]) - f32_to_f64(res[2 * m + 1]);
                    if (M.mask) {
                        // src/Fortran/elasclpr.f:19-27: constrained DOF k -> row and
                        // column k of the block zero, diagonal 1
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
        }   // diagonal warps

        // 2. off-diagonal units: entry (r, c) and, when c is a row of this tile,
        //    its transpose (c, r), which is the same sum transposed; warps take
        //    32 units at a time from a shared counter, so that the warps of 3a
        //    and 3b join when their work is done.  First a bounded wait (warp-
        //    uniform outcome) for the off-diagonal table.
        if (set == 0) {
            bool got = false;
            for (unsigned it = 0; it < ctl.waitLimit && !got; it++) got = mbar_try_wait(bar + 1, 0);
            offMissing = !__all_sync(0xffffffffu, got);
        }
        for (; !offMissing;) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&sNext, 32);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= T.nOff) break;
            const int t = base + lane;
            if (t >= T.nOff) continue;
            const int4 ent = sOff[t];
            const int b = (unsigned)ent.z >> 8, n = ent.z & 0xff;
            if (OP == MFEM_OP_LAP) {
                Kahan acc;
                for (int q = b; q < b + n; q++) {
                    const unsigned u = sC[q];
                    const int l = u >> 4;
                    const float4 gj = G[slot_j(u)], gk = G[slot_k(u)];
                    const float x = W[l].x * fmaf(gj.x, gk.x, fmaf(gj.y, gk.y, gj.z * gk.z));
                    if (q == b) { acc.s = x; acc.c = 0.f; } else acc.add(x);
                }
                const float v = acc.value();
                __stcs(values + ent.x, v);   // written once: evict first, as store_block9
                if (ent.y >= 0) __stcs(values + ent.y, v);
            } else {
                Kahan acc[9];
                // two contributions per pass, summed as one term (their
                // shared-memory loads are in flight together)
                int q = b;
                for (; q + 1 < b + n; q += 2) {
                    const unsigned u0 = sC[q], u1 = sC[q + 1];
                    const float4 gj0 = G[slot_j(u0)], gk0 = G[slot_k(u0)];
                    const float4 gj1 = G[slot_j(u1)], gk1 = G[slot_k(u1)];
                    const float2 w0 = W[u0 >> 4], w1 = W[u1 >> 4];
                    ela_accumulate2(acc, gj0, gk0, w0, gj1, gk1, w1, q == b);
                }
                if (q < b + n) {
                    const unsigned u = sC[q];
                    const float4 gj = G[slot_j(u)], gk = G[slot_k(u)];
                    const float2 w = W[u >> 4];
                    ela_accumulate(acc, gj, gk, w.x, w.y, q == b);
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
    }
    if (__syncthreads_or(offMissing)) {
        if (tid == 0) atomicOr(counters + 2, 1);
        return false;
    }
    if (tid == 0) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar + 1)) : "memory");
    }
    return true;
}

}  // namespace tilek
}  // namespace mfem
