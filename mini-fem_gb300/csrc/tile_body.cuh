// Device body of the FP32 tile kernel, shared by the single-mesh launch
// (tiles.cu) and the persistent cross-mesh launch (batch.cu).  See tiles.cu for
// the phases.
#pragma once

#include <cstdint>

#include "elem32.cuh"
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

// float -> double is exact; done with integer operations so that it does not
// occupy GB300's narrow FP64 pipe (zero and subnormal inputs take the
// conversion instruction).
__device__ __forceinline__ double f32_to_f64(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    const unsigned lo = b << 29;
    return __hiloint2double((int)hi, (int)lo);
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

// One 3x3 FP32 block to base[9p .. 9p+8] with three or four 16-, 8- and
// 4-byte stores chosen by the block's address modulo 16, instead of nine 4-byte
// stores: fewer memory transactions per block.
__device__ __forceinline__ void store_block9(float *base, size_t p, const float v[9]) {
    float *o = base + p * 9;
    const unsigned mis = (unsigned)(reinterpret_cast<uintptr_t>(o) >> 2) & 3u;
    if (mis == 0u) {
        *reinterpret_cast<float4 *>(o) = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4 *>(o + 4) = make_float4(v[4], v[5], v[6], v[7]);
        o[8] = v[8];
    } else if (mis == 1u) {
        o[0] = v[0];
        *reinterpret_cast<float2 *>(o + 1) = make_float2(v[1], v[2]);
        *reinterpret_cast<float4 *>(o + 3) = make_float4(v[3], v[4], v[5], v[6]);
        *reinterpret_cast<float2 *>(o + 7) = make_float2(v[7], v[8]);
    } else if (mis == 2u) {
        *reinterpret_cast<float2 *>(o) = make_float2(v[0], v[1]);
        *reinterpret_cast<float4 *>(o + 2) = make_float4(v[2], v[3], v[4], v[5]);
        *reinterpret_cast<float2 *>(o + 6) = make_float2(v[6], v[7]);
        o[8] = v[8];
    } else {
        o[0] = v[0];
        *reinterpret_cast<float4 *>(o + 1) = make_float4(v[1], v[2], v[3], v[4]);
        *reinterpret_cast<float4 *>(o + 5) = make_float4(v[5], v[6], v[7], v[8]);
    }
}

// The same for a 3x3 FP64 block (72 bytes, 8-byte aligned): four 16-byte
// stores and one 8-byte store.
__device__ __forceinline__ void store_block9(double *base, size_t p, const double v[9]) {
    double *o = base + p * 9;
    if (reinterpret_cast<uintptr_t>(o) & 15u) {
        o[0] = v[0];
        *reinterpret_cast<double2 *>(o + 1) = make_double2(v[1], v[2]);
        *reinterpret_cast<double2 *>(o + 3) = make_double2(v[3], v[4]);
        *reinterpret_cast<double2 *>(o + 5) = make_double2(v[5], v[6]);
        *reinterpret_cast<double2 *>(o + 7) = make_double2(v[7], v[8]);
    } else {
        *reinterpret_cast<double2 *>(o) = make_double2(v[0], v[1]);
        *reinterpret_cast<double2 *>(o + 2) = make_double2(v[2], v[3]);
        *reinterpret_cast<double2 *>(o + 4) = make_double2(v[4], v[5]);
        *reinterpret_cast<double2 *>(o + 6) = make_double2(v[6], v[7]);
        o[8] = v[8];
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

// Inverse of a symmetric 3x3 block by its six distinct cofactors in FP32;
// d = (d00, d11, d22, d01, d02, d12).  The block is first scaled by the power
// of two 2^-k that brings its largest diagonal entry to [1, 2) (exact), so that
// the cofactors (products of two entries) and the determinant (of three) stay
// inside the FP32 range for any entry magnitude; the inverse of the scaled
// block times 2^-k is the inverse.  Every cofactor is a 2x2 determinant
// a*b - c*d evaluated with Kahan's FMA method (within about one ulp), the
// determinant is their FMA dot product with the first row, and the inverse
// entries are cofactor * (1 / det): a few ulps relative error per entry for
// the block given.  Returns false for an exactly singular block, which is then
// left as it is.
__device__ __forceinline__ bool inv3_sym32(float d[6]) {
    const float mx = fmaxf(fabsf(d[0]), fmaxf(fabsf(d[1]), fabsf(d[2])));
    if (!(mx > 0.f) || mx > 3.0e38f) return false;   // zero, NaN or infinite diagonal
    const int ex = min(max((int)((__float_as_uint(mx) >> 23) & 0xffu) - 127, -126), 126);
    const float sc = __uint_as_float((unsigned)(127 - ex) << 23);   // 2^-ex, a normal float
    const float a = d[0] * sc, e = d[1] * sc, i = d[2] * sc, b = d[3] * sc, c = d[4] * sc,
                f = d[5] * sc;
    const float c00 = diff_prod(e, i, f, f);
    const float c01 = diff_prod(c, f, b, i);
    const float c02 = diff_prod(b, f, c, e);
    const float det = fmaf(a, c00, fmaf(b, c01, c * c02));
    if (det == 0.f) return false;
    const float r = sc / det;
    const float c11 = diff_prod(a, i, c, c);
    const float c12 = diff_prod(b, c, a, f);
    const float c22 = diff_prod(a, e, b, b);
    d[0] = c00 * r; d[1] = c11 * r; d[2] = c22 * r;
    d[3] = c01 * r; d[4] = c02 * r; d[5] = c12 * r;
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
    unsigned short *sC = reinterpret_cast<unsigned short *>(sm + L.contrib);
    int4 *sOff = reinterpret_cast<int4 *>(sm + L.off);
    int2 *sDiag = reinterpret_cast<int2 *>(sm + L.diag);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + L.bar);           // two barriers
    const int tid = threadIdx.x;

    // 0. stage the entry tables with the TMA engine (barrier 0)
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        // make the initialised barriers visible to the TMA (async) proxy
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned bo = (unsigned)T.nOffPad * 16u, bd = (unsigned)T.nRowsPad * 8u;
        mbar_expect_tx(bar, bo + bd + ctl.extraTx);
        if (bo) bulk_g2s(sOff, P.offEnt + T.offBegin, bo, bar);
        if (bd) bulk_g2s(sDiag, P.diagEnt + T.diagBegin, bd, bar);
    }

    // 1a. the weights of set 0 go to shared memory by asynchronous copies
    //     (cp.async, no register round trip); the connectivity of a thread's
    //     first two elements is loaded into registers; meanwhile the tile's node
    //     coordinates (hi and lo parts) are gathered into the contribution
    //     region, which the contribution lists fill only after phase 1
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
    float4 *Xh = reinterpret_cast<float4 *>(sm + L.contrib);
    float4 *Xl = Xh + T.nNodes;
    for (int i = tid; i < T.nNodes; i += kTileThreads) {
        const int n = P.nodes[T.nodeBegin + i];
        Xh[i] = M.hl[2 * n];
        Xl[i] = M.hl[2 * n + 1];
    }
    cp_async_wait_all();
    __syncthreads();

    // 1b. gradients of the tile's elements
    int flagged = 0;
    for (int i = tid; i < T.nElem; i += kTileThreads) {
        const ushort4 lc = i == i0 ? lc0 : i == i1 ? lc1 : P.lconn[T.elemBegin + i];
        ElemCoords C;
        C.h0 = Xh[lc.x]; C.h1 = Xh[lc.y]; C.h2 = Xh[lc.z]; C.h3 = Xh[lc.w];
        C.l0 = Xl[lc.x]; C.l1 = Xl[lc.y]; C.l2 = Xl[lc.z]; C.l3 = Xl[lc.w];
        float g[12];
        if (grad32_core(C, qthr2, g)) {
            const int *nb = P.nodes + T.nodeBegin;
            grad32_fp64(M.coord, make_int4(nb[lc.x], nb[lc.y], nb[lc.z], nb[lc.w]), g);
            flagged++;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) G[gslot(i, j)] = make_float4(g[3 * j], g[3 * j + 1], g[3 * j + 2], 0.f);
    }
    if (flagged) atomicAdd(counters + 1, flagged);
    __syncthreads();

    // the contribution lists (barrier 1), over the node coordinates: the
    // generic-proxy reads above are ordered before the async-proxy writes
    if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned bc = (unsigned)T.nContribPad * 2u;
        mbar_expect_tx(bar + 1, bc);
        if (bc) bulk_g2s(sC, P.contrib + T.contribBegin, bc, bar + 1);
    }
    // bounded wait for the staged segments (the CTA agrees on the outcome)
    bool ok = false;
    for (unsigned it = 0; it < ctl.waitLimit && !ok; it++)
        ok = mbar_try_wait(bar, 0) && mbar_try_wait(bar + 1, 0);
    if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicOr(counters + 2, 1);
        return false;
    }
    if (tid == 0) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar + 1)) : "memory");
    }

    for (int set = 0; set < S.nSets; set++) {
        float *values = S.values + (size_t)set * S.valuesStride;
        double *precOut = S.prec ? S.prec + (size_t)set * S.precStride : nullptr;
        if (set > 0) {
            // weights of this set (every thread is done with the previous set's)
            __syncthreads();
            const float2 *w = S.w + (size_t)set * S.wStride;
            for (int i = tid; i < T.nElem; i += kTileThreads) W[i] = w[P.elems[T.elemBegin + i]];
            __syncthreads();
        }

        // 2. off-diagonal units: entry (r, c) and, when c is a row of this tile,
        //    its transpose (c, r), which is the same sum transposed
        for (int t = tid; t < T.nOff; t += kTileThreads) {
            const int4 ent = sOff[t];
            const int b = (unsigned)ent.z >> 8, n = ent.z & 0xff;
            if (OP == MFEM_OP_LAP) {
                Kahan acc;
                for (int q = b; q < b + n; q++) {
                    const unsigned u = sC[q];
                    const int l = u >> 4;
                    const float4 gj = G[gslot(l, (u >> 2) & 3)], gk = G[gslot(l, u & 3)];
                    const float x = W[l].x * fmaf(gj.x, gk.x, fmaf(gj.y, gk.y, gj.z * gk.z));
                    if (q == b) { acc.s = x; acc.c = 0.f; } else acc.add(x);
                }
                const float v = acc.value();
                values[ent.x] = v;
                if (ent.y >= 0) values[ent.y] = v;
            } else {
                Kahan acc[9];
                for (int q = b; q < b + n; q++) {
                    const unsigned u = sC[q];
                    const int l = u >> 4;
                    const float4 gj = G[gslot(l, (u >> 2) & 3)], gk = G[gslot(l, u & 3)];
                    const float2 w = W[l];
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

        // 3. diagonal entries: four lanes per row sum a quarter of the row's
        //    contributions each and combine them without error; the first lane
        //    writes the block and its preconditioner block (inverted in FP32,
        //    stored as FP64)
        const int part = tid & 3;
        for (int base = 0; base < T.nRows; base += kTileThreads / 4) {
            const int rl = base + (tid >> 2);
            const bool active = rl < T.nRows;
            const int2 de = active ? sDiag[rl] : make_int2(0, 0);
            const int b = (unsigned)de.y >> 8, n = de.y & 0xff;
            const bool writer = active && part == 0;
            const int r = de.x;
            const int p = writer ? M.diagPos[r] : -1;
            const unsigned mk = (PREC && writer && M.mask) ? M.mask[r] : 0u;
            if (OP == MFEM_OP_LAP) {
                Kahan acc;
                for (int q = b + part; q < b + n; q += 4) {
                    const unsigned u = sC[q];
                    const int l = u >> 4;
                    const float4 g = G[gslot(l, (u >> 2) & 3)];
                    acc.add(W[l].x * fmaf(g.x, g.x, fmaf(g.y, g.y, g.z * g.z)));
                }
                quad_combine(acc);
                if (writer) {
                    const float v = acc.value();
                    if (p >= 0) values[p] = v;
                    if (PREC) precOut[r] = f32_to_f64(1.0f / v);
                }
            } else {
                Kahan acc[6];
                for (int q = b + part; q < b + n; q += 4) {
                    const unsigned u = sC[q];
                    const int l = u >> 4;
                    const float2 w = W[l];
                    ela_diag_accumulate(acc, G[gslot(l, (u >> 2) & 3)], w.x, w.y);
                }
#pragma unroll
                for (int m = 0; m < 6; m++) quad_combine(acc[m]);
                if (writer) {
                    float sv[6], d[6];
#pragma unroll
                    for (int m = 0; m < 6; m++) {
                        sv[m] = acc[m].value();
                        d[m] = sv[m];
                    }
                    if (p >= 0) {
                        const float v[9] = {sv[0], sv[3], sv[4], sv[3], sv[1], sv[5], sv[4], sv[5], sv[2]};
                        store_block9(values, (size_t)p, v);
                    }
                    if (PREC) {
                        // src/Fortran/elasclpr.f:19-27: constrained DOF k -> row and
                        // column k of the block zero, diagonal 1
                        if (mk & 1u) { d[0] = 1.f; d[3] = 0.f; d[4] = 0.f; }
                        if (mk & 2u) { d[1] = 1.f; d[3] = 0.f; d[5] = 0.f; }
                        if (mk & 4u) { d[2] = 1.f; d[4] = 0.f; d[5] = 0.f; }
                        if (p >= 0 && !inv3_sym32(d)) atomicAdd(counters, 1);
                        double x[6];
#pragma unroll
                        for (int m = 0; m < 6; m++) x[m] = f32_to_f64(d[m]);
                        const double o[9] = {x[0], x[3], x[4], x[3], x[1], x[5], x[4], x[5], x[2]};
                        store_block9(precOut, (size_t)r, o);
                    }
                }
            }
        }
    }
    return true;
}

}  // namespace tilek
}  // namespace mfem
