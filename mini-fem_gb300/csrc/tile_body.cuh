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

// One tile for nSets coefficient sets: the gradients are computed once, the
// weights, entries and preconditioner blocks once per set.  Returns false when
// the staged plan segments did not arrive within the bounded wait (error flag
// counters[2] set; the caller stops).
template <int OP, bool PREC>
__device__ __forceinline__ bool tile_body(const TileDesc &T, const TileMesh &M, const TileSets &S,
                                          const TilePlanView &P, const SmemLayout &L, float qthr2,
                                          unsigned char *sm, int *counters) {
    float4 *G = reinterpret_cast<float4 *>(sm);                       // 4 per element
    float4 *W = reinterpret_cast<float4 *>(sm + L.w);                 // 1 per element
    unsigned short *sC = reinterpret_cast<unsigned short *>(sm + L.contrib);
    int2 *sOff = reinterpret_cast<int2 *>(sm + L.off);
    int2 *sDiag = reinterpret_cast<int2 *>(sm + L.diag);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + L.bar);
    const int tid = threadIdx.x;

    // 0. stage the plan segments with the TMA engine
    if (tid == 0) {
        mbar_init(bar, 1);
        // make the initialised barrier visible to the TMA (async) proxy
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned bc = (unsigned)T.nContribPad * 2u, bo = (unsigned)T.nOffPad * 8u,
                       bd = (unsigned)T.nRowsPad * 8u;
        mbar_expect_tx(bar, bc + bo + bd);
        if (bc) bulk_g2s(sC, P.contrib + T.contribBegin, bc, bar);
        if (bo) bulk_g2s(sOff, P.offEnt + T.offBegin, bo, bar);
        if (bd) bulk_g2s(sDiag, P.diagEnt + T.diagBegin, bd, bar);
    }

    // 1. gradients of the tile's elements (and the weights of set 0)
    int flagged = 0;
    for (int i = tid; i < T.nElem; i += kTileThreads) {
        const int e = P.elems[T.elemBegin + i];
        float g[12];
        flagged += grad32(M.hi, M.lo, M.coord, M.e2n[e], qthr2, g);
#pragma unroll
        for (int j = 0; j < 4; j++) G[4 * i + j] = make_float4(g[3 * j], g[3 * j + 1], g[3 * j + 2], 0.f);
        W[i] = weights32<OP>(S.coef, e);
    }
    if (flagged) atomicAdd(counters + 1, flagged);
    __syncthreads();

    // bounded wait for the staged segments (the CTA agrees on the outcome)
    bool ok = false;
    for (int it = 0; it < (1 << 22) && !ok; it++) ok = mbar_try_wait(bar, 0);
    if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicOr(counters + 2, 1);
        return false;
    }
    if (tid == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");

  for (int set = 0; set < S.nSets; set++) {
    float *values = S.values + (size_t)set * S.valuesStride;
    double *precOut = S.prec ? S.prec + (size_t)set * S.precStride : nullptr;
    if (set > 0) {
        // weights of this set (every thread is done with the previous set's)
        __syncthreads();
        const double *coef = S.coef ? S.coef + (size_t)set * S.coefStride : nullptr;
        for (int i = tid; i < T.nElem; i += kTileThreads)
            W[i] = weights32<OP>(coef, P.elems[T.elemBegin + i]);
        __syncthreads();
    }

    // 2. off-diagonal entries
    for (int t = tid; t < T.nOff; t += kTileThreads) {
        const int2 ent = sOff[t];
        const int b = (unsigned)ent.y >> 8, n = ent.y & 0xff;
        if (OP == MFEM_OP_LAP) {
            Kahan acc;
            for (int q = b; q < b + n; q++) {
                const unsigned u = sC[q];
                const int l = u >> 4;
                const float4 gj = G[4 * l + ((u >> 2) & 3)], gk = G[4 * l + (u & 3)];
                acc.add(W[l].x * fmaf(gj.x, gk.x, fmaf(gj.y, gk.y, gj.z * gk.z)));
            }
            values[ent.x] = acc.value();
        } else {
            Kahan acc[9];
            for (int q = b; q < b + n; q++) {
                const unsigned u = sC[q];
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
            float *v = values + (size_t)ent.x * 9;
#pragma unroll
            for (int m = 0; m < 9; m++) v[m] = acc[m].value();
        }
    }

    // 3. diagonal entries + preconditioner: four lanes per row
    const int part = tid & 3;
    for (int base = 0; base < T.nRows; base += kTileThreads / 4) {
        const int rl = base + (tid >> 2);
        const bool active = rl < T.nRows;
        const int2 de = active ? sDiag[rl] : make_int2(0, 0);
        const int r = de.x;
        const int b = (unsigned)de.y >> 8, n = de.y & 0xff;
        if (OP == MFEM_OP_LAP) {
            Kahan acc;
            for (int q = b + part; q < b + n; q += 4) {
                const unsigned u = sC[q];
                const int l = u >> 4;
                const float4 g = G[4 * l + ((u >> 2) & 3)];
                acc.add(W[l].x * fmaf(g.x, g.x, fmaf(g.y, g.y, g.z * g.z)));
            }
            quad_combine(acc);
            if (active && part == 0) {
                const int p = M.diagPos[r];
                if (p >= 0) values[p] = acc.value();
                if (PREC) precOut[r] = 1.0 / ((double)acc.s - (double)acc.c);
            }
        } else {
            Kahan acc[6];
            for (int q = b + part; q < b + n; q += 4) {
                const unsigned u = sC[q];
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
#pragma unroll
            for (int m = 0; m < 6; m++) quad_combine(acc[m]);
            if (active && part == 0) {
                const int p = M.diagPos[r];
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
                    if (M.mask) dirichlet_mask3(a, M.mask[r]);
                    if (p >= 0 && !inv3_cofactor(a)) atomicAdd(counters, 1);
                    double *o = precOut + (size_t)r * 9;   // 72-byte blocks: 8-byte aligned
#pragma unroll
                    for (int m = 0; m < 9; m++) o[m] = a[m];
                }
            }
        }
    }
  }
    return true;
}

}  // namespace tilek
}  // namespace mfem
