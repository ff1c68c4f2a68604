// Consumer of the assembled system: operator apply (block-CSR SpMV), block-
// Jacobi apply and block-Jacobi preconditioned conjugate gradients, on the
// device.  No counterpart in the reference, whose driver names the step after
// assembly ("assembly, solver & update", src/main.cc:353) without implementing
// it; the preconditioner is the one prec_inversion produces
// (src/preconditioner.cc:25-49).
//
// Homogeneous Dirichlet constraints come from the check bounds
// (src/Fortran/elasclpr.f:19-27 masks the same DOFs in the preconditioner): a
// constrained DOF is taken as 0 in every product and its row is the identity,
// so the operator is M A M + (I - M) with M the 0/1 mask of free DOFs, whose
// block-Jacobi inverse is exactly the masked, inverted diagonal block.
//
// Arithmetic: with FP64 values the operator is an FP64 FMA chain per row; with
// FP32 values (the FP32 assembly) it runs on the FP32 pipes in double-float
// (x scaled by a power of two and split into FP32 hi + lo, exact hi products,
// TwoSum accumulation), GB300's FP64 pipe being 1/64 of its FP32 rate.
//
// Reductions are deterministic: fixed grid, fixed tree order in each CTA, CTA
// partials summed in index order by the CTA that finishes last (inside CG) or
// by one CTA.
#include <algorithm>
#include <cmath>

#include "context.h"
#include "dmul_int.cuh"
#include "elem32.cuh"
#include "spmv_df.cuh"

namespace mfem {

int op_dim_of(const Context &c) { return c.lastOp == MFEM_OP_LAP ? 1 : 9; }

namespace {

constexpr int kThreads = 256;
constexpr int kLanesPerRow = 4;          // SpMV: four lanes share a block row (measured best of 2-16)
constexpr int kRowsPerCta = kThreads / kLanesPerRow;

__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return f32_to_f64(v); }

// Tree sum of one value per thread into partial[blockIdx.x] (fixed order).
__device__ __forceinline__ void cta_sum(double v, double *partial) {
    __shared__ double s[kThreads / 32];
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; w++) t += s[w];
        partial[blockIdx.x] = t;
    }
}

// Scalars of the CG recurrence, kept on the device.
struct CgScalars {
    double rz, pq, alpha, beta, rr, bb, tol2;
    int iter, maxIter, stop;   // stop: converged or out of iterations; later kernels do nothing
};

// What a CG kernel needs to finish its own reduction: the CTA that completes
// last sums the CTA partials and updates the scalars, so that no separate
// reduction launch follows.  sc == nullptr: not inside CG.
struct CgLink {
    CgScalars *sc = nullptr;
    double *sums = nullptr;
    unsigned *counter = nullptr;              // CTAs done; zero between kernels
    unsigned long long *scaleMax = nullptr;   // FP32 values: max |p| the split of p used
    unsigned long long *nextMax = nullptr;    //   and max |p| of the p being formed
};

// Sums of nSums arrays of nCta partials, each in index order by a strided sum
// per thread and a fixed tree: run by the CTA that finishes last, which then
// calls `then` on one thread.  Every thread of the grid calls it after its
// CTA's partials are written; the counter is left at zero.  t: kThreads
// doubles of shared memory the caller no longer needs (its staging buffer),
// so that the kernel's shared-memory footprint does not grow.
template <class F>
__device__ __forceinline__ void last_cta_sums(const double *partial, int nCta, int nSums, double *sums,
                                              unsigned *counter, double *t, F then) {
    __shared__ bool last;
    __threadfence();   // the partials written by this CTA, before its count
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int k = 0; k < nSums; k++) {
        double v = 0.0;
        for (int i = threadIdx.x; i < nCta; i += kThreads) v += __ldcg(partial + (size_t)k * nCta + i);
        t[threadIdx.x] = v;
        __syncthreads();
        for (int w = kThreads / 2; w >= 1; w >>= 1) {
            if ((int)threadIdx.x < w) t[threadIdx.x] += t[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) sums[k] = t[0];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        then(sums);
        *counter = 0u;
    }
}

// alpha = (r . z) / (p . q)
__device__ __forceinline__ void cg_alpha(CgScalars *sc, const double *sums) {
    sc->pq = sums[0];
    sc->alpha = sc->pq != 0.0 ? sc->rz / sc->pq : 0.0;
}

// beta, the new r . z and r . r, the stop test; for FP32 values the max of the
// current p becomes the scale of the next p's split
__device__ __forceinline__ void cg_beta(CgScalars *sc, const double *sums, CgLink link) {
    const double rzNew = sums[0];
    sc->beta = sc->rz != 0.0 ? rzNew / sc->rz : 0.0;
    sc->rz = rzNew;
    sc->rr = sums[1];
    sc->iter++;
    if (sc->rr <= sc->tol2 * sc->bb || sc->iter >= sc->maxIter) sc->stop = 1;
    if (link.scaleMax) {
        *link.scaleMax = *link.nextMax;
        *link.nextMax = 0ull;
    }
}

__device__ __forceinline__ bool constrained(const unsigned char *mask, int node, int k, int dim) {
    return mask && (dim == 1 ? mask[node] != 0 : ((mask[node] >> k) & 1u));
}

// y = A x; with `partial`, also the CTA partial sums of x . y.  Four lanes
// share a block row: for every chunk of four blocks they copy the chunk's
// values (contiguous in CSR order) into shared memory with coalesced loads,
// then each lane multiplies one block by its gathered x entries.
template <typename V, int D>
__global__ void __launch_bounds__(kThreads)
k_spmv(const int *__restrict__ rowPtr, const int *__restrict__ col, const V *__restrict__ vals,
       const double *__restrict__ x, double *__restrict__ y, int N,
       const unsigned char *__restrict__ mask, double *__restrict__ partial,
       const int *__restrict__ stop, CgLink link) {
    if (stop && *stop) return;   // CG: converged in an earlier iteration of the batch
    constexpr int B = D * D;
    __shared__ V sv[kRowsPerCta][kLanesPerRow * B];
    const int g = threadIdx.x / kLanesPerRow;
    const int row = blockIdx.x * kRowsPerCta + g;
    const int sub = threadIdx.x % kLanesPerRow;
    const unsigned gmask = ((1u << kLanesPerRow) - 1u) << (threadIdx.x & (32 - kLanesPerRow));   // this row's lanes
    double a[D];
#pragma unroll
    for (int d = 0; d < D; d++) a[d] = 0.0;
    int kb = 0, ke = 0;
    if (row < N) {
        kb = rowPtr[row];
        ke = rowPtr[row + 1];
    }
    for (int k0 = kb; k0 < ke; k0 += kLanesPerRow) {
        const int nb = min(kLanesPerRow, ke - k0);
        const V *src = vals + (size_t)k0 * B;
        for (int m = sub; m < nb * B; m += kLanesPerRow) sv[g][m] = src[m];
        __syncwarp(gmask);
        if (sub < nb) {
            const int c = col[k0 + sub];
            const unsigned mc = mask ? mask[c] : 0u;
            double xc[D];
#pragma unroll
            for (int d = 0; d < D; d++)
                xc[d] = (D == 1 ? mc != 0u : ((mc >> d) & 1u)) ? 0.0 : x[(size_t)c * D + d];
            const V *v = sv[g] + sub * B;
#pragma unroll
            for (int i = 0; i < D; i++)
#pragma unroll
                for (int j = 0; j < D; j++) a[i] = fma(to_f64(v[D * i + j]), xc[j], a[i]);
        }
        __syncwarp(gmask);
    }
#pragma unroll
    for (int off = kLanesPerRow / 2; off >= 1; off >>= 1)
#pragma unroll
        for (int d = 0; d < D; d++) a[d] += __shfl_xor_sync(0xffffffffu, a[d], off);
    double dot = 0.0;
    if (row < N && sub == 0) {
#pragma unroll
        for (int d = 0; d < D; d++) {
            const double xv = x[(size_t)row * D + d];
            const double yv = constrained(mask, row, d, D) ? xv : a[d];
            y[(size_t)row * D + d] = yv;
            dot = fma(xv, yv, dot);
        }
    }
    if (partial) cta_sum(dot, partial);
    static_assert(sizeof(sv) >= sizeof(double) * kThreads, "staging buffer reused by the reduction");
    if (link.sc)
        last_cta_sums(partial, (int)gridDim.x, 1, link.sums, link.counter, reinterpret_cast<double *>(&sv[0][0]),
                      [&](const double *sm) { cg_alpha(link.sc, sm); });
}

// ---- FP32 values: the operator without the FP64 pipe ----
//
// x is scaled by the power of two 2^-kx that brings max |x| just below 1 (kx
// from the largest |x| bit pattern, kept on the device in *xmax) and split into
// FP32 hi + lo parts; every product a x_j is then the exact a hi (FP32 product
// and its FMA error) plus the rounded a lo, summed in double-float, and y is
// scaled back by 2^kx.

// Largest |x| bit pattern (non-negative doubles order as their bit patterns)
// of a CTA's values into *xmax: one atomic per CTA (every thread calls it).
__device__ __forceinline__ void block_max_into(unsigned long long b, unsigned long long *xmax) {
    __shared__ unsigned long long wm[kThreads / 32];
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, b, off);
        b = o > b ? o : b;
    }
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) b = wm[w] > b ? wm[w] : b;
        if (b) atomicMax(xmax, b);
    }
}

// grid of the grid-stride vector kernels that reduce a maximum: few enough
// CTAs that their atomics on one word stay cheap
constexpr long long kMaxCtas = 1024;

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// kx with 2^kx > max |x|; 0 for a zero or non-finite maximum.
__device__ __forceinline__ int scale_exp(const unsigned long long *xmax) {
    const int e = (int)(*xmax >> 52);
    return (e == 0 || e == 0x7ff) ? 0 : e - 1022;
}

// hi + lo FP32 parts of x 2^-kx, on the integer pipes.  Zero gives (0, 0); a
// value below 2^-60 max |x| (or subnormal) or a non-finite one gives a NaN hi
// part, so that every row that reads it takes the FP64 path.
__device__ __forceinline__ float2 split_x(double v, int kx) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if ((b << 1) == 0u) return make_float2(0.f, 0.f);
    const int e = (int)((b >> 52) & 0x7ffu);
    uint32_t hb, lb;
    if (e != 0x7ff && e - kx >= 1023 - 60 &&
        split_f32_bits(b - ((unsigned long long)(long long)kx << 52), &hb, &lb))
        return make_float2(__uint_as_float(hb), __uint_as_float(lb));
    return make_float2(__int_as_float(0x7fffffff), 0.f);
}

__global__ void __launch_bounds__(kThreads)
k_xmax(const double *__restrict__ x, long long n, unsigned long long *__restrict__ xmax) {
    unsigned long long b = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long v = abs_bits(x[i]);
        b = v > b ? v : b;
    }
    block_max_into(b, xmax);
}

// The split of x, with the constrained DOFs (mask) as zero: the operator's
// M x.
template <int D>
__global__ void k_split_x(const double *__restrict__ x, float2 *__restrict__ xs, long long n,
                          const unsigned long long *__restrict__ xmax, const unsigned char *__restrict__ mask,
                          const int *__restrict__ stop) {
    if (stop && *stop) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool z = mask && constrained(mask, (int)(i / D), (int)(i % D), D);
    xs[i] = z ? make_float2(0.f, 0.f) : split_x(x[i], scale_exp(xmax));
}

// asynchronous global -> shared copies (no register round trip): 4 bytes, and
// 16 bytes (both addresses 16-byte aligned; L2 only, the values stream)
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

// k_spmv32: lanes per block row, and blocks of a row staged per lane and chunk
constexpr int kLanes32 = 4;
constexpr int kRows32 = kThreads / kLanes32;
constexpr int kSpmvBlocksPerLane = 2;

// y = A x for FP32 values from the split xs: the hi products by TwoSum into s,
// every error term and lo product into t; the four lanes' (s, t) merged in
// double-float, each lane's pair renormalized after every chunk; y = (s + t)
// 2^kx, within 15 x 2^-48 of sum |a x| over the row (spmv_df.cuh).
//
// Four lanes share a block row and take its blocks in chunks of 8 (lane l the
// blocks l and l + 4): a chunk's values go to shared memory by 16-byte
// asynchronous copies (from the 16-byte boundary at or below the chunk, the
// last piece of the array by 4-byte copies) while its columns and x parts are
// gathered.  The constrained columns are zero in xs already (k_split_x).
//
// A row whose largest |hi product| is outside [2^-60, 2^100] (overflow, values
// near the FP32 underflow, an all-zero row, or an x entry that split_x marked)
// or whose sums are not finite is recomputed by its lanes with k_spmv's FP64
// chain on the unscaled x, in k_spmv's order and with its results.
template <int D, bool DOT>
__global__ void __launch_bounds__(kThreads)
k_spmv32(const int *__restrict__ rowPtr, const int *__restrict__ col, const float *__restrict__ vals,
         long long nVals, const float2 *__restrict__ xs, const unsigned long long *__restrict__ xmax,
         const double *__restrict__ x, double *__restrict__ y, int N,
         const unsigned char *__restrict__ mask, double *__restrict__ partial,
         const int *__restrict__ stop, CgLink link) {
    if (stop && *stop) return;
    constexpr int B = D * D, BPL = kSpmvBlocksPerLane, CH = kLanes32 * BPL;
    static_assert(kLanes32 >= D, "one lane per output component");
    // a chunk's values from the 16-byte boundary at or below its start: at
    // most 3 leading floats, whole 16-byte pieces
    constexpr int kPieces = (3 + CH * B + 3) / 4, kRow = 4 * kPieces;
    __shared__ __align__(16) float sv[kRows32][kRow];
    const int g = threadIdx.x / kLanes32;
    const int row = blockIdx.x * kRows32 + g;
    const int sub = threadIdx.x % kLanes32;
    const unsigned gmask = ((1u << kLanes32) - 1u) << (threadIdx.x & (32 - kLanes32));
    const float *vend = vals + nVals;
    float s[D], t[D];
#pragma unroll
    for (int d = 0; d < D; d++) s[d] = t[d] = 0.f;
    float pmax = 0.f;
    int kb = 0, ke = 0;
    if (row < N) {
        kb = rowPtr[row];
        ke = rowPtr[row + 1];
    }
    for (int k0 = kb; k0 < ke; k0 += CH) {
        const int nb = min(CH, ke - k0);
        int cc[BPL];
#pragma unroll
        for (int j = 0; j < BPL; j++) {
            const int k = k0 + sub + kLanes32 * j;
            cc[j] = k < ke ? col[k] : -1;
        }
        const float *cv = vals + (size_t)k0 * B;
        const float *base = reinterpret_cast<const float *>(reinterpret_cast<uintptr_t>(cv) & ~(uintptr_t)15);
        const int lead = (int)(cv - base);
        const int np = (lead + nb * B + 3) >> 2;
#pragma unroll
        for (int r = 0; r < (kPieces + kLanes32 - 1) / kLanes32; r++) {
            const int pc = sub + kLanes32 * r;
            if (pc < np) {
                const float *src = base + 4 * pc;
                float *dst = &sv[g][4 * pc];
                if (src + 4 <= vend) {
                    cp_async16(dst, src);
                } else {
                    // the last piece of the array: only what lies inside it
                    for (int q = 0; q < 4 && src + q < vend; q++) cp_async4(dst + q, src + q);
                }
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        float2 xv[BPL][D];
#pragma unroll
        for (int j = 0; j < BPL; j++) {
#pragma unroll
            for (int d = 0; d < D; d++)
                xv[j][d] = cc[j] >= 0 ? xs[(size_t)cc[j] * D + d] : make_float2(0.f, 0.f);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncwarp(gmask);
#pragma unroll
        for (int j = 0; j < BPL; j++) {
            if (cc[j] < 0) continue;
            const float *v = sv[g] + lead + (sub + kLanes32 * j) * B;
#pragma unroll
            for (int i = 0; i < D; i++) {
#pragma unroll
                for (int jj = 0; jj < D; jj++) {
                    pmax = fmaxf(pmax, spdf::accumulate(s[i], t[i], v[D * i + jj], xv[j][jj].x, xv[j][jj].y));
                }
            }
        }
#pragma unroll
        for (int i = 0; i < D; i++) spdf::renormalize(s[i], t[i]);
        __syncwarp(gmask);
    }
    // the row's four lanes: largest product, finiteness and the double-float
    // sums, combined without the FP64 pipe
    bool finite = true;
#pragma unroll
    for (int off = kLanes32 / 2; off >= 1; off >>= 1) {
        pmax = fmaxf(pmax, __shfl_xor_sync(0xffffffffu, pmax, off));
#pragma unroll
        for (int d = 0; d < D; d++) {
            const float s2 = __shfl_xor_sync(0xffffffffu, s[d], off);
            const float t2 = __shfl_xor_sync(0xffffffffu, t[d], off);
            spdf::merge(s[d], t[d], s2, t2);
        }
    }
#pragma unroll
    for (int d = 0; d < D; d++) finite = finite && isfinite(s[d]) && isfinite(t[d]);
    const bool bad = !(finite && pmax >= 0x1.0p-60f && pmax <= 0x1.0p100f);
    double a[D];
#pragma unroll
    for (int d = 0; d < D; d++) a[d] = 0.0;
    if (__any_sync(0xffffffffu, bad)) {
        if (bad) {
            for (int k = kb + sub; k < ke; k += kLanes32) {
                const int c = col[k];
                const unsigned mc = mask ? mask[c] : 0u;
                double xc[D];
#pragma unroll
                for (int d = 0; d < D; d++)
                    xc[d] = (D == 1 ? mc != 0u : ((mc >> d) & 1u)) ? 0.0 : x[(size_t)c * D + d];
                const float *v = vals + (size_t)k * B;
#pragma unroll
                for (int i = 0; i < D; i++)
#pragma unroll
                    for (int j = 0; j < D; j++) a[i] = fma(to_f64(v[D * i + j]), xc[j], a[i]);
            }
        }
#pragma unroll
        for (int off = kLanes32 / 2; off >= 1; off >>= 1)
#pragma unroll
            for (int d = 0; d < D; d++) a[d] += __shfl_xor_sync(0xffffffffu, a[d], off);
    }
    // every lane holds the row's sums: lane d writes component d (one FP64
    // addition per lane instead of D on one lane)
    double dot = 0.0;
    if (row < N && sub < D) {
        float sd = s[0], td = t[0];
        double ad = a[0];
#pragma unroll
        for (int d = 1; d < D; d++)
            if (sub == d) { sd = s[d]; td = t[d]; ad = a[d]; }
        const double xv = x[(size_t)row * D + sub];
        double yv = bad ? ad : scale_pow2(f32_to_f64(sd) + f32_to_f64(td), scale_exp(xmax));
        if (constrained(mask, row, sub, D)) yv = xv;
        y[(size_t)row * D + sub] = yv;
        if (DOT) dot = xv * yv;
    }
    if (DOT) cta_sum(dot, partial);
    static_assert(sizeof(sv) >= sizeof(double) * kThreads, "staging buffer reused by the reduction");
    if (DOT && link.sc)
        last_cta_sums(partial, (int)gridDim.x, 1, link.sums, link.counter, reinterpret_cast<double *>(&sv[0][0]),
                      [&](const double *sm) { cg_alpha(link.sc, sm); });
}

// z = P r (block-Jacobi), one thread per node.
template <int D>
__global__ void k_prec_apply(const double *__restrict__ prec, const double *__restrict__ r,
                             double *__restrict__ z, int N) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double *P = prec + (size_t)i * D * D;
#pragma unroll
    for (int a = 0; a < D; a++) {
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < D; b++) s = fma(P[D * a + b], r[(size_t)i * D + b], s);
        z[(size_t)i * D + a] = s;
    }
}

// r = b - A x (A x already in q); z = P r; partials of r . z, r . r and b . b.
template <int D>
__global__ void __launch_bounds__(kThreads)
k_cg_init(const double *__restrict__ prec, const double *__restrict__ b, const double *__restrict__ q,
          double *__restrict__ r, double *__restrict__ z, double *__restrict__ p,
          unsigned long long *__restrict__ pmax, int N, double *__restrict__ partial, int nCta) {
    unsigned long long pm = 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rz = 0.0, rr = 0.0, bb = 0.0;
    if (i < N) {
        double rv[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            const double bv = b[(size_t)i * D + d];
            rv[d] = bv - q[(size_t)i * D + d];
            r[(size_t)i * D + d] = rv[d];
            bb = fma(bv, bv, bb);
            rr = fma(rv[d], rv[d], rr);
        }
        const double *P = prec + (size_t)i * D * D;
#pragma unroll
        for (int a = 0; a < D; a++) {
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < D; c++) s = fma(P[D * a + c], rv[c], s);
            z[(size_t)i * D + a] = s;
            p[(size_t)i * D + a] = s;
            const unsigned long long sb = abs_bits(s);
            pm = sb > pm ? sb : pm;
            rz = fma(rv[a], s, rz);
        }
    }
    if (pmax) block_max_into(pm, pmax);
    cta_sum(rz, partial);
    __syncthreads();
    cta_sum(rr, partial + nCta);
    __syncthreads();
    cta_sum(bb, partial + 2 * nCta);
}

// Sums `nSums` arrays of nCta partials (in index order) into sums[0..nSums).
__global__ void k_sum_partials(const double *__restrict__ partial, int nCta, int nSums,
                               double *__restrict__ sums, const int *__restrict__ stop) {
    if (stop && *stop) return;
    __shared__ double s[kThreads];
    for (int k = 0; k < nSums; k++) {
        double t = 0.0;
        for (int i = threadIdx.x; i < nCta; i += kThreads) t += partial[(size_t)k * nCta + i];
        s[threadIdx.x] = t;
        __syncthreads();
        for (int w = kThreads / 2; w >= 1; w >>= 1) {
            if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) sums[k] = s[0];
        __syncthreads();
    }
}

__global__ void k_cg_start(CgScalars *sc, const double *sums, double tol2, int maxIter, CgLink link) {
    if (link.scaleMax) *link.scaleMax = *link.nextMax;   // the scale of p's first split
    sc->rz = sums[0];
    sc->rr = sums[1];
    sc->bb = sums[2];
    sc->tol2 = tol2;
    sc->iter = 0;
    sc->maxIter = maxIter;
    sc->stop = (sc->rr <= tol2 * sc->bb || maxIter <= 0) ? 1 : 0;
}

// x += alpha p; r -= alpha q; z = P r; partials of r . z and r . r.  Grid-
// stride over the nodes (nCta == gridDim.x CTAs, four per SM: several nodes
// per thread), so that the CTA reductions and the last CTA's sum are spread
// over more work.
template <int D>
__global__ void __launch_bounds__(kThreads)
k_cg_update(const double *__restrict__ prec, CgScalars *__restrict__ sc,
            const double *__restrict__ p, const double *__restrict__ q, double *__restrict__ x,
            double *__restrict__ r, double *__restrict__ z, int N, double *__restrict__ partial,
            int nCta, CgLink link) {
    if (sc->stop) return;
    const double alpha = sc->alpha;
    double rz = 0.0, rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        double rv[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            const size_t o = (size_t)i * D + d;
            x[o] = fma(alpha, p[o], x[o]);
            rv[d] = fma(-alpha, q[o], r[o]);
            r[o] = rv[d];
            rr = fma(rv[d], rv[d], rr);
        }
        const double *P = prec + (size_t)i * D * D;
#pragma unroll
        for (int a = 0; a < D; a++) {
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < D; c++) s = fma(P[D * a + c], rv[c], s);
            z[(size_t)i * D + a] = s;
            rz = fma(rv[a], s, rz);
        }
    }
    cta_sum(rz, partial);
    __syncthreads();
    cta_sum(rr, partial + nCta);
    __shared__ double t[kThreads];
    last_cta_sums(partial, nCta, 2, link.sums, link.counter, t,
                  [&](const double *sm) { cg_beta(sc, sm, link); });
}

// p = z + beta p; grid-stride.  For the FP32-valued operator also the split
// of p (constrained DOFs zero) at the scale of *link.scaleMax, the previous
// p's maximum, which the operator then uses, and max |p| into *link.nextMax
// for the next split.  A scale from the previous p only shifts where the split
// range lies: entries it cannot serve are marked and their rows take FP64.
template <int D>
__global__ void __launch_bounds__(kThreads)
k_cg_direction(const CgScalars *__restrict__ sc, const double *__restrict__ z, double *__restrict__ p,
               float2 *__restrict__ ps, const unsigned char *__restrict__ mask, long long n, CgLink link) {
    if (sc->stop) return;
    const double beta = sc->beta;
    const int kx = ps ? scale_exp(link.scaleMax) : 0;
    unsigned long long pm = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = fma(beta, p[i], z[i]);
        p[i] = v;
        if (ps) {
            const bool c = mask && constrained(mask, (int)(i / D), (int)(i % D), D);
            ps[i] = c ? make_float2(0.f, 0.f) : split_x(v, kx);
            const unsigned long long b = abs_bits(v);
            pm = b > pm ? b : pm;
        }
    }
    if (ps) block_max_into(pm, link.nextMax);
}

// Split of an SpMV operand for FP32 values: its hi/lo parts and the largest
// |x| bit pattern that sets their scale.
struct XSplit {
    float2 *xs = nullptr;
    unsigned long long *xmax = nullptr;
    bool ready = false;   // xs already holds the split at the scale of *xmax (CG)
};

// FP32 values: the split of x made here (into c.xsplit) unless given ready.
// Inside CG (link.sc set) the operator also finishes p . q and alpha.
template <int D>
void spmv_t(Context &c, const double *x, double *y, const unsigned char *mask, double *partial,
            const int *stop, XSplit xsp, CgLink link, cudaStream_t s) {
    const unsigned grid = blocks_for(c.nbNodes, kRowsPerCta);
    if (c.lastPrecision == MFEM_FP32) {
        const unsigned grid32 = blocks_for(c.nbNodes, kRows32);
        const long long n = (long long)c.nbNodes * D;
        if (!xsp.ready) {
            if (!xsp.xs) {
                char *w = (char *)c.xsplit.reserve(sizeof(float2) * (size_t)n + 256);
                xsp.xmax = reinterpret_cast<unsigned long long *>(w);
                xsp.xs = reinterpret_cast<float2 *>(w + 256);
            }
            MFEM_CUDA(cudaMemsetAsync(xsp.xmax, 0, sizeof(unsigned long long), s));
            k_xmax<<<(unsigned)std::min<long long>(blocks_for(n, kThreads), kMaxCtas), kThreads, 0, s>>>(x, n, xsp.xmax);
            check_launch("k_xmax");
            k_split_x<D><<<blocks_for(n, kThreads), kThreads, 0, s>>>(x, xsp.xs, n, xsp.xmax, mask, stop);
            check_launch("k_split_x");
        }
        const long long nv = (long long)c.nnz * D * D;
        if (partial)
            k_spmv32<D, true><<<grid32, kThreads, 0, s>>>(c.rowPtr.as<int>(), c.col.as<int>(), c.values.as<float>(),
                                                        nv, xsp.xs, xsp.xmax, x, y, c.nbNodes, mask, partial, stop,
                                                        link);
        else
            k_spmv32<D, false><<<grid32, kThreads, 0, s>>>(c.rowPtr.as<int>(), c.col.as<int>(), c.values.as<float>(),
                                                         nv, xsp.xs, xsp.xmax, x, y, c.nbNodes, mask, nullptr, stop,
                                                         CgLink{});
    } else {
        k_spmv<double, D><<<grid, kThreads, 0, s>>>(c.rowPtr.as<int>(), c.col.as<int>(), c.values.as<double>(),
                                                    x, y, c.nbNodes, mask, partial, stop, link);
    }
    check_launch("k_spmv");
}

void spmv(Context &c, const double *x, double *y, const unsigned char *mask, double *partial,
          const int *stop = nullptr, XSplit xsp = {}, CgLink link = {}) {
    if (op_dim_of(c) == 9) spmv_t<3>(c, x, y, mask, partial, stop, xsp, link, c.stream);
    else spmv_t<1>(c, x, y, mask, partial, stop, xsp, link, c.stream);
}

// CG iterations enqueued between two looks at the convergence flag
constexpr int kCgBatch = 8;

}  // namespace

static void require_assembled(const Context &c, bool needPrec) {
    MFEM_REQUIRE(c.lastOp >= 0 && c.values.ptr, MFEM_ERR_STATE, "no assembled matrix");
    if (needPrec) MFEM_REQUIRE(c.prec.ptr && c.precIsInit, MFEM_ERR_STATE, "no preconditioner");
}

static const unsigned char *solve_mask(const Context &c, int constrainedFlag) {
    return constrainedFlag && c.hasMask ? c.mask.as<unsigned char>() : nullptr;
}

void spmv_device(Context &c, const double *x, double *y, int constrainedFlag) {
    require_assembled(c, false);
    spmv(c, x, y, solve_mask(c, constrainedFlag), nullptr);
}

void prec_apply_device(Context &c, const double *r, double *z) {
    require_assembled(c, true);
    const unsigned g = blocks_for(c.nbNodes, kThreads);
    if (op_dim_of(c) == 9) k_prec_apply<3><<<g, kThreads, 0, c.stream>>>(c.prec.as<double>(), r, z, c.nbNodes);
    else k_prec_apply<1><<<g, kThreads, 0, c.stream>>>(c.prec.as<double>(), r, z, c.nbNodes);
    check_launch("k_prec_apply");
}

// Block-Jacobi PCG on the latest assembly; b and x are host arrays (x: initial
// guess in, solution out).
void pcg(Context &c, const double *b, double *x, double rtol, int maxIter, int constrainedFlag,
         int *iters, double *relres) {
    require_assembled(c, true);
    MFEM_REQUIRE(b && x, MFEM_ERR_INVALID_ARG, "null b or x");
    MFEM_REQUIRE(maxIter >= 0, MFEM_ERR_INVALID_ARG, "negative maxIter");
    const int D = op_dim_of(c) == 9 ? 3 : 1;
    const size_t n = (size_t)c.nbNodes * D;
    const int nCtaRows = (int)blocks_for(c.nbNodes, c.lastPrecision == MFEM_FP32 ? kRows32 : kRowsPerCta);
    const int nCtaNodes = (int)blocks_for(c.nbNodes, kThreads);
    const int nCta = std::max(nCtaRows, nCtaNodes);
    double *w = (double *)c.solver.reserve(sizeof(double) * (7 * n + 3 * (size_t)nCta + 12) + sizeof(CgScalars) + 64);
    double *vb = w, *vx = w + n, *vr = w + 2 * n, *vz = w + 3 * n, *vp = w + 4 * n, *vq = w + 5 * n;
    double *partial = w + 7 * n + 3;
    double *sums = partial + 3 * (size_t)nCta;
    CgScalars *sc = reinterpret_cast<CgScalars *>(sums + 8);
    // the fused reductions' CTA counter; for FP32 values the split of p (made
    // by the direction update) and the two maxima of |p|
    CgLink link;
    link.sc = sc;
    link.sums = sums;
    link.counter = reinterpret_cast<unsigned *>(w + 7 * n);
    XSplit ps;
    if (c.lastPrecision == MFEM_FP32) {
        ps.xs = reinterpret_cast<float2 *>(w + 6 * n);
        link.scaleMax = reinterpret_cast<unsigned long long *>(w + 7 * n + 1);
        link.nextMax = reinterpret_cast<unsigned long long *>(w + 7 * n + 2);
        ps.xmax = link.scaleMax;
        ps.ready = true;
    }
    CgScalars *hostSc = nullptr;
    MFEM_CUDA(cudaMallocHost(&hostSc, sizeof(CgScalars)));
    struct Free {
        CgScalars *p;
        ~Free() { cudaFreeHost(p); }
    } freeHost{hostSc};
    const unsigned char *mask = solve_mask(c, constrainedFlag);
    cudaStream_t s = c.stream;
    MFEM_CUDA(cudaMemcpyAsync(vb, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    MFEM_CUDA(cudaMemcpyAsync(vx, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    MFEM_CUDA(cudaMemsetAsync(w + 7 * n, 0, 3 * sizeof(double), s));   // counter, maxima
    const double *P = c.prec.as<double>();
    // r = b - A x, z = P r, p = z (and max |p|), then the split of p at that
    // maximum, which becomes the scale the first iterations use
    spmv(c, vx, vq, mask, nullptr);
    if (D == 3) k_cg_init<3><<<nCtaNodes, kThreads, 0, s>>>(P, vb, vq, vr, vz, vp, link.nextMax, c.nbNodes, partial, nCtaNodes);
    else k_cg_init<1><<<nCtaNodes, kThreads, 0, s>>>(P, vb, vq, vr, vz, vp, link.nextMax, c.nbNodes, partial, nCtaNodes);
    check_launch("k_cg_init");
    if (ps.xs) {
        if (D == 3) k_split_x<3><<<blocks_for((long long)n, kThreads), kThreads, 0, s>>>(vp, ps.xs, (long long)n, link.nextMax, mask, nullptr);
        else k_split_x<1><<<blocks_for((long long)n, kThreads), kThreads, 0, s>>>(vp, ps.xs, (long long)n, link.nextMax, mask, nullptr);
        check_launch("k_split_x");
    }
    k_sum_partials<<<1, kThreads, 0, s>>>(partial, nCtaNodes, 3, sums, nullptr);
    k_cg_start<<<1, 1, 0, s>>>(sc, sums, rtol * rtol, maxIter, link);
    MFEM_CUDA(cudaMemcpyAsync(hostSc, sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s));
    MFEM_CUDA(cudaStreamSynchronize(s));
    // batches of iterations, three launches each (operator + alpha, update +
    // beta, direction); every kernel of an iteration after the one that met
    // the tolerance returns at once, so the iterate stays the converged one
    const int *stop = &sc->stop;
    const unsigned gDir = (unsigned)std::min<long long>(blocks_for((long long)n, kThreads), kMaxCtas);
    // the vector update: four CTAs per SM (measured at 100^3 against 2, 3, 8
    // per SM and 1,024 or 2,048 CTAs)
    int sms = 0;
    MFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    const int gUpd = std::max(1, std::min(nCtaNodes, 4 * sms));
    while (!hostSc->stop) {
        for (int k = 0; k < kCgBatch; k++) {
            spmv(c, vp, vq, mask, partial, stop, ps, link);     // q = A p; p . q; alpha
            if (D == 3) k_cg_update<3><<<gUpd, kThreads, 0, s>>>(P, sc, vp, vq, vx, vr, vz, c.nbNodes, partial, gUpd, link);
            else k_cg_update<1><<<gUpd, kThreads, 0, s>>>(P, sc, vp, vq, vx, vr, vz, c.nbNodes, partial, gUpd, link);
            if (D == 3) k_cg_direction<3><<<gDir, kThreads, 0, s>>>(sc, vz, vp, ps.xs, mask, (long long)n, link);
            else k_cg_direction<1><<<gDir, kThreads, 0, s>>>(sc, vz, vp, ps.xs, mask, (long long)n, link);
        }
        check_launch("k_cg iteration");
        MFEM_CUDA(cudaMemcpyAsync(hostSc, sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s));
        MFEM_CUDA(cudaStreamSynchronize(s));
    }
    MFEM_CUDA(cudaMemcpyAsync(x, vx, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    MFEM_CUDA(cudaStreamSynchronize(s));
    const double bnorm = sqrt(hostSc->bb);
    const double rel = bnorm > 0.0 ? sqrt(hostSc->rr) / bnorm : 0.0;
    const int it = hostSc->iter;
    if (iters) *iters = it;
    if (relres) *relres = rel;
}

}  // namespace mfem
