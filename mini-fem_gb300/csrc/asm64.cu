// FP64 assembly and preconditioner kernels (built with -fmad=false).
//
// Replaces assembly() (src/assembly.cc:615-720: reset + assembly_{lap,ela}_seq),
// prec_init (src/preconditioner.cc:52-87) and prec_inversion
// (src/preconditioner.cc:25-49 with src/Fortran/elasclpr.f).
//
// Strategies:
//  * GATHER (owner computes, deterministic): k_grad64 writes one 128-byte
//    gradient record per element; k_diag_units64 / k_edge_units64 then sum, for
//    every upper CSR entry, its element contributions in ascending element order
//    starting from 0.0 -- the reference REF build's summation order -- and write
//    the entry and its transpose.  Bit-exact with the reference under
//    -fmad=false.  The diagonal kernel can also fuse prec_init + prec_inversion.
//  * SCATTER (colour order, no atomics): the gradient records, then one launch
//    per colour; sixteen threads per element add its 16 blocks into the values
//    it owns within the colour.
//  * ATOMIC: one launch, one thread per element, FP64 atomic adds (summation
//    order not deterministic).
#include <cstdint>
#include <vector>

#include "context.h"
#include "elem_math.cuh"

namespace mfem {

namespace {

constexpr int kThreads = 128;

// Multiply splits (elem_math.cuh) of the FP64 kernels, chosen by timing the
// 5.8M-tet elasticity cube: the gradient kernel sends its cross products and
// 1/vol scalings to the integer pipes, the diagonal units their gradient products
// and diagonal weightings, the off-diagonal units their gradient products and B
// weightings (1009 -> 1626 M elem/s for the FP64 step, with the locality order).
constexpr int kSplitGrad = kIntCross | kIntScale;
constexpr int kSplitDiag = kIntGrad | kIntDiagW;
constexpr int kSplitEdge = kIntGrad | kIntOffW;

// Chunk j of a gradient record: g_j into g, the weight of its spare slot
// returned.  Records are 32-byte aligned and read-only in the kernels that read
// them (written by an earlier launch).
__device__ __forceinline__ double ld_chunk(const double *R, unsigned j, double g[3]) {
    double w;
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
        : "=d"(g[0]), "=d"(g[1]), "=d"(g[2]), "=d"(w)
        : "l"(R + 4 * j));
    return w;
}

// (A, B, mu) of an ela record given the chunks j and k already loaded: A is in
// chunks 0 and 3, B in 1, mu in 2; the others come from their slots.
__device__ __forceinline__ void ela_weights(const double *R, unsigned j, double wj, unsigned k,
                                            double wk, double &A, double &B, double &mu) {
    if (j == 0 || j == 3) A = wj;
    else if (k == 0 || k == 3) A = wk;
    else A = __ldg(R + 3);
    if (j == 1) B = wj;
    else if (k == 1) B = wk;
    else B = __ldg(R + 7);
    if (j == 2) mu = wj;
    else if (k == 2) mu = wk;
    else mu = __ldg(R + 11);
}

__device__ __forceinline__ void store_record(double *rec, int e, const double g[12], double w0,
                                             double w1, double w2, double w3) {
    double2 *out = reinterpret_cast<double2 *>(rec + (size_t)e * kRec64);
    out[0] = make_double2(g[0], g[1]);
    out[1] = make_double2(g[2], w0);
    out[2] = make_double2(g[3], g[4]);
    out[3] = make_double2(g[5], w1);
    out[4] = make_double2(g[6], g[7]);
    out[5] = make_double2(g[8], w2);
    out[6] = make_double2(g[9], g[10]);
    out[7] = make_double2(g[11], w3);
}

__device__ __forceinline__ double fix_zero(double x) {
    // 0.0 + x: identical to x except that -0.0 becomes +0.0 (integer pipe)
    const long long b = __double_as_longlong(x);
    return __longlong_as_double(b == (long long)0x8000000000000000ULL ? 0LL : b);
}

// (A, B, mu) of every element from (E, nu), for the gradient kernel to read
// instead of forming them (two correctly rounded divisions on the FP64 pipe)
// every step; made once per coefficient upload.
__global__ void __launch_bounds__(kThreads)
k_lame64(const double *__restrict__ coef, int nbElem, double *__restrict__ lame) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbElem) return;
    double A, B, mu;
    lame_weights(coef[2 * (size_t)e], coef[2 * (size_t)e + 1], A, B, mu);
    lame[3 * (size_t)e] = A;
    lame[3 * (size_t)e + 1] = B;
    lame[3 * (size_t)e + 2] = mu;
}

// CACHED (ela with coefficients): the weights come from k_lame64's array, the
// same bits as forming them here.
template <int OP, bool COEF, bool CACHED = false>
__global__ void __launch_bounds__(kThreads)
k_grad64(const double *__restrict__ coord, const int4 *__restrict__ e2n,
         const double *__restrict__ coef, int nbElem, double *__restrict__ rec,
         const double *__restrict__ lame = nullptr) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbElem) return;
    double g[12];
    elem_gradients<kSplitGrad>(coord, e2n[e], g);
    if (!COEF) {
        store_record(rec, e, g, 0.0, 0.0, 0.0, 0.0);
    } else if (OP == MFEM_OP_LAP) {
        const double kappa = coef[e];
        store_record(rec, e, g, kappa, kappa, kappa, kappa);
    } else {
        double A, B, mu;
        if (CACHED) {
            A = lame[3 * (size_t)e];
            B = lame[3 * (size_t)e + 1];
            mu = lame[3 * (size_t)e + 2];
        } else {
            lame_weights(coef[2 * (size_t)e], coef[2 * (size_t)e + 1], A, B, mu);
        }
        store_record(rec, e, g, A, B, mu, A);
    }
}

// Diagonal units: entry (r, r) = sum over incident elements (ascending) of
// block (j, j).  Optionally fused with prec_init + prec_inversion.
// 9 CTAs of 128 threads per SM (56 registers; measured 0.9 % faster than 8).
template <int OP, bool COEF, bool PREC>
__global__ void __launch_bounds__(kThreads, 9)
k_diag_units64(const int *__restrict__ diagNode, const int *__restrict__ diagPos,
               const int *__restrict__ start, const unsigned *__restrict__ contrib,
               const double *__restrict__ rec, int nbNodes, double *__restrict__ values,
               double *__restrict__ prec, const unsigned char *__restrict__ mask,
               int *singular) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nbNodes) return;
    const int r = diagNode[t];
    const int p = diagPos[r];
    if (OP == MFEM_OP_LAP) {
        double acc = 0.0;
        if (p >= 0) {
            const int b = start[p], en = start[p + 1];
            for (int q = b; q < en; q++) {
                const unsigned u = contrib[q];
                const double *R = rec + (size_t)(u >> 4) * kRec64;
                double g[3];
                const double kappa = ld_chunk(R, (u >> 2) & 3, g);
                const double v = lap_entry<!COEF, kSplitDiag>(g, g, kappa);
                acc = (q == b) ? fix_zero(v) : acc + v;
            }
            values[p] = acc;
        }
        if (PREC) prec[r] = 1.0 / acc;
        return;
    }
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (p >= 0) {
        const int b = start[p], en = start[p + 1];
        for (int q = b; q < en; q++) {
            const unsigned u = contrib[q];
            const double *R = rec + (size_t)(u >> 4) * kRec64;
            const unsigned j = (u >> 2) & 3;
            double g[3], d[6];
            const double wj = ld_chunk(R, j, g);
            double A = 0.0, B = 0.0, mu = 0.0;
            if (COEF) ela_weights(R, j, wj, j, wj, A, B, mu);
            ela_diag_block<!COEF, kSplitDiag>(g, A, B, mu, d);
            if (q == b) {
#pragma unroll
                for (int m = 0; m < 6; m++) acc[m] = fix_zero(d[m]);
            } else {
#pragma unroll
                for (int m = 0; m < 6; m++) acc[m] = acc[m] + d[m];
            }
        }
        double *v = values + (size_t)p * 9;
        v[0] = acc[0]; v[1] = acc[3]; v[2] = acc[4];
        v[3] = acc[3]; v[4] = acc[1]; v[5] = acc[5];
        v[6] = acc[4]; v[7] = acc[5]; v[8] = acc[2];
    }
    if (PREC) {
        double a[9] = {acc[0], acc[3], acc[4], acc[3], acc[1], acc[5], acc[4], acc[5], acc[2]};
        if (mask) dirichlet_mask3(a, mask[r]);
        if (p >= 0) {
            if (lu_inverse3(a) != 0) atomicAdd(singular, 1);
        }
        double *o = prec + (size_t)r * 9;
#pragma unroll
        for (int m = 0; m < 9; m++) o[m] = a[m];
    }
}

// Upper off-diagonal units: entry (r, c), c > r, and its transpose (c, r).
// 8 CTAs of 128 threads per SM (64 registers): more warps to keep the FP64
// pipe fed than the 7 the unbounded register count allows (measured 0.4 % faster).
template <int OP, bool COEF>
__global__ void __launch_bounds__(kThreads, 8)
k_edge_units64(const int2 *__restrict__ unitPos, int nUnits, const int *__restrict__ start,
               const unsigned *__restrict__ contrib, const double *__restrict__ rec,
               double *__restrict__ values) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nUnits) return;
    const int2 pp = unitPos[t];
    const int b = start[pp.x], en = start[pp.x + 1];
    if constexpr (OP == MFEM_OP_LAP) {
        double acc = 0.0;
        for (int q = b; q < en; q++) {
            const unsigned u = contrib[q];
            const double *R = rec + (size_t)(u >> 4) * kRec64;
            double gj[3], gk[3];
            const double kappa = ld_chunk(R, (u >> 2) & 3, gj);
            ld_chunk(R, u & 3, gk);
            const double v = lap_entry<!COEF, kSplitEdge>(gj, gk, kappa);
            acc = (q == b) ? fix_zero(v) : acc + v;
        }
        values[pp.x] = acc;
        values[pp.y] = acc;
    } else {
    double acc[9];
#pragma unroll
    for (int m = 0; m < 9; m++) acc[m] = 0.0;
    for (int q = b; q < en; q++) {
        const unsigned u = contrib[q];
        const double *R = rec + (size_t)(u >> 4) * kRec64;
        const unsigned j = (u >> 2) & 3, k = u & 3;
        double gj[3], gk[3], c[9];
        const double wj = ld_chunk(R, j, gj), wk = ld_chunk(R, k, gk);
        double A = 0.0, B = 0.0, mu = 0.0;
        if (COEF) ela_weights(R, j, wj, k, wk, A, B, mu);
        ela_block<!COEF, kSplitEdge>(gj, gk, A, B, mu, c);
        if (q == b) {
#pragma unroll
            for (int m = 0; m < 9; m++) acc[m] = fix_zero(c[m]);
        } else {
#pragma unroll
            for (int m = 0; m < 9; m++) acc[m] = acc[m] + c[m];
        }
    }
    double *v = values + (size_t)pp.x * 9;
    double *w = values + (size_t)pp.y * 9;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int bb = 0; bb < 3; bb++) {
            __stcs(v + 3 * a + bb, acc[3 * a + bb]);   // written once: evict first
            __stcs(w + 3 * bb + a, acc[3 * a + bb]);
        }
    }
}

// The weight fields of the gradient records (A, B, mu or kappa) for another
// coefficient set on the same mesh; the gradients stay.
template <int OP>
__global__ void __launch_bounds__(kThreads)
k_weights64(const double *__restrict__ coef, int nbElem, double *__restrict__ rec) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbElem) return;
    double *r = rec + (size_t)e * kRec64;
    if (OP == MFEM_OP_LAP) {
        const double kappa = coef[e];
        r[3] = kappa; r[7] = kappa; r[11] = kappa; r[15] = kappa;
    } else {
        double A, B, mu;
        lame_weights(coef[2 * (size_t)e], coef[2 * (size_t)e + 1], A, B, mu);
        r[3] = A; r[7] = B; r[11] = mu; r[15] = A;
    }
}

// ---- element-parallel strategies (scatter within a colour / atomics) ----------

// Sixteen threads per element, one per ordered node pair (j, k), reading the
// element's gradient record: block (k, j) computed on its own is bitwise the
// transpose of block (j, k) (every product commutes), so no pair waits for
// another.  Within a colour no two elements share a node, so the read-modify-
// writes never collide; colours run one launch after another.
template <int OP, bool COEF>
__global__ void __launch_bounds__(kThreads)
k_elem_scatter64(const int *__restrict__ elems, int count, const double *__restrict__ rec,
                 const int *__restrict__ elemPos, double *__restrict__ values) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long item = t >> 4;
    if (item >= count) return;
    const int jk = (int)(t & 15);
    const unsigned j = jk >> 2, k = jk & 3;
    const int e = elems[item];
    const double *r = rec + (size_t)e * kRec64;
    const int p = elemPos[(size_t)e * 16 + jk];
    double gj[3], gk[3];
    const double wj = ld_chunk(r, j, gj), wk = ld_chunk(r, k, gk);
    if (OP == MFEM_OP_LAP) {
        const double v = lap_entry<!COEF, kSplitEdge>(gj, gk, wj);
        values[p] = values[p] + v;
    } else {
        double A = 2.25, B = 1.25, mu = 1.0;
        if (COEF) ela_weights(r, j, wj, k, wk, A, B, mu);
        double c[9];
        ela_block<!COEF, kSplitEdge>(gj, gk, A, B, mu, c);
        double *v = values + (size_t)p * 9;
#pragma unroll
        for (int m = 0; m < 9; m++) v[m] = v[m] + c[m];
    }
}

// Atomic strategy: one thread per element, gradients in registers, its ten
// distinct blocks added with FP64 atomics (order not deterministic).
template <int OP, bool COEF>
__global__ void __launch_bounds__(kThreads)
k_elem_atomic64(const int *__restrict__ elems, int count, const double *__restrict__ coord,
                 const int4 *__restrict__ e2n, const double *__restrict__ coef,
                 const int *__restrict__ elemPos, double *__restrict__ values) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int e = elems ? elems[t] : t;
    double g[12];
    elem_gradients<kSplitGrad>(coord, e2n[e], g);
    double A = 2.25, B = 1.25, mu = 1.0, kappa = 1.0;
    if (COEF) {
        if (OP == MFEM_OP_LAP) kappa = coef[e];
        else lame_weights(coef[2 * (size_t)e], coef[2 * (size_t)e + 1], A, B, mu);
    }
    const int *pos = elemPos + (size_t)e * 16;
#pragma unroll
    for (int j = 0; j < 4; j++) {
#pragma unroll
        for (int k = j; k < 4; k++) {
            const int pjk = pos[4 * j + k], pkj = pos[4 * k + j];
            if (OP == MFEM_OP_LAP) {
                const double v = lap_entry<!COEF, kSplitEdge>(g + 3 * j, g + 3 * k, kappa);
                atomicAdd(values + pjk, v);
                if (k != j) atomicAdd(values + pkj, v);
            } else {
                double c[9];
                ela_block<!COEF, kSplitEdge>(g + 3 * j, g + 3 * k, A, B, mu, c);
                double *vj = values + (size_t)pjk * 9;
                double *vk = values + (size_t)pkj * 9;
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int bb = 0; bb < 3; bb++) {
                        const double x = c[3 * a + bb];
                        atomicAdd(vj + 3 * a + bb, x);
                        if (k != j) atomicAdd(vk + 3 * bb + a, x);
                    }
            }
        }
    }
}

// ---- preconditioner (separate calls) ------------------------------------------

__global__ void k_prec_init64(const double *__restrict__ values, const int *__restrict__ diagPos,
                              int nbNodes, int dim, double *__restrict__ prec) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nbNodes * dim) return;
    const int r = (int)(i / dim), k = (int)(i % dim);
    const int p = diagPos[r];
    prec[i] = p >= 0 ? values[(size_t)p * dim + k] : 0.0;
}

__global__ void k_prec_init32(const float *__restrict__ values, const int *__restrict__ diagPos,
                              int nbNodes, int dim, double *__restrict__ prec) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nbNodes * dim) return;
    const int r = (int)(i / dim), k = (int)(i % dim);
    const int p = diagPos[r];
    prec[i] = p >= 0 ? (double)values[(size_t)p * dim + k] : 0.0;
}

template <int OP>
__global__ void k_prec_invert(double *__restrict__ prec, const int *__restrict__ diagPos,
                              const unsigned char *__restrict__ mask, int nbNodes,
                              int *singular) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    if (OP == MFEM_OP_LAP) {
        prec[r] = 1.0 / prec[r];
        return;
    }
    double a[9];
    double *P = prec + (size_t)r * 9;
#pragma unroll
    for (int m = 0; m < 9; m++) a[m] = P[m];
    if (mask) dirichlet_mask3(a, mask[r]);
    if (diagPos[r] >= 0) {
        if (lu_inverse3(a) != 0) atomicAdd(singular, 1);
    }
#pragma unroll
    for (int m = 0; m < 9; m++) P[m] = a[m];
}

template <int OP, bool COEF>
void launch_gather(Context &c, bool fusePrec) {
    const GatherPlan &g = c.gather;
    const int E = c.nbElem, N = c.nbNodes;
    double *rec = (double *)c.grad.reserve(sizeof(double) * kRec64 * (size_t)E);
    if constexpr (OP == MFEM_OP_ELA && COEF) {
        if (!c.lameValid) {
            double *lame = (double *)c.lame.reserve(sizeof(double) * 3 * (size_t)E);
            k_lame64<<<blocks_for(E, kThreads), kThreads, 0, c.stream>>>(c.coef.as<double>(), E, lame);
            check_launch("k_lame64");
            c.lameValid = true;
        }
        c.timer.begin("grad64", c.stream);
        k_grad64<OP, COEF, true><<<blocks_for(E, kThreads), kThreads, 0, c.stream>>>(
            c.coord.as<double>(), c.e2n.as<int4>(), c.coef.as<double>(), E, rec, c.lame.as<double>());
    } else {
        c.timer.begin("grad64", c.stream);
        k_grad64<OP, COEF><<<blocks_for(E, kThreads), kThreads, 0, c.stream>>>(
            c.coord.as<double>(), c.e2n.as<int4>(), c.coef.as<double>(), E, rec);
    }
    check_launch("k_grad64");
    c.timer.end(c.stream);
    const int dim = OP == MFEM_OP_LAP ? 1 : 9;
    double *vals = c.values.as<double>();
    double *prec = fusePrec ? (double *)c.prec.reserve(sizeof(double) * (size_t)N * dim) : nullptr;
    const unsigned char *mask = c.hasMask ? c.mask.as<unsigned char>() : nullptr;
    int *sing = status_ptr(c) + 4;
    if (fusePrec) MFEM_CUDA(cudaMemsetAsync(sing, 0, sizeof(int), c.stream));
    // The diagonal and off-diagonal units read the same records and write
    // disjoint entries: they run concurrently, the diagonal ones on the side
    // stream, so that each fills the FP64 pipe where the other leaves gaps
    // (3.307 -> 3.274 ms a step at 100^3).  Per-kernel timing (mfem_profile)
    // runs them one after the other.
    const bool concurrent = !c.timer.on && g.nUnits > 0;
    cudaStream_t ds = c.stream;
    if (concurrent) {
        if (!c.side) {
            MFEM_CUDA(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
            MFEM_CUDA(cudaEventCreateWithFlags(&c.sideFork, cudaEventDisableTiming));
            MFEM_CUDA(cudaEventCreateWithFlags(&c.sideJoin, cudaEventDisableTiming));
        }
        MFEM_CUDA(cudaEventRecord(c.sideFork, c.stream));
        MFEM_CUDA(cudaStreamWaitEvent(c.side, c.sideFork, 0));
        ds = c.side;
    }
    c.timer.begin(fusePrec ? "diag_units64+prec" : "diag_units64", c.stream);
    if (fusePrec)
        k_diag_units64<OP, COEF, true><<<blocks_for(N, kThreads), kThreads, 0, ds>>>(
            g.diagNode.as<int>(), c.diagPos.as<int>(), g.unitStart.as<int>(),
            g.contrib.as<unsigned>(), rec, N, vals, prec, mask, sing);
    else
        k_diag_units64<OP, COEF, false><<<blocks_for(N, kThreads), kThreads, 0, ds>>>(
            g.diagNode.as<int>(), c.diagPos.as<int>(), g.unitStart.as<int>(),
            g.contrib.as<unsigned>(), rec, N, vals, prec, mask, sing);
    check_launch("k_diag_units64");
    c.timer.end(c.stream);
    if (g.nUnits > 0) {
        c.timer.begin("edge_units64", c.stream);
        k_edge_units64<OP, COEF><<<blocks_for(g.nUnits, kThreads), kThreads, 0, c.stream>>>(
            g.unitPos.as<int2>(), g.nUnits, g.unitStart.as<int>(), g.contrib.as<unsigned>(), rec,
            vals);
        check_launch("k_edge_units64");
        c.timer.end(c.stream);
    }
    if (concurrent) {
        MFEM_CUDA(cudaEventRecord(c.sideJoin, c.side));
        MFEM_CUDA(cudaStreamWaitEvent(c.stream, c.sideJoin, 0));
    }
}

template <int OP, bool COEF>
void launch_elementwise(Context &c, bool atomic) {
    const int dim = OP == MFEM_OP_LAP ? 1 : 9;
    const int E = c.nbElem;
    double *vals = c.values.as<double>();
    c.timer.begin(atomic ? "atomic64" : "scatter64", c.stream);
    MFEM_CUDA(cudaMemsetAsync(vals, 0, sizeof(double) * (size_t)c.nnz * dim, c.stream));
    if (atomic) {
        k_elem_atomic64<OP, COEF><<<blocks_for(E, kThreads), kThreads, 0, c.stream>>>(
            nullptr, E, c.coord.as<double>(), c.e2n.as<int4>(), c.coef.as<double>(),
            c.elemPos.as<int>(), vals);
        check_launch("k_elem_atomic64");
        c.timer.end(c.stream);
        return;
    }
    double *rec = (double *)c.grad.reserve(sizeof(double) * kRec64 * (size_t)E);
    const Coloring &col = c.coloring;
    // the record pass and the colour loop as one CUDA graph: on small meshes a
    // launch per colour costs more than the colour's work
    std::vector<long long> key = {OP, COEF, (long long)(uintptr_t)rec, (long long)(uintptr_t)vals,
                                  (long long)(uintptr_t)c.elemPos.ptr, (long long)(uintptr_t)col.colorElems.ptr,
                                  (long long)(uintptr_t)c.coord.ptr, (long long)(uintptr_t)c.e2n.ptr,
                                  (long long)(uintptr_t)c.coef.ptr, E};
    key.insert(key.end(), col.hOffsets.begin(), col.hOffsets.end());
    CachedGraph &cg = c.scatterGraph;
    if (!cg.exec || cg.key != key) {
        if (cg.exec) {
            MFEM_CUDA(cudaGraphExecDestroy(cg.exec));
            cg.exec = nullptr;
        }
        cudaGraph_t graph;
        MFEM_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        k_grad64<OP, COEF><<<blocks_for(E, kThreads), kThreads, 0, c.stream>>>(
            c.coord.as<double>(), c.e2n.as<int4>(), c.coef.as<double>(), E, rec);
        for (int k = 0; k < col.nbColors; k++) {
            const int b = col.hOffsets[k], n = col.hOffsets[k + 1] - b;
            if (n <= 0) continue;
            k_elem_scatter64<OP, COEF><<<blocks_for(16LL * n, kThreads), kThreads, 0, c.stream>>>(
                col.colorElems.as<int>() + b, n, rec, c.elemPos.as<int>(), vals);
        }
        const cudaError_t launchErr = cudaGetLastError();
        MFEM_CUDA(cudaStreamEndCapture(c.stream, &graph));
        MFEM_CUDA(launchErr);
        const cudaError_t instErr = cudaGraphInstantiate(&cg.exec, graph, 0);
        cudaGraphDestroy(graph);
        MFEM_CUDA(instErr);
        cg.key.swap(key);
    }
    MFEM_CUDA(cudaGraphLaunch(cg.exec, c.stream));
    c.timer.end(c.stream);
}

}  // namespace

void assemble_fp64(Context &c, int op, int strategy, bool fusePrec) {
    const bool coef = c.coefOp == op;
    const int dim = op == MFEM_OP_LAP ? 1 : 9;
    c.values.reserve(sizeof(double) * (size_t)c.nnz * dim);
    if (strategy == MFEM_GATHER) {
        build_gather_plan(c);
        if (op == MFEM_OP_LAP) {
            if (coef) launch_gather<MFEM_OP_LAP, true>(c, fusePrec);
            else launch_gather<MFEM_OP_LAP, false>(c, fusePrec);
        } else {
            if (coef) launch_gather<MFEM_OP_ELA, true>(c, fusePrec);
            else launch_gather<MFEM_OP_ELA, false>(c, fusePrec);
        }
    } else {
        build_elem_pos(c);
        const bool atomic = strategy == MFEM_ATOMIC;
        MFEM_REQUIRE(atomic || c.coloring.built, MFEM_ERR_STATE,
                     "scatter strategy needs mfem_coloring_creation first");
        if (op == MFEM_OP_LAP) {
            if (coef) launch_elementwise<MFEM_OP_LAP, true>(c, atomic);
            else launch_elementwise<MFEM_OP_LAP, false>(c, atomic);
        } else {
            if (coef) launch_elementwise<MFEM_OP_ELA, true>(c, atomic);
            else launch_elementwise<MFEM_OP_ELA, false>(c, atomic);
        }
    }
    c.lastOp = op;
    c.lastPrecision = MFEM_FP64;
    c.precIsInit = fusePrec && strategy == MFEM_GATHER;
}

// FP64 gather on caller-provided buffers: coordinates, coefficients (NULL: the
// reference constants), gradient-record scratch (16 doubles per element) and
// values.  Uses the context's topology and gather plan, which must exist;
// launches on `s` and allocates nothing.
void gather_fp64_into(const Context &c, int op, const double *coord, const double *coef,
                      double *rec, double *values, cudaStream_t s) {
    const GatherPlan &g = c.gather;
    const int E = c.nbElem, N = c.nbNodes;
    const int *dp = c.diagPos.as<int>(), *st = g.unitStart.as<int>(), *dn = g.diagNode.as<int>();
    const unsigned *ct = g.contrib.as<unsigned>();
    const int2 *up = g.unitPos.as<int2>();
    const int4 *e2n = c.e2n.as<int4>();
    if (op == MFEM_OP_LAP) {
        if (coef) {
            k_grad64<MFEM_OP_LAP, true><<<blocks_for(E, kThreads), kThreads, 0, s>>>(coord, e2n, coef, E, rec);
            k_diag_units64<MFEM_OP_LAP, true, false><<<blocks_for(N, kThreads), kThreads, 0, s>>>(dn, dp, st, ct, rec, N, values, nullptr, nullptr, nullptr);
            if (g.nUnits > 0)
                k_edge_units64<MFEM_OP_LAP, true><<<blocks_for(g.nUnits, kThreads), kThreads, 0, s>>>(up, g.nUnits, st, ct, rec, values);
        } else {
            k_grad64<MFEM_OP_LAP, false><<<blocks_for(E, kThreads), kThreads, 0, s>>>(coord, e2n, nullptr, E, rec);
            k_diag_units64<MFEM_OP_LAP, false, false><<<blocks_for(N, kThreads), kThreads, 0, s>>>(dn, dp, st, ct, rec, N, values, nullptr, nullptr, nullptr);
            if (g.nUnits > 0)
                k_edge_units64<MFEM_OP_LAP, false><<<blocks_for(g.nUnits, kThreads), kThreads, 0, s>>>(up, g.nUnits, st, ct, rec, values);
        }
    } else {
        if (coef) {
            k_grad64<MFEM_OP_ELA, true><<<blocks_for(E, kThreads), kThreads, 0, s>>>(coord, e2n, coef, E, rec);
            k_diag_units64<MFEM_OP_ELA, true, false><<<blocks_for(N, kThreads), kThreads, 0, s>>>(dn, dp, st, ct, rec, N, values, nullptr, nullptr, nullptr);
            if (g.nUnits > 0)
                k_edge_units64<MFEM_OP_ELA, true><<<blocks_for(g.nUnits, kThreads), kThreads, 0, s>>>(up, g.nUnits, st, ct, rec, values);
        } else {
            k_grad64<MFEM_OP_ELA, false><<<blocks_for(E, kThreads), kThreads, 0, s>>>(coord, e2n, nullptr, E, rec);
            k_diag_units64<MFEM_OP_ELA, false, false><<<blocks_for(N, kThreads), kThreads, 0, s>>>(dn, dp, st, ct, rec, N, values, nullptr, nullptr, nullptr);
            if (g.nUnits > 0)
                k_edge_units64<MFEM_OP_ELA, false><<<blocks_for(g.nUnits, kThreads), kThreads, 0, s>>>(up, g.nUnits, st, ct, rec, values);
        }
    }
    check_launch("gather_fp64_into");
}

// FP64 gather of one coefficient set into caller-chosen buffers, with the fused
// preconditioner when prec != NULL (batched assembly; same kernels and results
// as assemble_fp64 with the gather strategy).
void gather_fp64_sets(const Context &c, int op, const double *coef, double *rec, double *values,
                      double *prec, const unsigned char *mask, int *singular, cudaStream_t s,
                      bool gradientsReady) {
    const GatherPlan &g = c.gather;
    const int E = c.nbElem, N = c.nbNodes;
    const int *dp = c.diagPos.as<int>(), *st = g.unitStart.as<int>(), *dn = g.diagNode.as<int>();
    const unsigned *ct = g.contrib.as<unsigned>();
    const int2 *up = g.unitPos.as<int2>();
    const int4 *e2n = c.e2n.as<int4>();
    const double *coord = c.coord.as<double>();
    auto run = [&](auto grad, auto diag, auto diagp, auto edge) {
        // the records' gradients depend on the mesh only: after the first set
        // of a mesh only the weights are rewritten (none at all for constants)
        if (!gradientsReady) {
            grad<<<blocks_for(E, kThreads), kThreads, 0, s>>>(coord, e2n, coef, E, rec, nullptr);
        } else if (coef) {
            if (op == MFEM_OP_LAP) k_weights64<MFEM_OP_LAP><<<blocks_for(E, kThreads), kThreads, 0, s>>>(coef, E, rec);
            else k_weights64<MFEM_OP_ELA><<<blocks_for(E, kThreads), kThreads, 0, s>>>(coef, E, rec);
        }
        if (prec)
            diagp<<<blocks_for(N, kThreads), kThreads, 0, s>>>(dn, dp, st, ct, rec, N, values, prec, mask, singular);
        else
            diag<<<blocks_for(N, kThreads), kThreads, 0, s>>>(dn, dp, st, ct, rec, N, values, nullptr, nullptr, nullptr);
        if (g.nUnits > 0)
            edge<<<blocks_for(g.nUnits, kThreads), kThreads, 0, s>>>(up, g.nUnits, st, ct, rec, values);
    };
    if (op == MFEM_OP_LAP) {
        if (coef) run(k_grad64<MFEM_OP_LAP, true>, k_diag_units64<MFEM_OP_LAP, true, false>,
                      k_diag_units64<MFEM_OP_LAP, true, true>, k_edge_units64<MFEM_OP_LAP, true>);
        else run(k_grad64<MFEM_OP_LAP, false>, k_diag_units64<MFEM_OP_LAP, false, false>,
                 k_diag_units64<MFEM_OP_LAP, false, true>, k_edge_units64<MFEM_OP_LAP, false>);
    } else {
        if (coef) run(k_grad64<MFEM_OP_ELA, true>, k_diag_units64<MFEM_OP_ELA, true, false>,
                      k_diag_units64<MFEM_OP_ELA, true, true>, k_edge_units64<MFEM_OP_ELA, true>);
        else run(k_grad64<MFEM_OP_ELA, false>, k_diag_units64<MFEM_OP_ELA, false, false>,
                 k_diag_units64<MFEM_OP_ELA, false, true>, k_edge_units64<MFEM_OP_ELA, false>);
    }
    check_launch("gather_fp64_sets");
}

void prec_init_fp64(Context &c, int op) {
    const int dim = op == MFEM_OP_LAP ? 1 : 9;
    double *prec = (double *)c.prec.reserve(sizeof(double) * (size_t)c.nbNodes * dim);
    const long long n = (long long)c.nbNodes * dim;
    c.timer.begin("prec_init", c.stream);
    if (c.lastPrecision == MFEM_FP64)
        k_prec_init64<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.values.as<double>(),
                                                                c.diagPos.as<int>(), c.nbNodes, dim, prec);
    else
        k_prec_init32<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.values.as<float>(),
                                                                c.diagPos.as<int>(), c.nbNodes, dim, prec);
    check_launch("k_prec_init");
    c.timer.end(c.stream);
}

int prec_invert(Context &c, int op) {
    int *sing = status_ptr(c) + 4;
    MFEM_CUDA(cudaMemsetAsync(sing, 0, sizeof(int), c.stream));
    const unsigned char *mask = c.hasMask ? c.mask.as<unsigned char>() : nullptr;
    c.timer.begin("prec_invert", c.stream);
    if (op == MFEM_OP_LAP)
        k_prec_invert<MFEM_OP_LAP><<<blocks_for(c.nbNodes, kThreads), kThreads, 0, c.stream>>>(
            c.prec.as<double>(), c.diagPos.as<int>(), mask, c.nbNodes, sing);
    else
        k_prec_invert<MFEM_OP_ELA><<<blocks_for(c.nbNodes, kThreads), kThreads, 0, c.stream>>>(
            c.prec.as<double>(), c.diagPos.as<int>(), mask, c.nbNodes, sing);
    check_launch("k_prec_invert");
    c.timer.end(c.stream);
    int h[5];
    read_status(c, h, 5);
    return h[4];
}

}  // namespace mfem
