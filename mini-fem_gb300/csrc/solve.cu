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
// Reductions are deterministic: fixed grid, fixed tree order in each CTA, CTA
// partials summed by one CTA in index order.
#include <algorithm>
#include <cmath>

#include "context.h"
#include "elem32.cuh"

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
       const int *__restrict__ stop) {
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

// Scalars of the CG recurrence, kept on the device.
struct CgScalars {
    double rz, pq, alpha, beta, rr, bb, tol2;
    int iter, maxIter, stop;   // stop: converged or out of iterations; later kernels do nothing
};

// r = b - A x (A x already in q); z = P r; partials of r . z, r . r and b . b.
template <int D>
__global__ void __launch_bounds__(kThreads)
k_cg_init(const double *__restrict__ prec, const double *__restrict__ b, const double *__restrict__ q,
          double *__restrict__ r, double *__restrict__ z, double *__restrict__ p, int N,
          double *__restrict__ partial, int nCta) {
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
            rz = fma(rv[a], s, rz);
        }
    }
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

__global__ void k_cg_start(CgScalars *sc, const double *sums, double tol2, int maxIter) {
    sc->rz = sums[0];
    sc->rr = sums[1];
    sc->bb = sums[2];
    sc->tol2 = tol2;
    sc->iter = 0;
    sc->maxIter = maxIter;
    sc->stop = (sc->rr <= tol2 * sc->bb || maxIter <= 0) ? 1 : 0;
}

__global__ void k_cg_alpha(CgScalars *sc, const double *sums) {
    if (sc->stop) return;
    sc->pq = sums[0];
    sc->alpha = sc->pq != 0.0 ? sc->rz / sc->pq : 0.0;
}

// x += alpha p; r -= alpha q; z = P r; partials of r . z and r . r.
template <int D>
__global__ void __launch_bounds__(kThreads)
k_cg_update(const double *__restrict__ prec, const CgScalars *__restrict__ sc,
            const double *__restrict__ p, const double *__restrict__ q, double *__restrict__ x,
            double *__restrict__ r, double *__restrict__ z, int N, double *__restrict__ partial,
            int nCta) {
    if (sc->stop) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = sc->alpha;
    double rz = 0.0, rr = 0.0;
    if (i < N) {
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
}

__global__ void k_cg_beta(CgScalars *sc, const double *sums) {
    if (sc->stop) return;
    const double rzNew = sums[0];
    sc->beta = sc->rz != 0.0 ? rzNew / sc->rz : 0.0;
    sc->rz = rzNew;
    sc->rr = sums[1];
    sc->iter++;
    if (sc->rr <= sc->tol2 * sc->bb || sc->iter >= sc->maxIter) sc->stop = 1;
}

// p = z + beta p
__global__ void k_cg_direction(const CgScalars *__restrict__ sc, const double *__restrict__ z,
                               double *__restrict__ p, long long n) {
    if (sc->stop) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = fma(sc->beta, p[i], z[i]);
}

template <int D>
void spmv_t(const Context &c, const double *x, double *y, const unsigned char *mask, double *partial,
            const int *stop, cudaStream_t s) {
    const unsigned grid = blocks_for(c.nbNodes, kRowsPerCta);
    if (c.lastPrecision == MFEM_FP32)
        k_spmv<float, D><<<grid, kThreads, 0, s>>>(c.rowPtr.as<int>(), c.col.as<int>(), c.values.as<float>(),
                                                   x, y, c.nbNodes, mask, partial, stop);
    else
        k_spmv<double, D><<<grid, kThreads, 0, s>>>(c.rowPtr.as<int>(), c.col.as<int>(), c.values.as<double>(),
                                                    x, y, c.nbNodes, mask, partial, stop);
    check_launch("k_spmv");
}

void spmv(const Context &c, const double *x, double *y, const unsigned char *mask, double *partial,
          const int *stop = nullptr) {
    if (op_dim_of(c) == 9) spmv_t<3>(c, x, y, mask, partial, stop, c.stream);
    else spmv_t<1>(c, x, y, mask, partial, stop, c.stream);
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
    const int nCtaRows = (int)blocks_for(c.nbNodes, kRowsPerCta);
    const int nCtaNodes = (int)blocks_for(c.nbNodes, kThreads);
    const int nCta = std::max(nCtaRows, nCtaNodes);
    double *w = (double *)c.solver.reserve(sizeof(double) * (6 * n + 3 * (size_t)nCta + 8) + sizeof(CgScalars) + 64);
    double *vb = w, *vx = w + n, *vr = w + 2 * n, *vz = w + 3 * n, *vp = w + 4 * n, *vq = w + 5 * n;
    double *partial = w + 6 * n;
    double *sums = partial + 3 * (size_t)nCta;
    CgScalars *sc = reinterpret_cast<CgScalars *>(sums + 8);
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
    const double *P = c.prec.as<double>();
    // r = b - A x, z = P r, p = z
    spmv(c, vx, vq, mask, nullptr);
    if (D == 3) k_cg_init<3><<<nCtaNodes, kThreads, 0, s>>>(P, vb, vq, vr, vz, vp, c.nbNodes, partial, nCtaNodes);
    else k_cg_init<1><<<nCtaNodes, kThreads, 0, s>>>(P, vb, vq, vr, vz, vp, c.nbNodes, partial, nCtaNodes);
    check_launch("k_cg_init");
    k_sum_partials<<<1, kThreads, 0, s>>>(partial, nCtaNodes, 3, sums, nullptr);
    k_cg_start<<<1, 1, 0, s>>>(sc, sums, rtol * rtol, maxIter);
    MFEM_CUDA(cudaMemcpyAsync(hostSc, sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, s));
    MFEM_CUDA(cudaStreamSynchronize(s));
    // batches of iterations; every kernel of an iteration after the one that
    // met the tolerance returns at once, so the iterate stays the converged one
    const int *stop = &sc->stop;
    while (!hostSc->stop) {
        for (int k = 0; k < kCgBatch; k++) {
            spmv(c, vp, vq, mask, partial, stop);              // q = A p, partials of p . q
            k_sum_partials<<<1, kThreads, 0, s>>>(partial, nCtaRows, 1, sums, stop);
            k_cg_alpha<<<1, 1, 0, s>>>(sc, sums);
            if (D == 3) k_cg_update<3><<<nCtaNodes, kThreads, 0, s>>>(P, sc, vp, vq, vx, vr, vz, c.nbNodes, partial, nCtaNodes);
            else k_cg_update<1><<<nCtaNodes, kThreads, 0, s>>>(P, sc, vp, vq, vx, vr, vz, c.nbNodes, partial, nCtaNodes);
            k_sum_partials<<<1, kThreads, 0, s>>>(partial, nCtaNodes, 2, sums, stop);
            k_cg_beta<<<1, 1, 0, s>>>(sc, sums);
            k_cg_direction<<<blocks_for((long long)n, kThreads), kThreads, 0, s>>>(sc, vz, vp, (long long)n);
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
