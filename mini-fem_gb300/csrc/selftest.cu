// Self-test of the integer-pipe double multiplication (dmul_int.cuh): compares
// dmul_bits with the FP64 unit's product on seeded operand pairs drawn from
// three families -- random bit patterns (every exponent, so the range checks
// are exercised), operands with exponents near 1.0, and operands with short
// significands (exact products and rounding ties).
#include "context.h"
#include "dmul_int.cuh"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_selftest_dmul(long long n, unsigned long long seed,
                                unsigned long long *counts) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long fast = 0, bad = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t A = mix64((uint64_t)i * 0x9E3779B97F4A7C15ull + seed);
        uint64_t B = mix64(A + 0x632BE59BD9B4E019ull);
        const int family = (int)(i % 3);
        if (family == 1) {
            A = (A & 0x800fffffffffffffull) | ((uint64_t)(973 + (A >> 20) % 100) << 52);
            B = (B & 0x800fffffffffffffull) | ((uint64_t)(973 + (B >> 20) % 100) << 52);
        } else if (family == 2) {
            const int ka = (int)(A % 27), kb = (int)(B % 27);
            A = (A & (0x800fffffffffffffull << ka) & ~0x7ff0000000000000ull) | (1000ull << 52);
            B = (B & (0x800fffffffffffffull << kb) & ~0x7ff0000000000000ull) | (1030ull << 52);
        }
        uint64_t r;
        if (mfem::dmul_bits(A, B, &r)) {
            fast++;
            const double ref = __dmul_rn(__longlong_as_double((long long)A),
                                         __longlong_as_double((long long)B));
            if (r != (uint64_t)__double_as_longlong(ref)) bad++;
        }
    }
    atomicAdd(counts, fast);
    atomicAdd(counts + 1, bad);
}

}  // namespace

extern "C" int mfem_selftest_dmul(mfem_context *ctx, long long n, unsigned long long seed,
                                  unsigned long long *fastPath, unsigned long long *mismatches) {
    if (!ctx) return MFEM_ERR_INVALID_ARG;
    mfem::Context &c = ctx->c;
    try {
        MFEM_REQUIRE(n >= 0 && fastPath && mismatches, MFEM_ERR_INVALID_ARG,
                     "n must be >= 0 and the outputs non-null");
        MFEM_CUDA(cudaSetDevice(c.device));
        mfem::DevBuf counts;
        unsigned long long *d = (unsigned long long *)counts.reserve(2 * sizeof(unsigned long long));
        MFEM_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), c.stream));
        k_selftest_dmul<<<152 * 8, 256, 0, c.stream>>>(n, seed, d);
        mfem::check_launch("k_selftest_dmul");
        unsigned long long h[2];
        MFEM_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
        *fastPath = h[0];
        *mismatches = h[1];
        c.lastError.clear();
        return MFEM_OK;
    } catch (const mfem::Error &e) {
        c.lastError = e.what();
        return e.code;
    }
}

// ---- FP64 pipe rate --------------------------------------------------------------
// The FP64 gather is bound by the FP64 pipe, whose rate the HBM and bf16
// figures of a roofline do not give.  Every thread advances 8 independent
// chains of FP64 additions (kind 0) or fused multiply-adds (kind 1) for `iters`
// steps; operations per second = threads * 8 * iters / elapsed.
namespace {

template <int KIND>
__global__ void __launch_bounds__(256) k_fp64_rate(int iters, double seed, double *sink) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = seed + (double)(threadIdx.x + k);
    const double b = 1.0000000001, c = 1e-300;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = KIND == 0 ? a[k] + c : fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += a[k];
    if (s == 12345.678) sink[0] = s;   // keeps the chains; never true in practice
}

}  // namespace

extern "C" int mfem_fp64_rate(mfem_context *ctx, int kind, double *opsPerSecond) {
    return mfem::run_guarded(ctx, [&](mfem::Context &c) {
        MFEM_REQUIRE((kind == 0 || kind == 1) && opsPerSecond, MFEM_ERR_INVALID_ARG,
                     "kind is 0 (add) or 1 (fma); non-null output");
        int sms = 0;
        MFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
        const int blocks = sms * 8, threads = 256, iters = 4096;
        mfem::DevBuf sink;
        double *d = (double *)sink.reserve(sizeof(double));
        cudaEvent_t e0, e1;
        MFEM_CUDA(cudaEventCreate(&e0));
        MFEM_CUDA(cudaEventCreate(&e1));
        float best = 0.f;
        for (int rep = 0; rep < 4; rep++) {   // the first launch warms up
            MFEM_CUDA(cudaEventRecord(e0, c.stream));
            if (kind == 0) k_fp64_rate<0><<<blocks, threads, 0, c.stream>>>(iters, 1.0, d);
            else k_fp64_rate<1><<<blocks, threads, 0, c.stream>>>(iters, 1.0, d);
            MFEM_CUDA(cudaEventRecord(e1, c.stream));
            MFEM_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            MFEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0 && (best == 0.f || ms < best)) best = ms;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        mfem::check_launch("k_fp64_rate");
        *opsPerSecond = (double)blocks * threads * 8.0 * iters / (best * 1e-3);
    });
}
