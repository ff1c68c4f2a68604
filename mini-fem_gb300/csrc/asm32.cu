// FP32 assembly: element arithmetic and CSR values in FP32, every entry summed
// with Kahan compensation, FP64 kept for the coordinate differences (through a
// hi/lo float split of the coordinates) and for the 3x3 diagonal-block
// inversion; elements flagged as slivers by a quality test get double-float
// gradients (grad_df.cuh).
//
// Same structure as the FP64 gather (gradient records, then one thread per upper
// CSR entry and its transpose); records are 64 bytes (12 gradient floats + the
// weights).  The diagonal kernel writes the FP64 preconditioner directly from
// the compensated sum (prec_init + prec_inversion fused).
#include "context.h"
#include "elem_math.cuh"
#include "grad_df.cuh"

namespace mfem {

namespace {

constexpr int kThreads = 128;
constexpr int kRec32 = 16;

__global__ void k_split_coords(const double *__restrict__ coord, int nbNodes,
                               float4 *__restrict__ hi, float4 *__restrict__ lo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbNodes) return;
    const double x = coord[3 * i], y = coord[3 * i + 1], z = coord[3 * i + 2];
    float xh, yh, zh, xl, yl, zl;
    split_hilo(x, xh, xl);
    split_hilo(y, yh, yl);
    split_hilo(z, zh, zl);
    hi[i] = make_float4(xh, yh, zh, 0.f);
    lo[i] = make_float4(xl, yl, zl, 0.f);
}

// FP32 coefficients of the record kernel: kappa (lap) or (E, 1/2 - nu) (ela,
// the form lame32 takes; the subtraction in FP64).
__global__ void k_coef_to_f32(const double *__restrict__ in, long long n, int perElem,
                              float *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool nuSlot = perElem == 2 && (i & 1);
    out[i] = __double2float_rn(nuSlot ? 0.5 - in[i] : in[i]);
}

// a*b - c*d with one rounding error less than the plain expression (Kahan).
__device__ __forceinline__ float diff_prod(float a, float b, float c, float d) {
    const float w = c * d;
    const float e = fmaf(-c, d, w);
    const float f = fmaf(a, b, -w);
    return f + e;
}

template <int OP, bool COEF>
__global__ void __launch_bounds__(kThreads)
k_grad32(const float4 *__restrict__ hi, const float4 *__restrict__ lo,
         const double *__restrict__ coord, const int4 *__restrict__ e2n,
         const float *__restrict__ coef, int nbElem, float qthr2, float *__restrict__ rec,
         int *flagged) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbElem) return;
    const int4 nd = e2n[e];
    const float4 h0 = hi[nd.x], h1 = hi[nd.y], h2 = hi[nd.z], h3 = hi[nd.w];
    const float4 l0 = lo[nd.x], l1 = lo[nd.y], l2 = lo[nd.z], l3 = lo[nd.w];
    const float xa = (h0.x - h3.x) + (l0.x - l3.x), ya = (h0.y - h3.y) + (l0.y - l3.y),
                za = (h0.z - h3.z) + (l0.z - l3.z);
    const float xb = (h2.x - h3.x) + (l2.x - l3.x), yb = (h2.y - h3.y) + (l2.y - l3.y),
                zb = (h2.z - h3.z) + (l2.z - l3.z);
    const float xc = (h1.x - h3.x) + (l1.x - l3.x), yc = (h1.y - h3.y) + (l1.y - l3.y),
                zc = (h1.z - h3.z) + (l1.z - l3.z);
    float g[12];
    g[0] = diff_prod(yb, zc, yc, zb); g[1] = diff_prod(zb, xc, zc, xb); g[2] = diff_prod(xb, yc, xc, yb);
    g[3] = diff_prod(ya, zb, yb, za); g[4] = diff_prod(za, xb, zb, xa); g[5] = diff_prod(xa, yb, xb, ya);
    g[6] = diff_prod(yc, za, ya, zc); g[7] = diff_prod(zc, xa, za, xc); g[8] = diff_prod(xc, ya, xa, yc);
    const float vol = fmaf(xa, g[0], fmaf(ya, g[1], za * g[2]));
    // quality: |6V| / (|a| |b| |c|), squared
    const float na = fmaf(xa, xa, fmaf(ya, ya, za * za));
    const float nb = fmaf(xb, xb, fmaf(yb, yb, zb * zb));
    const float nc = fmaf(xc, xc, fmaf(yc, yc, zc * zc));
    float4 *out = reinterpret_cast<float4 *>(rec + (size_t)e * kRec32);
    if (vol * vol < qthr2 * (na * nb) * nc) {
        // sliver: double-float gradients from the same hi/lo coordinates
        // (grad_df.cuh); a zero volume takes the FP64 formula and its infinities
        atomicAdd(flagged, 1);
        const float hx[4][3] = {{h0.x, h0.y, h0.z}, {h1.x, h1.y, h1.z}, {h2.x, h2.y, h2.z}, {h3.x, h3.y, h3.z}};
        const float lx[4][3] = {{l0.x, l0.y, l0.z}, {l1.x, l1.y, l1.z}, {l2.x, l2.y, l2.z}, {l3.x, l3.y, l3.z}};
        if (!grad_df(hx, lx, g)) {
            double gd[12];
            elem_gradients(coord, nd, gd);
#pragma unroll
            for (int i = 0; i < 12; i++) g[i] = __double2float_rn(gd[i]);
        }
    } else {
        g[9] = -((g[0] + g[3]) + g[6]);
        g[10] = -((g[1] + g[4]) + g[7]);
        g[11] = -((g[2] + g[5]) + g[8]);
        const float r = 1.0f / vol;
#pragma unroll
        for (int i = 0; i < 12; i++) g[i] *= r;
    }
    out[0] = make_float4(g[0], g[1], g[2], g[3]);
    out[1] = make_float4(g[4], g[5], g[6], g[7]);
    out[2] = make_float4(g[8], g[9], g[10], g[11]);
    float A = 2.25f, B = 1.25f, mu = 1.0f;
    if (COEF) {
        if (OP == MFEM_OP_LAP) {
            A = coef[e];
        } else {
            const float2 w = lame32(coef[2 * (size_t)e], coef[2 * (size_t)e + 1]);
            B = w.x;
            mu = w.y;
            A = B + mu;
        }
    } else if (OP == MFEM_OP_LAP) {
        A = 1.0f;
    }
    out[3] = make_float4(A, B, mu, 0.f);
}

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

__device__ __forceinline__ void ldrec(const float *R, int j, float *g) {
    g[0] = R[3 * j];
    g[1] = R[3 * j + 1];
    g[2] = R[3 * j + 2];
}

template <int OP>
__global__ void __launch_bounds__(kThreads)
k_diag_units32(const int *__restrict__ diagPos, const int *__restrict__ start,
               const unsigned *__restrict__ contrib, const float *__restrict__ rec,
               int nbNodes, float *__restrict__ values, double *__restrict__ prec,
               const unsigned char *__restrict__ mask, int *singular) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    const int p = diagPos[r];
    if (OP == MFEM_OP_LAP) {
        Kahan acc;
        if (p >= 0) {
            for (int q = start[p]; q < start[p + 1]; q++) {
                const unsigned u = contrib[q];
                const float *R = rec + (size_t)(u >> 4) * kRec32;
                float g[3];
                ldrec(R, (u >> 2) & 3, g);
                acc.add(R[12] * fmaf(g[0], g[0], fmaf(g[1], g[1], g[2] * g[2])));
            }
            values[p] = acc.s - acc.c;
        }
        if (prec) prec[r] = 1.0 / ((double)acc.s - (double)acc.c);
        return;
    }
    Kahan acc[6];
    if (p >= 0) {
        for (int q = start[p]; q < start[p + 1]; q++) {
            const unsigned u = contrib[q];
            const float *R = rec + (size_t)(u >> 4) * kRec32;
            float g[3];
            ldrec(R, (u >> 2) & 3, g);
            const float A = R[12], B = R[13], mu = R[14];
            const float p00 = g[0] * g[0], p11 = g[1] * g[1], p22 = g[2] * g[2];
            acc[0].add(fmaf(p00, A, (p11 + p22) * mu));
            acc[1].add(fmaf(p11, A, (p00 + p22) * mu));
            acc[2].add(fmaf(p22, A, (p00 + p11) * mu));
            acc[3].add(g[0] * g[1] * B);
            acc[4].add(g[0] * g[2] * B);
            acc[5].add(g[1] * g[2] * B);
        }
        float *v = values + (size_t)p * 9;
        const float d0 = acc[0].s - acc[0].c, d4 = acc[1].s - acc[1].c, d8 = acc[2].s - acc[2].c;
        const float o1 = acc[3].s - acc[3].c, o2 = acc[4].s - acc[4].c, o5 = acc[5].s - acc[5].c;
        v[0] = d0; v[1] = o1; v[2] = o2;
        v[3] = o1; v[4] = d4; v[5] = o5;
        v[6] = o2; v[7] = o5; v[8] = d8;
    }
    if (prec) {
        double s[6];
#pragma unroll
        for (int m = 0; m < 6; m++) s[m] = (double)acc[m].s - (double)acc[m].c;
        double a[9] = {s[0], s[3], s[4], s[3], s[1], s[5], s[4], s[5], s[2]};
        if (mask) dirichlet_mask3(a, mask[r]);
        if (p >= 0 && lu_inverse3(a) != 0) atomicAdd(singular, 1);
        double *o = prec + (size_t)r * 9;
#pragma unroll
        for (int m = 0; m < 9; m++) o[m] = a[m];
    }
}

template <int OP>
__global__ void __launch_bounds__(kThreads)
k_edge_units32(const int2 *__restrict__ unitPos, int nUnits, const int *__restrict__ start,
               const unsigned *__restrict__ contrib, const float *__restrict__ rec,
               float *__restrict__ values) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nUnits) return;
    const int2 pp = unitPos[t];
    const int b = start[pp.x], en = start[pp.x + 1];
    if (OP == MFEM_OP_LAP) {
        Kahan acc;
        for (int q = b; q < en; q++) {
            const unsigned u = contrib[q];
            const float *R = rec + (size_t)(u >> 4) * kRec32;
            float gj[3], gk[3];
            ldrec(R, (u >> 2) & 3, gj);
            ldrec(R, u & 3, gk);
            acc.add(R[12] * fmaf(gj[0], gk[0], fmaf(gj[1], gk[1], gj[2] * gk[2])));
        }
        const float v = acc.s - acc.c;
        values[pp.x] = v;
        values[pp.y] = v;
        return;
    }
    Kahan acc[9];
    for (int q = b; q < en; q++) {
        const unsigned u = contrib[q];
        const float *R = rec + (size_t)(u >> 4) * kRec32;
        float gj[3], gk[3];
        ldrec(R, (u >> 2) & 3, gj);
        ldrec(R, u & 3, gk);
        const float A = R[12], B = R[13], mu = R[14];
        const float p00 = gj[0] * gk[0], p11 = gj[1] * gk[1], p22 = gj[2] * gk[2];
        acc[0].add(fmaf(p00, A, (p11 + p22) * mu));
        acc[4].add(fmaf(p11, A, (p00 + p22) * mu));
        acc[8].add(fmaf(p22, A, (p00 + p11) * mu));
        acc[1].add(gj[0] * gk[1] * B);
        acc[2].add(gj[0] * gk[2] * B);
        acc[3].add(gj[1] * gk[0] * B);
        acc[5].add(gj[1] * gk[2] * B);
        acc[6].add(gj[2] * gk[0] * B);
        acc[7].add(gj[2] * gk[1] * B);
    }
    float *v = values + (size_t)pp.x * 9;
    float *w = values + (size_t)pp.y * 9;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int bb = 0; bb < 3; bb++) {
            const float x = acc[3 * a + bb].s - acc[3 * a + bb].c;
            v[3 * a + bb] = x;
            w[3 * bb + a] = x;
        }
}

template <int OP, bool COEF>
void launch32(Context &c, bool fusePrec) {
    const GatherPlan &g = c.gather;
    const int E = c.nbElem, N = c.nbNodes;
    float4 *hi = (float4 *)c.scratch.reserve(sizeof(float4) * 2 * (size_t)N);
    float4 *lo = hi + N;
    c.timer.begin("split_coords", c.stream);
    k_split_coords<<<blocks_for(N, 256), 256, 0, c.stream>>>(c.coord.as<double>(), N, hi, lo);
    check_launch("k_split_coords");
    c.timer.end(c.stream);
    const float *coef = nullptr;
    if (COEF) {
        const long long n = (long long)E * (OP == MFEM_OP_LAP ? 1 : 2);
        float *cf = (float *)c.scratch2.reserve(sizeof(float) * n);
        c.timer.begin("coef_to_f32", c.stream);
        k_coef_to_f32<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.coef.as<double>(), n,
                                                                  OP == MFEM_OP_LAP ? 1 : 2, cf);
        check_launch("k_coef_to_f32");
        c.timer.end(c.stream);
        coef = cf;
    }
    float *rec = (float *)c.grad.reserve(sizeof(float) * kRec32 * (size_t)E);
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st + 4, 0, sizeof(int) * 2, c.stream));
    const float q = c.sliverThreshold;
    c.timer.begin("grad32", c.stream);
    k_grad32<OP, COEF><<<blocks_for(E, kThreads), kThreads, 0, c.stream>>>(
        hi, lo, c.coord.as<double>(), c.e2n.as<int4>(), coef, E, q * q, rec, st + 5);
    check_launch("k_grad32");
    c.timer.end(c.stream);
    c.flaggedPending = true;
    const int dim = OP == MFEM_OP_LAP ? 1 : 9;
    float *vals = c.values.as<float>();
    double *prec = fusePrec ? (double *)c.prec.reserve(sizeof(double) * (size_t)N * dim) : nullptr;
    const unsigned char *mask = c.hasMask ? c.mask.as<unsigned char>() : nullptr;
    c.timer.begin(fusePrec ? "diag_units32+prec" : "diag_units32", c.stream);
    k_diag_units32<OP><<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(
        c.diagPos.as<int>(), g.unitStart.as<int>(), g.contrib.as<unsigned>(), rec, N, vals, prec,
        mask, st + 4);
    check_launch("k_diag_units32");
    c.timer.end(c.stream);
    if (g.nUnits > 0) {
        c.timer.begin("edge_units32", c.stream);
        k_edge_units32<OP><<<blocks_for(g.nUnits, kThreads), kThreads, 0, c.stream>>>(
            g.unitPos.as<int2>(), g.nUnits, g.unitStart.as<int>(), g.contrib.as<unsigned>(), rec,
            vals);
        check_launch("k_edge_units32");
        c.timer.end(c.stream);
    }
}

}  // namespace

void assemble_fp32(Context &c, int op, int strategy, bool fusePrec) {
    MFEM_REQUIRE(strategy == MFEM_GATHER, MFEM_ERR_INVALID_ARG,
                 "FP32 assembly offers the gather strategy");
    if (c.fp32Kernel == 1) {
        build_tile_plan(c);
        if (!c.tiles.unfit) {
            assemble_tiles32(c, op, fusePrec);
            return;
        }
    }
    const bool coef = c.coefOp == op;
    const int dim = op == MFEM_OP_LAP ? 1 : 9;
    c.values.reserve(sizeof(float) * (size_t)c.nnz * dim);
    build_gather_plan(c);
    if (op == MFEM_OP_LAP) {
        if (coef) launch32<MFEM_OP_LAP, true>(c, fusePrec);
        else launch32<MFEM_OP_LAP, false>(c, fusePrec);
    } else {
        if (coef) launch32<MFEM_OP_ELA, true>(c, fusePrec);
        else launch32<MFEM_OP_ELA, false>(c, fusePrec);
    }
    c.lastOp = op;
    c.lastPrecision = MFEM_FP32;
    c.precIsInit = fusePrec;
}

}  // namespace mfem
