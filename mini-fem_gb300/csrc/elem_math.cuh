// Per-element arithmetic of the FP64 path, in the reference's exact expression
// order (this header is only included by translation units built with
// -fmad=false, so no product/sum pair is contracted into an FMA).
#pragma once

#include <cuda_runtime.h>

#include "dmul_int.cuh"

namespace mfem {

// Multiply split: which products of a formula go to the integer pipes
// (dmul_ipipe) and which to the FP64 unit.  Both give the same bits, so a split
// only balances the two pipes; each kernel picks its own (a template argument).
enum : int {
    kIntGrad = 1,    // g_j[a] * g_k[b] in the blocks
    kIntDiagA = 2,   // p_aa * A
    kIntOffW = 4,    // p_ab * B
    kIntCross = 8,   // cross products of the edge vectors
    kIntScale = 16,  // gradients times 1/vol
    kIntDiagMu = 32, // p_aa * mu
    kIntDiagW = kIntDiagA | kIntDiagMu,
};

template <bool INT>
__device__ __forceinline__ double dmul(double a, double b) {
    if constexpr (INT) return dmul_ipipe(a, b);
    else return a * b;
}

// Per-element gradient record, 16 doubles = 128 bytes in four 32-byte chunks
// (g_j.x, g_j.y, g_j.z, w_j), so that one 256-bit load brings a gradient and a
// weight.  The weights sit in the spare slots: ela w = (A, B, mu, A), lap
// w = (kappa, kappa, kappa, kappa).
constexpr int kRec64 = 16;

__device__ __forceinline__ double neg(double x) {
    // sign flip on the integer pipe (exact, like the unary minus of the reference)
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}

// assembly.cc:85-121 elem_coef_seq: gradients of the barycentric coordinates
// scaled by the reciprocal of the signed 6*volume.  Note the reference's b/c
// order: xb = n2 - n3, xc = n1 - n3.
template <int SPLIT = 0>
__device__ __forceinline__ void elem_gradients(const double *__restrict__ coord, int4 nd,
                                               double g[12]) {
    const double x0 = coord[3 * nd.x], y0 = coord[3 * nd.x + 1], z0 = coord[3 * nd.x + 2];
    const double x1 = coord[3 * nd.y], y1 = coord[3 * nd.y + 1], z1 = coord[3 * nd.y + 2];
    const double x2 = coord[3 * nd.z], y2 = coord[3 * nd.z + 1], z2 = coord[3 * nd.z + 2];
    const double x3 = coord[3 * nd.w], y3 = coord[3 * nd.w + 1], z3 = coord[3 * nd.w + 2];
    const double xa = x0 - x3, xb = x2 - x3, xc = x1 - x3;
    const double ya = y0 - y3, yb = y2 - y3, yc = y1 - y3;
    const double za = z0 - z3, zb = z2 - z3, zc = z1 - z3;
    constexpr bool X = (SPLIT & kIntCross) != 0;
    const double g00 = dmul<X>(yb, zc) - dmul<X>(yc, zb), g01 = dmul<X>(zb, xc) - dmul<X>(zc, xb),
                 g02 = dmul<X>(xb, yc) - dmul<X>(xc, yb);
    const double g10 = dmul<X>(ya, zb) - dmul<X>(yb, za), g11 = dmul<X>(za, xb) - dmul<X>(zb, xa),
                 g12 = dmul<X>(xa, yb) - dmul<X>(xb, ya);
    const double g20 = dmul<X>(yc, za) - dmul<X>(ya, zc), g21 = dmul<X>(zc, xa) - dmul<X>(za, xc),
                 g22 = dmul<X>(xc, ya) - dmul<X>(xa, yc);
    const double g30 = neg((g00 + g10) + g20);
    const double g31 = neg((g01 + g11) + g21);
    const double g32 = neg((g02 + g12) + g22);
    const double vol = (xa * g00 + ya * g01) + za * g02;
    const double r = 1.0 / vol;
    constexpr bool S = (SPLIT & kIntScale) != 0;
    g[0] = dmul<S>(g00, r); g[1] = dmul<S>(g01, r); g[2] = dmul<S>(g02, r);
    g[3] = dmul<S>(g10, r); g[4] = dmul<S>(g11, r); g[5] = dmul<S>(g12, r);
    g[6] = dmul<S>(g20, r); g[7] = dmul<S>(g21, r); g[8] = dmul<S>(g22, r);
    g[9] = dmul<S>(g30, r); g[10] = dmul<S>(g31, r); g[11] = dmul<S>(g32, r);
}

// Lame weights from Young's modulus and Poisson ratio; A = lambda + 2 mu,
// B = lambda + mu.  At (A, B, mu) = (2.25, 1.25, 1) the block formulas below are
// the reference's (assembly.cc:423-446) bit for bit.
__device__ __forceinline__ void lame_weights(double E, double nu, double &A, double &B,
                                             double &mu) {
    const double lam = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
    mu = E / (2.0 * (1.0 + nu));
    A = lam + 2.0 * mu;
    B = lam + mu;
}

// The 3x3 block (j,k) of the elasticity element matrix, row-major c[3a+b]:
//   c(a,a) = ((p00*w0 + p11*w1) + p22*w2) with w = A on the a-th term, mu else
//   c(a,b) = p_ab * B
// (assembly.cc:423-446; the reference's constants are A = 2.25, B = 1.25, mu = 1).
template <bool REFW, int SPLIT = 0>
__device__ __forceinline__ void ela_block(const double *gj, const double *gk, double A,
                                          double B, double mu, double c[9]) {
    constexpr bool G = (SPLIT & kIntGrad) != 0, W = (SPLIT & kIntDiagA) != 0,
                   M = (SPLIT & kIntDiagMu) != 0, O = (SPLIT & kIntOffW) != 0;
    const double p00 = dmul<G>(gj[0], gk[0]), p11 = dmul<G>(gj[1], gk[1]),
                 p22 = dmul<G>(gj[2], gk[2]);
    const double p01 = dmul<G>(gj[0], gk[1]), p02 = dmul<G>(gj[0], gk[2]),
                 p10 = dmul<G>(gj[1], gk[0]), p12 = dmul<G>(gj[1], gk[2]),
                 p20 = dmul<G>(gj[2], gk[0]), p21 = dmul<G>(gj[2], gk[1]);
    if (REFW) {
        c[0] = (dmul<W>(p00, 2.25) + p11) + p22;
        c[4] = (p00 + dmul<W>(p11, 2.25)) + p22;
        c[8] = (p00 + p11) + dmul<W>(p22, 2.25);
        c[1] = dmul<O>(p01, 1.25);
        c[2] = dmul<O>(p02, 1.25);
        c[3] = dmul<O>(p10, 1.25);
        c[5] = dmul<O>(p12, 1.25);
        c[6] = dmul<O>(p20, 1.25);
        c[7] = dmul<O>(p21, 1.25);
    } else {
        c[0] = (dmul<W>(p00, A) + dmul<M>(p11, mu)) + dmul<M>(p22, mu);
        c[4] = (dmul<M>(p00, mu) + dmul<W>(p11, A)) + dmul<M>(p22, mu);
        c[8] = (dmul<M>(p00, mu) + dmul<M>(p11, mu)) + dmul<W>(p22, A);
        c[1] = dmul<O>(p01, B);
        c[2] = dmul<O>(p02, B);
        c[3] = dmul<O>(p10, B);
        c[5] = dmul<O>(p12, B);
        c[6] = dmul<O>(p20, B);
        c[7] = dmul<O>(p21, B);
    }
}

// Diagonal block (j,j): symmetric bit for bit, six distinct values
// (c0, c4, c8, c1 = c3, c2 = c6, c5 = c7).
template <bool REFW, int SPLIT = 0>
__device__ __forceinline__ void ela_diag_block(const double *g, double A, double B,
                                               double mu, double d[6]) {
    constexpr bool G = (SPLIT & kIntGrad) != 0, W = (SPLIT & kIntDiagA) != 0,
                   M = (SPLIT & kIntDiagMu) != 0, O = (SPLIT & kIntOffW) != 0;
    const double p00 = dmul<G>(g[0], g[0]), p11 = dmul<G>(g[1], g[1]), p22 = dmul<G>(g[2], g[2]);
    const double p01 = dmul<G>(g[0], g[1]), p02 = dmul<G>(g[0], g[2]), p12 = dmul<G>(g[1], g[2]);
    if (REFW) {
        d[0] = (dmul<W>(p00, 2.25) + p11) + p22;
        d[1] = (p00 + dmul<W>(p11, 2.25)) + p22;
        d[2] = (p00 + p11) + dmul<W>(p22, 2.25);
        d[3] = dmul<O>(p01, 1.25);
        d[4] = dmul<O>(p02, 1.25);
        d[5] = dmul<O>(p12, 1.25);
    } else {
        d[0] = (dmul<W>(p00, A) + dmul<M>(p11, mu)) + dmul<M>(p22, mu);
        d[1] = (dmul<M>(p00, mu) + dmul<W>(p11, A)) + dmul<M>(p22, mu);
        d[2] = (dmul<M>(p00, mu) + dmul<M>(p11, mu)) + dmul<W>(p22, A);
        d[3] = dmul<O>(p01, B);
        d[4] = dmul<O>(p02, B);
        d[5] = dmul<O>(p12, B);
    }
}

// assembly.cc:555-557: (gj0*gk0 + gj1*gk1) + gj2*gk2, weighted by kappa.
template <bool REFW, int SPLIT = 0>
__device__ __forceinline__ double lap_entry(const double *gj, const double *gk, double kappa) {
    constexpr bool G = (SPLIT & kIntGrad) != 0, W = (SPLIT & kIntDiagA) != 0;
    const double s = (dmul<G>(gj[0], gk[0]) + dmul<G>(gj[1], gk[1])) + dmul<G>(gj[2], gk[2]);
    return REFW ? s : dmul<W>(kappa, s);
}

// hi + lo split of a coordinate: hi = fl32(x), lo = fl32(x - hi), on the
// integer pipes (split_f32_bits) except for zero and extreme magnitudes.
__device__ __forceinline__ void split_hilo(double x, float &h, float &l) {
    uint32_t hb, lb;
    if (split_f32_bits((uint64_t)__double_as_longlong(x), &hb, &lb)) {
        h = __uint_as_float(hb);
        l = __uint_as_float(lb);
    } else {
        h = __double2float_rn(x);
        l = __double2float_rn(x - (double)h);
    }
}

// Lame weights (B, mu) = (lambda + mu, mu) in FP32 from Young's modulus E and
// h = 1/2 - nu, rounded to FP32 from its FP64 value: then 1 - 2 nu = 2h, 1 + nu =
// 3/2 - h and nu = 1/2 - h carry no cancellation, where 1 - 2 nu formed from an
// FP32 nu near 1/2 loses digits (its relative error grows as 1 / (1 - 2 nu)).
__device__ __forceinline__ float2 lame32(float E, float h) {
    const float nu = 0.5f - h, onePlus = 1.5f - h;
    const float lam = (E * nu) / (onePlus * (2.0f * h));
    const float mu = E / (2.0f * onePlus);
    return make_float2(lam + mu, mu);
}

// DLAMCH('S'): smallest normal double.
constexpr double kSafeMin = 2.2250738585072014e-308;

__device__ __forceinline__ void swap_if(bool c, double &x, double &y) {
    const double t = x;
    x = c ? y : x;
    y = c ? t : y;
}

// Inverse of a 3x3 block in column-major storage, following the operation order
// of LAPACK's DGETRF (recursive DGETRF2: IDAMAX pivot, reciprocal scaling when
// |pivot| >= DLAMCH('S'), C := C + (-u) l updates) and DGETRI (DTRTI2 with
// DTRMV's zero test and DSCAL by -inv(u_jj), then inv(A) L = inv(U) by DGEMV
// columns, then column swaps), as the reference calls them for its 3x3 blocks
// (src/Fortran/elasclpr.f:39,44).  Returns LAPACK's INFO: 0, or k when U(k,k) is
// exactly zero, in which case the block holds the LU factors (DGETRI returns
// before touching it).
__device__ __forceinline__ int lu_inverse3(double a[9]) {
    int info = 0;
    // ---- DGETRF: column 0 panel
    int p0 = 0;
    {
        double mx = fabs(a[0]);
        if (fabs(a[1]) > mx) { p0 = 1; mx = fabs(a[1]); }
        if (fabs(a[2]) > mx) { p0 = 2; }
    }
    const double piv0 = p0 == 0 ? a[0] : (p0 == 1 ? a[1] : a[2]);
    if (piv0 != 0.0) {
        swap_if(p0 == 1, a[0], a[1]);
        swap_if(p0 == 2, a[0], a[2]);
        if (fabs(a[0]) >= kSafeMin) {
            const double r = 1.0 / a[0];
            a[1] = r * a[1];
            a[2] = r * a[2];
        } else {
            a[1] = a[1] / a[0];
            a[2] = a[2] / a[0];
        }
    } else {
        info = 1;
    }
    // interchange applied to columns 1 and 2
    swap_if(p0 == 1, a[3], a[4]);
    swap_if(p0 == 2, a[3], a[5]);
    swap_if(p0 == 1, a[6], a[7]);
    swap_if(p0 == 2, a[6], a[8]);
    // trailing update A22 := A22 + (-u) * l
    {
        const double t1 = neg(a[3]);
        a[4] = a[4] + t1 * a[1];
        a[5] = a[5] + t1 * a[2];
        const double t2 = neg(a[6]);
        a[7] = a[7] + t2 * a[1];
        a[8] = a[8] + t2 * a[2];
    }
    // ---- column 1 panel (rows 1..2)
    const int p1 = fabs(a[5]) > fabs(a[4]) ? 2 : 1;
    const double piv1 = p1 == 1 ? a[4] : a[5];
    if (piv1 != 0.0) {
        swap_if(p1 == 2, a[4], a[5]);
        if (fabs(a[4]) >= kSafeMin) {
            const double r = 1.0 / a[4];
            a[5] = r * a[5];
        } else {
            a[5] = a[5] / a[4];
        }
    } else if (info == 0) {
        info = 2;
    }
    swap_if(p1 == 2, a[7], a[8]);
    a[8] = a[8] + neg(a[7]) * a[5];
    if (a[8] == 0.0 && info == 0) info = 3;
    swap_if(p1 == 2, a[1], a[2]);   // second interchange on the first column of L
    (void)info;

    // ---- DGETRI
    if (a[0] == 0.0) return 1;
    if (a[4] == 0.0) return 2;
    if (a[8] == 0.0) return 3;
    // DTRTI2: inverse of U in place
    a[0] = 1.0 / a[0];
    a[4] = 1.0 / a[4];
    {
        const double ajj = neg(a[4]);
        if (a[3] != 0.0) a[3] = a[3] * a[0];
        a[3] = ajj * a[3];
    }
    a[8] = 1.0 / a[8];
    {
        const double ajj = neg(a[8]);
        if (a[6] != 0.0) a[6] = a[6] * a[0];
        if (a[7] != 0.0) {
            const double t = a[7];
            a[6] = a[6] + t * a[3];
            a[7] = a[7] * a[4];
        }
        a[6] = ajj * a[6];
        a[7] = ajj * a[7];
    }
    // inv(A) * L = inv(U), columns 1 then 0
    {
        const double w2 = a[5];
        a[5] = 0.0;
        const double t = neg(w2);
        a[3] = a[3] + t * a[6];
        a[4] = a[4] + t * a[7];
        a[5] = a[5] + t * a[8];
    }
    {
        const double w1 = a[1], w2 = a[2];
        a[1] = 0.0;
        a[2] = 0.0;
        const double t1 = neg(w1);
        a[0] = a[0] + t1 * a[3];
        a[1] = a[1] + t1 * a[4];
        a[2] = a[2] + t1 * a[5];
        const double t2 = neg(w2);
        a[0] = a[0] + t2 * a[6];
        a[1] = a[1] + t2 * a[7];
        a[2] = a[2] + t2 * a[8];
    }
    // column interchanges, last pivot first
    swap_if(p1 == 2, a[3], a[6]);
    swap_if(p1 == 2, a[4], a[7]);
    swap_if(p1 == 2, a[5], a[8]);
    swap_if(p0 == 1, a[0], a[3]);
    swap_if(p0 == 1, a[1], a[4]);
    swap_if(p0 == 1, a[2], a[5]);
    swap_if(p0 == 2, a[0], a[6]);
    swap_if(p0 == 2, a[1], a[7]);
    swap_if(p0 == 2, a[2], a[8]);
    return 0;
}

// src/Fortran/elasclpr.f:19-27: for every constrained DOF k, zero row and column
// k of the block and put 1 on the diagonal.
__device__ __forceinline__ void dirichlet_mask3(double a[9], unsigned mask) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (mask & (1u << k)) {
#pragma unroll
            for (int q = 0; q < 3; q++) {
                a[k + 3 * q] = 0.0;
                a[q + 3 * k] = 0.0;
            }
            a[k + 3 * k] = 1.0;
        }
    }
}

}  // namespace mfem
