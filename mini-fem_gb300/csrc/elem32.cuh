// Per-element arithmetic of the FP32 path (shared by the record kernel and the
// tile kernel).  Coordinates arrive split into float hi + lo parts so that the
// edge vectors are the FP64 differences rounded once to FP32; cross products use
// Kahan's a*b - c*d with an FMA; elements below the quality threshold get their
// gradients from the FP64 formula (elem_math.cuh) instead.
#pragma once

#include <cuda_runtime.h>

#include "elem_math.cuh"

namespace mfem {

// a*b - c*d with one rounding error less than the plain expression (Kahan).
__device__ __forceinline__ float diff_prod(float a, float b, float c, float d) {
    const float w = c * d;
    const float e = fmaf(-c, d, w);
    const float f = fmaf(a, b, -w);
    return f + e;
}

// The eight coordinate words (hi and lo of the four nodes) of one element.
struct ElemCoords {
    float4 h0, h1, h2, h3, l0, l1, l2, l3;
};

// Gradients g[4][3] of one element in FP32 from its loaded coordinates.
// Returns true, with g not computed, when the element is flagged: quality
// |6V| / (|a||b||c|) below sqrt(qthr2).
__device__ __forceinline__ bool grad32_core(const ElemCoords &C, float qthr2, float g[12]) {
    const float xa = (C.h0.x - C.h3.x) + (C.l0.x - C.l3.x), ya = (C.h0.y - C.h3.y) + (C.l0.y - C.l3.y),
                za = (C.h0.z - C.h3.z) + (C.l0.z - C.l3.z);
    const float xb = (C.h2.x - C.h3.x) + (C.l2.x - C.l3.x), yb = (C.h2.y - C.h3.y) + (C.l2.y - C.l3.y),
                zb = (C.h2.z - C.h3.z) + (C.l2.z - C.l3.z);
    const float xc = (C.h1.x - C.h3.x) + (C.l1.x - C.l3.x), yc = (C.h1.y - C.h3.y) + (C.l1.y - C.l3.y),
                zc = (C.h1.z - C.h3.z) + (C.l1.z - C.l3.z);
    g[0] = diff_prod(yb, zc, yc, zb); g[1] = diff_prod(zb, xc, zc, xb); g[2] = diff_prod(xb, yc, xc, yb);
    g[3] = diff_prod(ya, zb, yb, za); g[4] = diff_prod(za, xb, zb, xa); g[5] = diff_prod(xa, yb, xb, ya);
    g[6] = diff_prod(yc, za, ya, zc); g[7] = diff_prod(zc, xa, za, xc); g[8] = diff_prod(xc, ya, xa, yc);
    const float vol = fmaf(xa, g[0], fmaf(ya, g[1], za * g[2]));
    const float na = fmaf(xa, xa, fmaf(ya, ya, za * za));
    const float nb = fmaf(xb, xb, fmaf(yb, yb, zb * zb));
    const float nc = fmaf(xc, xc, fmaf(yc, yc, zc * zc));
    if (vol * vol < qthr2 * (na * nb) * nc) return true;
    g[9] = -((g[0] + g[3]) + g[6]);
    g[10] = -((g[1] + g[4]) + g[7]);
    g[11] = -((g[2] + g[5]) + g[8]);
    const float r = 1.0f / vol;
#pragma unroll
    for (int i = 0; i < 12; i++) g[i] *= r;
    return false;
}

__device__ __forceinline__ float f64_to_f32(double x);

// Gradients of a flagged element: the FP64 formula (its cross products and
// 1/vol scalings on the integer pipes, elem_math.cuh), rounded to FP32.
__device__ __forceinline__ void grad32_fp64(const double *__restrict__ coord, int4 nd, float g[12]) {
    double gd[12];
    elem_gradients(coord, nd, gd);
#pragma unroll
    for (int i = 0; i < 12; i++) g[i] = f64_to_f32(gd[i]);
}

// double -> float, round to nearest even, with integer operations so that it
// stays off GB300's narrow FP64 pipe; values outside the normal float range
// (and zero) take the conversion instruction.
__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned e = (hi >> 20) & 0x7ffu;
    if (e <= 1023u - 127u || e >= 1023u + 127u) return __double2float_rn(x);
    const unsigned m23 = ((hi & 0xfffffu) << 3) | (lo >> 29);   // top 23 mantissa bits
    const unsigned rem = lo & 0x1fffffffu;                        // the 29 bits dropped
    unsigned r = (hi & 0x80000000u) | ((e - 1023u + 127u) << 23) | m23;
    if (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) r += 1u;   // carries into the exponent
    return __uint_as_float(r);
}

// x * 2^k, exact, by exponent arithmetic on the integer pipe when x and the
// result are normal; otherwise (zero, subnormal, out of range) by a multiply.
__device__ __forceinline__ double scale_pow2(double x, int k) {
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e > 0 && e + k > 0 && e + k < 0x7ff) return __longlong_as_double(b + ((long long)k << 52));
    if (x == 0.0) return x;
    const int kk = max(-1022, min(1023, k));
    return x * __longlong_as_double((long long)(kk + 1023) << 52);
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

// Weights of the FP32 blocks: (B, mu) for ela, (kappa, 0) for lap, from the FP64
// per-element coefficients (NULL: the reference constants B = 1.25, mu = 1,
// kappa = 1).  1/2 - nu from the hi/lo split of nu, within an FP32 ulp, without
// the FP64 pipe.
template <int OP>
__device__ __forceinline__ float2 weights32(const double *__restrict__ coef, int e) {
    if (OP == MFEM_OP_LAP) return make_float2(coef ? f64_to_f32(coef[e]) : 1.0f, 0.f);
    if (!coef) return make_float2(1.25f, 1.0f);
    const double2 c = reinterpret_cast<const double2 *>(coef)[e];
    float nh, nl;
    split_hilo(c.y, nh, nl);
    return lame32(f64_to_f32(c.x), (0.5f - nh) - nl);
}

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
};

}  // namespace mfem
