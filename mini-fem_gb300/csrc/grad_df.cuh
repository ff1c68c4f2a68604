// Gradients of a poorly shaped element in double-float arithmetic.
//
// The FP32 path computes element gradients in FP32 (elem32.cuh) and re-does the
// elements whose quality |6V| / (|a||b||c|) falls below a threshold in higher
// precision, because the FP32 volume of a flat element loses about log2(1/q)
// bits.  That higher precision is done here with pairs of FP32 numbers
// (value = hi + lo, about 47 significant bits) on the FP32 pipes: GB300's FP64
// pipe runs at 1/64 of its FP32 rate,
// and the coordinates are already at hand as FP32 hi/lo pairs (x = hi + lo to
// within 2^-48 |x|).
//
// Error-free transformations (Knuth's TwoSum, Dekker's Fast2Sum, the FMA-based
// TwoProd) and the double-float add / multiply built on them follow the
// published double-float ("double-single") algorithms; the reciprocal of the
// volume is the FP32 reciprocal refined by one Newton step in double-float.
// The formula is the reference's (src/assembly.cc:85-121): edge vectors
// a = x0 - x3, b = x2 - x3, c = x1 - x3; g0 = b x c, g1 = a x b, g2 = c x a,
// g3 = -(g0 + g1 + g2), all over vol = a . g0.  Each result is rounded to FP32
// once at the end, so it matches the FP64 gradients rounded to FP32 except for
// values near a rounding boundary: the CPU test bounds the difference by 1.5 x
// 2^-24 of the element's largest gradient component, down to quality 1e-4.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define MFEM_DF __host__ __device__ __forceinline__
#else
#define MFEM_DF static inline
#endif

namespace mfem {
namespace df {

struct F2 {
    float h, l;
};

MFEM_DF F2 two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

MFEM_DF F2 fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
    const float s = a + b;
    return {s, b - (s - a)};
}

// renormalised with TwoSum, not Fast2Sum: after a hard cancellation of the hi
// parts the lo parts may be the larger
MFEM_DF F2 add(F2 a, F2 b) {
    const F2 s = two_sum(a.h, b.h);
    return two_sum(s.h, s.l + (a.l + b.l));
}

MFEM_DF F2 neg(F2 a) { return {-a.h, -a.l}; }

MFEM_DF F2 mul(F2 a, F2 b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.h, -p);
    return fast_two_sum(p, fmaf(a.h, b.l, fmaf(a.l, b.h, e)));
}

// a * b - c * d
MFEM_DF F2 cross(F2 a, F2 b, F2 c, F2 d) { return add(mul(a, b), neg(mul(c, d))); }

// (ph + pl) - (qh + ql) for coordinates split into FP32 hi and lo parts
MFEM_DF F2 diff(float ph, float pl, float qh, float ql) {
    const F2 s = two_sum(ph, -qh);
    return two_sum(s.h, s.l + (pl - ql));
}

// FP32 rounding of a * b
MFEM_DF float mul_round(F2 a, F2 b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.h, -p);
    return p + fmaf(a.h, b.l, fmaf(a.l, b.h, e));
}

}  // namespace df

// Gradients g[4][3] (row-major, g[3j + k]) of the element whose node j has
// coordinates hi[j][k] + lo[j][k].  Returns false, g unset, when the element's
// quality is below 1e-4 or its double-float volume is zero or not finite; the
// caller then takes the FP64 formula (whose 1/vol gives the reference's
// infinities for a zero volume).
MFEM_DF bool grad_df(const float hi[4][3], const float lo[4][3], float g[12]) {
    using namespace df;
    F2 a[3], b[3], c[3];
    for (int k = 0; k < 3; k++) {
        a[k] = diff(hi[0][k], lo[0][k], hi[3][k], lo[3][k]);
        b[k] = diff(hi[2][k], lo[2][k], hi[3][k], lo[3][k]);
        c[k] = diff(hi[1][k], lo[1][k], hi[3][k], lo[3][k]);
    }
    F2 G[12];
    G[0] = cross(b[1], c[2], c[1], b[2]);
    G[1] = cross(b[2], c[0], c[2], b[0]);
    G[2] = cross(b[0], c[1], c[0], b[1]);
    G[3] = cross(a[1], b[2], b[1], a[2]);
    G[4] = cross(a[2], b[0], b[2], a[0]);
    G[5] = cross(a[0], b[1], b[0], a[1]);
    G[6] = cross(c[1], a[2], a[1], c[2]);
    G[7] = cross(c[2], a[0], a[2], c[0]);
    G[8] = cross(c[0], a[1], a[0], c[1]);
    for (int k = 0; k < 3; k++) G[9 + k] = neg(add(add(G[k], G[3 + k]), G[6 + k]));
    const F2 vol = add(add(mul(a[0], G[0]), mul(a[1], G[1])), mul(a[2], G[2]));
    if (!(vol.h != 0.0f) || !isfinite(vol.h)) return false;
    // below quality 1e-4 the cancellations outgrow the pairs' 47 bits: the FP64
    // formula (about 5,000 such elements in the 1.2M-tet stress mesh)
    const float na = fmaf(a[0].h, a[0].h, fmaf(a[1].h, a[1].h, a[2].h * a[2].h));
    const float nb = fmaf(b[0].h, b[0].h, fmaf(b[1].h, b[1].h, b[2].h * b[2].h));
    const float nc = fmaf(c[0].h, c[0].h, fmaf(c[1].h, c[1].h, c[2].h * c[2].h));
    if (vol.h * vol.h < 1e-8f * (na * nb) * nc) return false;
    // 1 / vol: the FP32 reciprocal r0, then r = r0 + r0 (1 - vol r0)
    const float r0 = 1.0f / vol.h;
    const float p = vol.h * r0;
    const float pe = fmaf(vol.h, r0, -p) + vol.l * r0;
    const F2 r = fast_two_sum(r0, r0 * ((1.0f - p) - pe));
    for (int i = 0; i < 12; i++) g[i] = mul_round(G[i], r);
    return true;
}

}  // namespace mfem
