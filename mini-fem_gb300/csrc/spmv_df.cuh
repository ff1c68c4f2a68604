// Double-float accumulation of the FP32-valued operator (solve.cu: k_spmv32),
// in a form that compiles for the host too, so that its accuracy is checked on
// the CPU (tests/spmv_df_check.cc).
//
// A product a x_j with a an FP32 value and x_j = hi + lo (FP32 parts of the
// scaled FP64 entry) is formed as the exact a hi (its FP32 rounding p and the
// FMA error e, TwoProd) plus a lo rounded; p goes into the running sum s by
// Knuth's TwoSum, e, the TwoSum error and a lo into the tail t; after every
// chunk of blocks the pair is renormalized.  Measured (spmv_df_check, 1.8
// million rows of 1-40 random blocks summing to zero, random and near-constant
// x): the merged result within 15 x 2^-48 of the sum of |a x| for 3x3 blocks
// (28 without the renormalization), 8 x 2^-48 for scalars, 0.6 x 2^-48 on
// average.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define MFEM_SPDF __host__ __device__ __forceinline__
#else
#define MFEM_SPDF static inline
#endif

namespace mfem {
namespace spdf {

// (s, t) += a (xh + xl); returns |a xh| rounded, the product's magnitude
MFEM_SPDF float accumulate(float &s, float &t, float a, float xh, float xl) {
    const float p = a * xh;
    const float e = fmaf(a, xh, -p);
    const float s1 = s + p;
    const float bp = s1 - s;
    const float err = (s - (s1 - bp)) + (p - bp);
    s = s1;
    t = fmaf(a, xl, t) + (e + err);
    return fabsf(p);
}

// (s, t) -> (s + t rounded, its error): moves the tail's bulk into the head, so
// that the tail's own roundings stay relative to 2^-24 |s| (TwoSum, as t may
// exceed s after cancellation)
MFEM_SPDF void renormalize(float &s, float &t) {
    const float s1 = s + t;
    const float bp = s1 - s;
    t = (s - (s1 - bp)) + (t - bp);
    s = s1;
}

// (s, t) += (s2, t2): TwoSum of the heads, the tails and its error added
MFEM_SPDF void merge(float &s, float &t, float s2, float t2) {
    const float s1 = s + s2;
    const float bp = s1 - s;
    const float err = (s - (s1 - bp)) + (s2 - bp);
    s = s1;
    t = (t + t2) + err;
}

}  // namespace spdf
}  // namespace mfem
