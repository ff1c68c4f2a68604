// Double-precision multiplication on the integer pipes.
//
// GB300 issues FP64 arithmetic at about two operations per clock per SM
// (1/64 of its FP32 rate), and the bit-exact FP64 assembly is bound by that
// pipe.  dmul_ipipe(a, b) forms the same correctly rounded product (IEEE 754
// multiplication, round to nearest, ties to even) with 32-bit integer
// multiply-adds and shifts, which run on other pipes: a kernel that sends part of
// its products here and the rest to the FP64 unit runs both at once.
//
// Method (the schoolbook soft-float multiplication, as in Hauser's SoftFloat):
//   * operands with biased exponents 1..2046 whose product stays in the normal
//     range take the fast path; zeros, subnormals, infinities, NaNs and
//     products near the exponent limits go to the FP64 unit (__dmul_rn);
//   * the 53-bit significands (implicit bit set) are multiplied exactly into
//     106 bits with four 32x32->64 products;
//   * bits 43..105 of the product are kept in a 64-bit word whose bit 0 is
//     OR-ed with the sticky bit (any of bits 0..42 set); the product's leading
//     bit is bit 105 or 104, so the 53-bit result is that word shifted right by
//     10 or 9, rounded to nearest even by adding (half - 1 + lsb) before the
//     shift;
//   * exponent and significand are added as integers, so a rounding carry out of
//     the significand increments the exponent (and reaches infinity exactly when
//     IEEE rounding overflows).
// The result is bit-identical to the hardware product on every fast-path input;
// tests check it against the CPU's and the GPU's multiplication.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define MFEM_HD __host__ __device__ __forceinline__
#else
#define MFEM_HD static inline
#endif

namespace mfem {

// Fast-path product of the bit patterns A and B; returns false (and leaves
// *out unset) when the operands or the result are outside the normal range.
MFEM_HD bool dmul_bits(uint64_t A, uint64_t B, uint64_t *out) {
    const uint32_t ah = (uint32_t)(A >> 32), al = (uint32_t)A;
    const uint32_t bh = (uint32_t)(B >> 32), bl = (uint32_t)B;
    const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu;
    // biased exponent of the result, less one, for a product below 2^105
    const int e = (int)(ea + eb) - 1024;
    if (ea - 1u >= 2046u || eb - 1u >= 2046u || (uint32_t)(e - 1) >= 2044u) return false;
    const uint32_t a1 = (ah & 0xfffffu) | 0x100000u, b1 = (bh & 0xfffffu) | 0x100000u;
    // (a1 2^32 + al)(b1 2^32 + bl) = t3 2^64 + (uint32)t2 2^32 + (uint32)t0
    const uint64_t t0 = (uint64_t)al * bl;
    const uint64_t t1 = (uint64_t)a1 * bl + (t0 >> 32);
    const uint64_t t2 = (uint64_t)al * b1 + (uint32_t)t1;
    const uint64_t t3 = (uint64_t)a1 * b1 + (t1 >> 32) + (t2 >> 32);
    const uint32_t p1 = (uint32_t)t2, p0 = (uint32_t)t0;
    const uint64_t m = (t3 << 21) | (p1 >> 11) | (uint64_t)(((p1 & 0x7ffu) | p0) != 0u);
    const uint32_t top = (uint32_t)(m >> 62);          // 1 when the product is >= 2^105
    const uint32_t sh = 9u + top;
    const uint64_t r = (m + ((1ull << (sh - 1u)) - 1ull) + ((m >> sh) & 1ull)) >> sh;
    *out = ((((uint64_t)(uint32_t)(e + (int)top)) << 52) + r) |
           ((uint64_t)((ah ^ bh) & 0x80000000u) << 32);
    return true;
}

// hi = fl32(x) and lo = fl32(x - hi) (round to nearest even; x - hi is exact in
// FP64) from the bit pattern X of a double with biased exponent in
// [1023 - 60, 1023 + 100]; returns false otherwise (zero, tiny, huge, special).
// The dropped 29 significand bits give x - hi directly: m29 when hi was
// rounded down, -(2^29 - m29) when it was rounded up, times 2^(e - 1075); the
// FP32 rounding of that integer is a u32 -> f32 conversion and an exponent add.
MFEM_HD bool split_f32_bits(uint64_t X, uint32_t *hi, uint32_t *lo) {
    const uint32_t hw = (uint32_t)(X >> 32), lw = (uint32_t)X;
    const uint32_t e = (hw >> 20) & 0x7ffu;
    if (e < 1023u - 60u || e > 1023u + 100u) return false;
    const uint32_t sign = hw & 0x80000000u;
    const uint32_t m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
    const uint32_t m29 = lw & 0x1fffffffu;
    const bool up = m29 > 0x10000000u || (m29 == 0x10000000u && (m23 & 1u));
    *hi = (sign | ((e - 1023u + 127u) << 23) | m23) + (up ? 1u : 0u);
    const uint32_t mag = up ? 0x20000000u - m29 : m29;
    if (mag == 0u) {
        *lo = 0u;
        return true;
    }
#ifdef __CUDA_ARCH__
    const float f = __uint2float_rn(mag);
    uint32_t fb = __float_as_uint(f);
#else
    const float f = (float)mag;
    uint32_t fb;
    memcpy(&fb, &f, 4);
#endif
    fb += (uint32_t)((int32_t)e - 1075) << 23;
    *lo = fb | (up ? sign ^ 0x80000000u : sign);
    return true;
}

#ifdef __CUDACC__
__device__ __forceinline__ double dmul_ipipe(double a, double b) {
    uint64_t r;
    if (dmul_bits((uint64_t)__double_as_longlong(a), (uint64_t)__double_as_longlong(b), &r))
        return __longlong_as_double((long long)r);
    return __dmul_rn(a, b);
}
#endif

}  // namespace mfem
