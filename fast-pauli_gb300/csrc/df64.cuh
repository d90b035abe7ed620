// df64.cuh -- double-float ("df64") arithmetic for the float64 expectation
// kernels.
//
// GB300 executes float64 at 1.19 TFLOP/s, 1/64 of its float32 rate, and the
// float64 expectation kernels are float64-pipe bound.  A float64 value x is
// carried here as an unevaluated sum hi + lo of two floats (48 significand
// bits, relative representation error <= 2^-48), products are formed exactly
// with the fused multiply-add error term and sums are accumulated with
// Knuth's error-free TwoSum, so that sums of products keep ~2^-47 relative
// accuracy while every operation runs on the float32 / integer pipes.
// Published method: T. J. Dekker, "A floating-point technique for extending
// the available precision", Numer. Math. 18 (1971); D. E. Knuth, TAOCP vol. 2,
// 4.2.2 (TwoSum); A. Thall, "Extended-precision floating-point numbers for
// GPU computation" (2006).
//
// split_bits: the float64 -> (hi, lo) split from the IEEE-754 bit pattern with
// integer operations only: hi keeps the top 24 significand bits (truncated),
// lo = the next 29 bits rounded to 24.  Magnitudes outside float's normal
// range (|x| < 2^-126 or |x| >= 2^128) are not representable: the kernels
// using this split take unit-norm state amplitudes (|x| <= 1); amplitudes
// below 2^-126 (and lo parts below 2^-126) flush to zero, an absolute error
// < 2^-126 per amplitude.
#pragma once

#include <cstdint>

namespace fpg
{

// (hi, lo) of the float64 whose bit pattern is (bh << 32) | bl
__device__ __forceinline__ void split_bits(uint32_t bl, uint32_t bh, float &hi, float &lo)
{
    const uint32_t sign = bh & 0x80000000u;
    const int E = (int)((bh >> 20) & 0x7ffu);
    const int fe = E - 1023 + 127;     // float exponent field of hi
    const uint32_t m23 = ((bh & 0xfffffu) << 3) | (bl >> 29);
    hi = __uint_as_float((fe > 0 && fe < 255) ? (sign | ((uint32_t)fe << 23) | m23) : sign);
    // lo = (bl & (2^29 - 1)) * 2^(E - 1075)
    const int se = E - 1075 + 127;     // float exponent field of 2^(E-1075)
    const float scale = se > 0 ? __uint_as_float((uint32_t)se << 23) : 0.0f;
    const float l = (float)(bl & 0x1fffffffu) * scale;
    lo = __uint_as_float(__float_as_uint(l) | sign);
}

// Range of the df64 kernels.  Per element: |x| < 2^40, so that products
// (< 2^80) and sums of up to 2^40 of them stay below float's largest value.
// Per state column (and over an operand such as the coefficients): the
// largest |x| at least 2^-39 unless the column is all zero, so that the
// products that make up its results (down to 2^-78) and their error terms
// (2^-48 smaller) stay in float's normal range; values far below a column's
// largest contribute errors below 2^-126 each, far below 2^-48 of its
// results.  A kernel that meets an element outside the first bound, or the
// split pass (k_df_split) a column outside the second, raises a per-call
// flag, and the float64 form of the kernel, launched after it on the same
// stream, then recomputes the result (it returns at once while the flag is
// clear).  bh = high word of the float64.
__device__ __forceinline__ bool df_out_of_range(uint32_t bh)
{
    return ((bh >> 20) & 0x7ffu) >= 1023u + 40u; // |x| >= 2^40, inf or nan
}

// The column bound as the high word of |x| (monotone in |x|): 2^-39
constexpr uint32_t kDfColumnMinKey = (1023u - 39u) << 20;

// One complex128 amplitude as df64: (re_h, re_l, im_h, im_l) from its four
// 32-bit words; bad |= a part outside the df64 range.
__device__ __forceinline__ float4 split_complex(uint4 w, bool &bad)
{
    float4 r;
    split_bits(w.x, w.y, r.x, r.y);
    split_bits(w.z, w.w, r.z, r.w);
    bad |= df_out_of_range(w.y) | df_out_of_range(w.w);
    return r;
}

// The error-free steps below use the _rn intrinsics: the compiler never
// merges them into a fused multiply-add, which would make p (or s) differ
// from the value the error term is computed against.

// (sh, sl) += (xh + xl) * (yh + yl), to ~2^-47 relative of the product
__device__ __forceinline__ void df_fma(float xh, float xl, float yh, float yl, float &sh, float &sl)
{
    const float p = __fmul_rn(xh, yh);
    float e = __fmaf_rn(xh, yh, -p); // exact: xh*yh = p + e
    e = __fmaf_rn(xh, yl, e);
    e = __fmaf_rn(xl, yh, e);
    // TwoSum(sh, p): s + err = sh + p exactly
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// (sh, sl) += (xh + xl) * (yh + yl) for an accumulator whose high part is
// offset by a power of two sigma that bounds the sum: the caller starts with
// sh = sigma, sl = 0 and keeps every partial sum and term below sigma / 16 in
// magnitude, so sh stays inside (sigma / 2, 2 sigma) and on one grid.  Then
// s - sh is exact (Sterbenz) and one fused multiply-add returns the rounding
// error of s: 6 float32 operations per term instead of the 12 of df_fma,
// with the error bounded by ~2^-47 sigma per term rather than by the
// products.  The caller takes sh - sigma (exact) as the high part of the sum.
__device__ __forceinline__ void df_fma_offset(float xh, float xl, float yh, float yl, float &sh, float &sl)
{
    const float s = __fmaf_rn(xh, yh, sh);
    const float d = __fsub_rn(s, sh);      // exact
    const float r = __fmaf_rn(xh, yh, -d); // xh*yh - d = rounding error of s, rounded once
    sl = __fmaf_rn(xh, yl, sl);
    sl = __fmaf_rn(xl, yh, sl);
    sl = __fadd_rn(sl, r);
    sh = s;
}

// The offset for df_fma_offset: a power of two > 16 m2 (m2 >= 0 finite), at
// least 2^-126, so that sums of up to 8 terms of magnitude <= m2 keep the
// offset accumulator inside its binade pair.  Rounding of 16 * m2 is
// monotone, so the result also exceeds the exact 16 m2.
__device__ __forceinline__ float df_offset_for(float m2)
{
    const float m16 = __fmul_rn(m2, 16.0f);
    return __uint_as_float((__float_as_uint(m16) & 0x7f800000u) + 0x00800000u);
}

// (sh, sl) = (xh + xl) * (yh + yl), to ~2^-47 relative of the product: the
// first term of a sum, with no addition
__device__ __forceinline__ void df_mul(float xh, float xl, float yh, float yl, float &sh, float &sl)
{
    const float p = __fmul_rn(xh, yh);
    float e = __fmaf_rn(xh, yh, -p);
    e = __fmaf_rn(xh, yl, e);
    e = __fmaf_rn(xl, yh, e);
    sh = p;
    sl = e;
}

// (ah, al) += (bh, bl) without renormalising: TwoSum of the high parts, the
// low part absorbing its error and bl.  Like df_fma the low part grows with
// each term: callers renormalise (df_norm) every few terms.
__device__ __forceinline__ void df_add_lazy(float &ah, float &al, float bh, float bl)
{
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    ah = s;
    al = __fadd_rn(al, __fadd_rn(err, bl));
}

// Renormalise (h, l) so that |l| <= ulp(h) / 2 (FastTwoSum).  df_fma lets the
// low part grow with the number of terms it has absorbed, which costs its
// rounding ~2^-24 |l| per step: callers renormalise every few dozen terms.
__device__ __forceinline__ void df_norm(float &h, float &l)
{
    const float s = __fadd_rn(h, l);
    l = __fsub_rn(l, __fsub_rn(s, h));
    h = s;
}

// (ah, al) += (bh, bl), renormalised
__device__ __forceinline__ void df_add(float &ah, float &al, float bh, float bl)
{
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    ah = s;
    al = __fadd_rn(al, __fadd_rn(err, bl));
    df_norm(ah, al);
}

__device__ __forceinline__ double df_to_double(float h, float l)
{
    return (double)h + (double)l;
}

} // namespace fpg
