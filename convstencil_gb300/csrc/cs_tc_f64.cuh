// cs_tc_f64.cuh — the FP64 number format of the tcgen05 digit kernels
// (cs_kernels_split_tc.cu for 2D, cs_kernels_split_tc3d.cu for 3D): weights
// and inputs cut into six balanced 9-bit digits held exactly in FP16 (the
// inputs with integer operations only), and the exact integer recombination
// of the level sums with one rounding to FP64.
#pragma once

#include <cuda_fp16.h>

#include <cmath>

#include "cs_internal.h"
#include "cs_split_common.cuh"

namespace cs {
namespace tc {

// Six balanced base-512 digits of w / 2^ew (|w| / 2^ew < 1/4, so the top
// digit stays within 128) for the 49 taps of a 7x7 kernel, or for the first
// `taps` (27: a 3x3x3 kernel).
struct F64Weights {
    __half d[6][49];
    int ew;
};

inline F64Weights f64_slice_weights(const Weights &w, int taps = 49)
{
    F64Weights s{};
    double mx = 0.0;
    for (int i = 0; i < taps; ++i) mx = std::fmax(mx, std::fabs(w.v[i]));
    int e = 0;
    if (mx > 0.0) {
        std::frexp(mx, &e);  // mx < 2^e
        e += 2;              // |w| / 2^ew < 1/4
    }
    s.ew = e;
    for (int i = 0; i < taps; ++i) {
        double a = std::ldexp(w.v[i], split::kDigitBits - e);  // |a| < 128, exact
        for (int k = 0; k < 6; ++k) {
            const double d = std::rint(a);
            s.d[k][i] = __float2half_rn((float)d);
            a = (a - d) * 512.0;  // exact: a - d is a multiple of a's last bit
        }
    }
    return s;
}

// ---- FP64 digits and recombination (integer operations only)

// 256 in each of six 9-bit fields: Y = X + kF64Bias has fields u in [0, 511]
// (top field up to 384) with X = sum (u_k - 256) 512^(5-k).
constexpr unsigned long long kF64Bias = 256ull * ((1ull << 54) - 1) / 511;

// Biased-digit word of one FP64 value (bits lo, hi) of a tile whose largest
// biased exponent is eb1 (at least 1): X = round(x / 2^(eb1 - 1074)), so
// |X| <= 2^52, returned as X + kF64Bias. The shift is clamped at 63: any
// mantissa (< 2^53) shifted by 55 or more rounds to 0 as it should.
__device__ __forceinline__ unsigned long long f64_biased_fixed(unsigned lo, unsigned hi, int eb1)
{
    const int e = (int)((hi >> 20) & 0x7FFu);
    const int ee = max(e, 1);  // subnormals: no implicit bit, exponent 1
    const unsigned long long mant =
        ((unsigned long long)((hi & 0xFFFFFu) | (e ? 0x100000u : 0u)) << 32) | lo;
    const unsigned long long x = ((mant >> min(eb1 - ee, 63)) + 1) >> 1;  // round half up
    const unsigned long long neg = (unsigned long long)(long long)((int)hi >> 31);  // 0 or all ones
    return (kF64Bias - neg) + (x ^ neg);  // kF64Bias + x, or kF64Bias - x = (kF64Bias + 1) + ~x
}

// Digit k (0 = most significant) of two biased words, as an FP16 pair:
// FP16 (1024 + u) has the bits 0x6400 | u, and (1024 + u) - 1280 = u - 256
// is exact in FP16. (The top field is at most 384, so masking it is harmless.)
template <int K>
__device__ __forceinline__ unsigned f64_digit_pair(unsigned long long ya, unsigned long long yb)
{
    constexpr int sh = split::kDigitBits * (5 - K);
    const unsigned ta = (unsigned)(ya >> sh);
    const unsigned tb = sh >= 16 ? (unsigned)(yb >> (sh - 16)) : (unsigned)(yb << (16 - sh));
    const unsigned w = ((ta & 0x1FFu) | (tb & 0x1FF0000u)) | 0x64006400u;
    const __half2 h = __hsub2(*reinterpret_cast<const __half2 *>(&w), __halves2half2(__ushort_as_half(0x6500),
                                                                                     __ushort_as_half(0x6500)));
    return *reinterpret_cast<const unsigned *>(&h);
}

// T = sum over levels of S_L 2^(42 - 9L), level 5 without its last three
// bits: |T| < 2^63. Multiply-adds on the FMA pipe (the integer ALU pipe is
// this kernel's busiest).
__device__ __forceinline__ long long f64_combine(const float (&lv)[6])
{
    long long t = (long long)(__float2int_rn(lv[5]) >> 3);
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(t) : "r"(__float2int_rn(lv[4])), "r"(1 << 6));
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(t) : "r"(__float2int_rn(lv[3])), "r"(1 << 15));
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(t) : "r"(__float2int_rn(lv[2])), "r"(1 << 24));
    unsigned tl, th;
    asm("mov.b64 {%0, %1}, %2;" : "=r"(tl), "=r"(th) : "l"(t));
    // levels 0 and 1 sit wholly in the upper word: S1 2^33 + S0 2^42
    th += (unsigned)(__float2int_rn(lv[1]) * 2 + __float2int_rn(lv[0]) * 1024);
    asm("mov.b64 %0, {%1, %2};" : "=l"(t) : "r"(tl), "r"(th));
    return t;
}

// f64_combine for level sums below 2^22 in magnitude (one z tap of a 3D
// input plane: 9 taps, so level L sums at most 9 * 5 * 2^16 < 2^22): the
// integers come out of the FP32 sums by one addition of 1.5 * 2^23 (exact in
// that range: the sum lands in [2^23, 2^24), where the spacing is 1, and its
// low mantissa bits are 2^22 + S) and one integer subtraction, instead of
// the conversion unit's __float2int_rn (16 per clock per SM, three parts per
// 3D output). Same T as f64_combine.
__device__ __forceinline__ int f32_small_int(float s)
{
    return __float_as_int(__fadd_rn(s, 12582912.0f)) - 0x4B400000;
}
__device__ __forceinline__ long long f64_combine_small(const float (&lv)[6])
{
    long long t = (long long)(f32_small_int(lv[5]) >> 3);
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(t) : "r"(f32_small_int(lv[4])), "r"(1 << 6));
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(t) : "r"(f32_small_int(lv[3])), "r"(1 << 15));
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(t) : "r"(f32_small_int(lv[2])), "r"(1 << 24));
    unsigned tl, th;
    asm("mov.b64 {%0, %1}, %2;" : "=r"(tl), "=r"(th) : "l"(t));
    th += (unsigned)(f32_small_int(lv[1]) * 2 + f32_small_int(lv[0]) * 1024);
    asm("mov.b64 %0, {%1, %2};" : "=l"(t) : "r"(tl), "r"(th));
    return t;
}

// Results outside the normal FP64 range (subnormal or overflowing): FP64
// arithmetic, kept out of line so that the common path carries no FP64
// instruction (the compiler cannot if-convert a call).
static __device__ __noinline__ double f64_from_fixed_rare(long long t, int c)
{
    return scalbn((double)t, c);
}

// FP64 value of T * 2^c, rounded to nearest even: the 64-bit integer is
// converted once (cvt.rn.f64.s64, exact rounding) and the power of two is
// added to the exponent field; results outside the normal range take the
// out-of-line FP64 route.
__device__ __forceinline__ double f64_from_fixed(long long t, int c)
{
    const double d = __ll2double_rn(t);
    const long long bits = __double_as_longlong(d);
    const int e = (int)((bits >> 52) & 0x7FF);
    const int ne = e + c;
    if (e == 0) return d;  // t == 0
    if (ne >= 1 && ne <= 2046) return __longlong_as_double(bits + ((long long)c << 52));
    return f64_from_fixed_rare(t, c);
}

// Marks a tile whose window holds an Inf or NaN (its outputs become NaN).
constexpr int kNonFiniteTile = -100000;

}  // namespace tc
}  // namespace cs
