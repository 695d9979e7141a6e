// cs_split_common.cuh — pieces shared by the split-precision kernels:
// error-free FP32 transformations, the balanced-digit slicing of (hi, lo)
// pairs and of the weights, and the FP16 mma.sync wrapper.
#pragma once

#include <cuda_fp16.h>

#include <cmath>

#include "cs_internal.h"

namespace cs {
namespace split {

// s + e == a + b exactly (Knuth's TwoSum, no ordering requirement).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// ---- packed FP32 pairs (f32x2): one instruction, two independent lanes,
// each lane rounded exactly as the scalar operation would be.
typedef unsigned long long f2x;

__device__ __forceinline__ f2x f2_add(f2x a, f2x b)
{
    f2x r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b)
{
    f2x r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b)
{
    f2x r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2_fma(f2x a, f2x b, f2x c)
{
    f2x r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2x v, float &x, float &y)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(v));
}

constexpr int kDigits = 5;       // x and w slices
constexpr int kDigitBits = 9;    // balanced base-512 digits, |d| <= 256
constexpr float kRadix = 512.f;

struct SliceWeights {
    __half d[kDigits][49];  // digits of w / 2^Ew: row-major 7x7, or 3x3x3 in the first 27
    int ew;                 // weight scale exponent: |w| < 2^(ew-1)
};

__device__ __forceinline__ void mma16816(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned pack_h2(float lo_elem, float hi_elem)
{
    const __half2 h = __floats2half2_rn(lo_elem, hi_elem);  // .x = first (lower address)
    return *reinterpret_cast<const unsigned *>(&h);
}

// Cuts x' = a + b (|a| < 256, |b| <= ulp(a)/2 after the power-of-two scaling)
// into five balanced base-512 digits. The remainder after each digit is kept
// exactly as the unevaluated pair (a - d, b): a - d is exact (both are
// multiples of a's last bit g, and |a - d| < 1 or both are integers), b stays
// below g/2, and scaling by 512 is exact, so no renormalisation is needed.
// d = rint(a + b) may differ from the exact rounding by one ulp of the sum;
// the next remainder then stays within 1/2 + 2^-24 and every digit within 256.
__device__ __forceinline__ void slice_digits(float a, float b, float (&d)[kDigits])
{
#pragma unroll
    for (int k = 0; k < kDigits - 1; ++k) {
        d[k] = rintf(a + b);
        a = (a - d[k]) * kRadix;
        b = b * kRadix;
    }
    d[kDigits - 1] = rintf(a + b);
}

// The digits of slice_digits for two points (a0 + b0, a1 + b1) at once, as
// FP16 pairs (first point in the low half), on packed FP32 pair
// instructions. rint(s) is taken as (s + M) - M with M = 1.5 * 2^23 + 512:
// for |s| < 2^22, s + M lies in [2^23, 2^24), where the FP32 spacing is 1,
// so it rounds to M + rint(s) exactly (M is even, so ties go to the same
// even integer as rint), and its low 10 mantissa bits hold 512 + d (256..768
// for |d| <= 256). FP16 (1024 + u) has the bits 0x6400 | u, so a byte
// permute and a mask-and-or build both halves, and one FP16 subtraction of
// 1536 leaves the digits exactly. Each lane of a pair instruction rounds as
// the scalar one, so the digits equal slice_digits' (a zero digit is +0).
__device__ __forceinline__ void slice_digit_pairs_x2(f2x a, f2x b, unsigned (&w)[kDigits])
{
    const f2x m2 = 0x4B4002004B400200ull;  // (M, M)
    const f2x r2 = 0x4400000044000000ull;  // (512, 512)
    const __half2 bias = __halves2half2(__ushort_as_half(0x6600), __ushort_as_half(0x6600));  // 1536
#pragma unroll
    for (int k = 0; k < kDigits; ++k) {
        const f2x t = f2_add(f2_add(a, b), m2);
        unsigned t0, t1, u;
        asm("mov.b64 {%0, %1}, %2;" : "=r"(t0), "=r"(t1) : "l"(t));
        asm("prmt.b32 %0, %1, %2, 0x5410;" : "=r"(u) : "r"(t0), "r"(t1));
        u = (u & 0x03FF03FFu) | 0x64006400u;
        const __half2 h = __hsub2(*reinterpret_cast<const __half2 *>(&u), bias);
        w[k] = *reinterpret_cast<const unsigned *>(&h);
        if (k + 1 < kDigits) {
            a = f2_mul(f2_sub(a, f2_sub(t, m2)), r2);
            b = f2_mul(b, r2);
        }
    }
}

// Scale exponent of a tile from the largest |hi| in its window: every
// |x| / 2^ex < 1/2. Clamped below at -110 so that the slicing factor
// 2^(kDigitBits - ex) stays finite in FP32; a tile whose values are all below
// 2^-111 is cut relative to 2^-110, a range where the (hi, lo) format has
// already lost its low part to underflow.
constexpr int kMinTileExp = -110;
__device__ __forceinline__ int tile_exponent(float vmax)
{
    int ex = 0;
    if (vmax > 0.f) {
        frexpf(vmax, &ex);  // vmax < 2^ex
        ex = max(ex + 1, kMinTileExp);
    }
    return ex;
}

constexpr int MT_X = 64, MT_Y = 32;              // CTA output tile
constexpr int SL_X = MT_X + 6, SL_Y = MT_Y + 6;  // input tile with radius-3 halo
// Halves per slice row. 102 halves = 51 words = 19 mod 32 banks: when the
// K indices of one A-fragment load straddle two window rows, the two rows'
// words land in disjoint banks.
constexpr int SL_PITCH = 102;
constexpr int SL_PLANE = SL_Y * SL_PITCH;


// Balanced base-512 digits of w / 2^ew for the 49 taps (exact in double);
// ew is chosen so that every |w| / 2^ew < 1/2.
// The first `taps` weights (49: a 7x7 kernel; 27: a 3x3x3 kernel), one scale.
inline SliceWeights slice_weights(const Weights &w, int taps = 49)
{
    SliceWeights s{};
    double mx = 0.0;
    for (int i = 0; i < taps; ++i) mx = std::fmax(mx, std::fabs(w.v[i]));
    int e = 0;
    if (mx > 0.0) {
        std::frexp(mx, &e);  // mx < 2^e
        e += 1;
    }
    s.ew = e;
    for (int i = 0; i < taps; ++i) {
        double a = std::ldexp(w.v[i], kDigitBits - e);
        for (int k = 0; k < kDigits; ++k) {  // balanced digits, |d| <= 256
            const double d = std::rint(a);
            s.d[k][i] = __float2half_rn((float)d);
            a = (a - d) * (double)kRadix;
        }
    }
    return s;
}

}  // namespace split
}  // namespace cs
