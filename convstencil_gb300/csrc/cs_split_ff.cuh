// cs_split_ff.cuh — double-float (FP32 hi + lo) arithmetic shared by the
// CUDA-core split kernels (cs_kernels_split.cu, cs_kernels_split3d.cu):
// one tap of a double-float dot product, its packed two-lane form, the weight
// packs and the compile-time tap patterns.
#pragma once

#include <cstring>

#include "cs_internal.h"
#include "cs_split_common.cuh"

namespace cs {
namespace ff {

using split::two_sum;

// One tap of a double-float dot product: (sh, sl) += (wh + wl) * (xh + xl).
__device__ __forceinline__ void ff_tap(float &sh, float &sl, float wh, float wl, float xh, float xl)
{
    const float p = wh * xh;
    const float ep = fmaf(wh, xh, -p);  // exact error of the product
    float s, q;
    two_sum(sh, p, s, q);
    sh = s;
    sl += q;
    sl += ep;
    sl = fmaf(wh, xl, sl);
    sl = fmaf(wl, xh, sl);
}

// ff_tap into an empty sum (sh = sl = 0): the TwoSum with zero is exact, so
// only the product, its error and the two cross terms remain. Equal to
// ff_tap from (0, 0) up to the sign of a zero.
__device__ __forceinline__ void ff_first(float &sh, float &sl, float wh, float wl, float xh, float xl)
{
    sh = wh * xh;
    sl = fmaf(wh, xh, -sh);
    sl = fmaf(wh, xl, sl);
    sl = fmaf(wl, xh, sl);
}

__device__ __forceinline__ float2 ff_finish(float sh, float sl)
{
    float h, l;
    two_sum(sh, sl, h, l);
    return make_float2(h, l);
}

// ff_tap on two independent accumulators at once (f32x2). w = (wh, wh),
// nw = (-wh, -wh), wl = (wl, wl). Per lane the operations and their
// roundings are ff_tap's: -p is formed as (-wh) * xh, which rounds to exactly
// the negated product, and every use of p is rewritten around it.
__device__ __forceinline__ void ff_tap2(split::f2x &sh, split::f2x &sl, split::f2x w, split::f2x nw,
                                        split::f2x wl, split::f2x xh, split::f2x xl)
{
    using namespace split;
    const f2x np = f2_mul(nw, xh);                    // -p
    const f2x ep = f2_fma(w, xh, np);                 // exact error of the product
    const f2x s = f2_sub(sh, np);                     // sh + p
    const f2x bb = f2_sub(s, sh);
    const f2x q = f2_sub(f2_sub(sh, f2_sub(s, bb)), f2_add(np, bb));  // (sh - (s - bb)) + (p - bb)
    sh = s;
    sl = f2_add(sl, q);
    sl = f2_add(sl, ep);
    sl = f2_fma(w, xl, sl);
    sl = f2_fma(wl, xh, sl);
}

// ff_finish on both lanes.
__device__ __forceinline__ void ff_finish2(split::f2x sh, split::f2x sl, float2 &r0, float2 &r1)
{
    using namespace split;
    const f2x s = f2_add(sh, sl);
    const f2x bb = f2_sub(s, sh);
    const f2x e = f2_add(f2_sub(sh, f2_sub(s, bb)), f2_sub(sl, bb));
    f2_unpack(s, r0.x, r1.x);
    f2_unpack(e, r0.y, r1.y);
}

template <int K>
struct FW {
    float hi[K];
    float lo[K];
};

// Weights as packed pairs for ff_tap2.
template <int K>
struct FW2 {
    split::f2x w[K], nw[K], wl[K];
};

__host__ __device__ constexpr int iabs_(int x) { return x < 0 ? -x : x; }

template <int P, int R>
__host__ __device__ constexpr bool tap2s(int i, int j)
{
    return P == PAT_DENSE ? true : P == PAT_STAR ? (i == R || j == R) : (iabs_(i - R) + iabs_(j - R) <= R);
}

// Row-major index of the first tap of a 2D pattern: the tap that starts
// each output's sum (ff_first instead of ff_tap).
template <int P, int R>
__host__ __device__ constexpr int first_tap2()
{
    for (int i = 0; i < 2 * R + 1; ++i)
        for (int j = 0; j < 2 * R + 1; ++j)
            if (tap2s<P, R>(i, j)) return i * (2 * R + 1) + j;
    return 0;
}

// ff_first for the first tap of a sum, ff_tap for the others.
__device__ __forceinline__ void ff_acc(bool first, float &sh, float &sl, float wh, float wl, float xh, float xl)
{
    if (first)
        ff_first(sh, sl, wh, wl, xh, xl);
    else
        ff_tap(sh, sl, wh, wl, xh, xl);
}

template <int P, int R>
__host__ __device__ constexpr bool tap3s(int a, int i, int j)
{
    return P == PAT_DENSE ? true
           : P == PAT_STAR ? ((a != R) + (i != R) + (j != R) <= 1)
                           : (iabs_(a - R) + iabs_(i - R) + iabs_(j - R) <= R);
}

template <int K>
FW<K> pack_ff(const Weights &w)
{
    FW<K> p;
    for (int i = 0; i < K; ++i) {
        const float h = (float)w.v[i];
        p.hi[i] = h;
        p.lo[i] = (float)(w.v[i] - (double)h);
    }
    return p;
}

template <int K>
FW2<K> pack_ff2(const Weights &w)
{
    FW2<K> p;
    auto pk = [](float x) {
        unsigned u;
        std::memcpy(&u, &x, sizeof u);
        return ((split::f2x)u << 32) | u;
    };
    for (int i = 0; i < K; ++i) {
        const float hi = (float)w.v[i];
        const float lo = (float)(w.v[i] - (double)hi);
        p.w[i] = pk(hi);
        p.nw[i] = pk(-hi);
        p.wl[i] = pk(lo);
    }
    return p;
}

}  // namespace ff
}  // namespace cs
