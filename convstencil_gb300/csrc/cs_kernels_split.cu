// cs_kernels_split.cu — split-precision sweeps: grids of FP32 (hi, lo) pairs.
//
// A value is x = hi + lo with |lo| <= ulp(hi)/2 (about 48 significant bits,
// 8 bytes per point, the same HBM traffic as FP64). GB300 runs FP32 at ~63x
// and FP16 tensor MMA at ~550x the FP64 rate, so the sweeps avoid FP64 math:
//
//  * k*_ff: double-float arithmetic on FP32 cores. Per tap: an exact product
//    of the high parts (TwoProd via FMA), an error-free TwoSum into the
//    running sum, and the cross terms hi*lo in plain FP32. About 12 FP32 ops
//    per tap; error ~2^-44 per sweep. Used for the small stencils (3 to 27
//    taps), which stay HBM-bound with it.
//
//  * k2d_mma: exact fixed-point slices on FP16 tensor cores, for dense 7x7
//    kernels (box2d3r and the reference's fused 2D kernels). Per CTA tile the
//    inputs are scaled by a power of two 2^-E so |x'| < 1/2 and cut into five
//    balanced 9-bit digits d_k (|d_k| <= 256, exact in FP16); the weights are
//    cut the same way (e_l, scale = the largest weight). A product d_k*e_l is
//    an integer of at most 16 bits, and one level s = k + l holds at most 5
//    pairs, so a level's 49-tap sum stays below 5*49*2^16 < 2^24: the FP32
//    accumulators of mma.sync.m16n8k16 hold every level EXACTLY. Levels 0..4
//    (15 pairs) are kept: 45 bits of each operand, dropped terms below ~2^-47
//    of the scale, and a weight 2^-8 below the largest still carries ~37
//    bits. The five level sums are recombined with error-free transformations
//    into a (hi, lo) pair. Outputs are 2x4 blocks: one MMA column per output
//    of a block, one MMA row per block, K = the 8x10 input window of a block
//    (80 = 5 k-steps of 16).
#include "cs_internal.h"
#include "cs_split_common.cuh"
#include "cs_split_ff.cuh"

#include <cstring>
#include <mutex>

#include <cuda_fp16.h>

#include <algorithm>

namespace cs {
namespace {

using namespace ff;
using split::kDigitBits;
using split::kDigits;
using split::MT_X;
using split::MT_Y;
using split::SL_PITCH;
using split::SL_PLANE;
using split::SL_X;
using split::SL_Y;
using split::SliceWeights;
using split::mma16816;
using split::pack_h2;
using split::slice_digits;
using split::two_sum;

// ----------------------------------------------------------- CUDA-core forms
template <int R>
__global__ void __launch_bounds__(256) k1d_ff(const float2 *__restrict__ in, float2 *__restrict__ out,
                                              long long n, FW<2 * R + 1> w)
{
    constexpr int T = 1024;
    __shared__ float2 s[T + 2 * R];
    const long long x0 = (long long)blockIdx.x * T;
    for (int i = threadIdx.x; i < T + 2 * R; i += blockDim.x) {
        const long long gx = x0 - R + i;
        s[i] = (gx < n + R) ? in[gx] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < T / 256; ++p) {
        const int lx = threadIdx.x + p * 256;
        float sh = 0.f, sl = 0.f;
#pragma unroll
        for (int t = 0; t <= 2 * R; ++t) ff_acc(t == 0, sh, sl, w.hi[t], w.lo[t], s[lx + t].x, s[lx + t].y);
        const long long gx = x0 + lx;
        if (gx < n) out[gx] = ff_finish(sh, sl);
    }
}

template <int R, int P>
__global__ void __launch_bounds__(256) k2d_ff(const float2 *__restrict__ in, float2 *__restrict__ out,
                                              int m, int n, long long ld,
                                              FW<(2 * R + 1) * (2 * R + 1)> w)
{
    constexpr int K = 2 * R + 1, TX = 64, TY = 32, RPT = 8;
    constexpr int SX = TX + 2 * R, SY = TY + 2 * R;
    __shared__ float2 s[SY * SX];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    for (int idx = threadIdx.x; idx < SY * SX; idx += blockDim.x) {
        const int sy = idx / SX, sx = idx - sy * SX;
        const int gy = y0 - R + sy, gx = x0 - R + sx;
        s[idx] = (gy < m + R && gx < n + R) ? in[(long long)gy * ld + gx] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int c = threadIdx.x & 63, g = threadIdx.x >> 6;
    float sh[RPT], sl[RPT];
#pragma unroll
    for (int o = 0; o < RPT; ++o) sh[o] = sl[o] = 0.f;
    const float2 *col = s + (g * RPT) * SX + c;
#pragma unroll
    for (int ir = 0; ir < RPT + 2 * R; ++ir) {
        float2 v[K];
#pragma unroll
        for (int j = 0; j < K; ++j) v[j] = col[ir * SX + j];
#pragma unroll
        for (int i = 0; i < K; ++i) {
            const int o = ir - i;
            if (o >= 0 && o < RPT) {
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if (tap2s<P, R>(i, j))
                        ff_acc(i * K + j == first_tap2<P, R>(), sh[o], sl[o], w.hi[i * K + j],
                               w.lo[i * K + j], v[j].x, v[j].y);
            }
        }
    }
#pragma unroll
    for (int o = 0; o < RPT; ++o) {
        const int y = y0 + g * RPT + o, x = x0 + c;
        if (y < m && x < n) out[(long long)y * ld + x] = ff_finish(sh[o], sl[o]);
    }
}

// ----------------------------------------------- temporal blocking (T steps)
// A tile plus a halo of R*T cells is loaded once; T steps run in shared
// memory, ping-ponging between two buffers, each step's region shrinking by R
// on every side. Cells outside the grid's interior are written as zero after
// every intermediate step (the Dirichlet halo), so T steps here equal T
// single-step sweeps; each output is summed in the same tap order with the
// same double-float arithmetic as k2d_ff / k1d_ff, so the results are
// bitwise identical. HBM traffic per step drops by T, compute grows by the
// recomputed halo (~10-15 % for T = 4).
//
// 2D (radius 1): a tile of (64 - 2T) x 32 outputs, so that every step's
// region (at most 64 columns) is one 64-wide row of threads, and four row
// segments of 64 threads. Each thread rolls a 3 x 3 register window down its
// rows: three shared-memory loads and no index division per output (the
// small-grid case is issue-bound: 1024^2 star2d1r 202 -> 228 GStencil/s
// against a thread-per-output mapping of 64 x 32 tiles).
template <int P, int T>
__global__ void __launch_bounds__(256) k2d_ff_tb(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                 int m, int n, long long ld, FW<9> w)
{
    constexpr int H = T, TX = 64 - 2 * T, TY = 32;
    constexpr int SX = TX + 2 * H, SY = TY + 2 * H;
    static_assert(SX == 64, "one 64-wide row of threads per step region");
    __shared__ float2 buf[2][SY * SX];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    for (int idx = threadIdx.x; idx < SY * SX; idx += blockDim.x) {
        const int sy = idx / SX, sx = idx - sy * SX;
        const int gy = y0 - H + sy, gx = x0 - H + sx;
        const bool inside = gy >= 0 && gy < m && gx >= 0 && gx < n;
        buf[0][idx] = inside ? in[(long long)gy * ld + gx] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int cx = threadIdx.x & 63, seg = threadIdx.x >> 6;
    const float2 zero = make_float2(0.f, 0.f);
    constexpr int kFirst = first_tap2<P, 1>();
#pragma unroll
    for (int t = 1; t <= T; ++t) {
        const float2 *src = buf[(t - 1) & 1];
        float2 *dst = buf[t & 1];
        constexpr int kSegs = 4;
        const int ry = SY - 2 * t, rx = SX - 2 * t, per = (ry + kSegs - 1) / kSegs;
        const int r0 = t + seg * per, r1 = min(t + ry, r0 + per);
        if (cx < rx && r0 < r1) {
            const int sx = t + cx, gx = x0 - H + sx;
            const bool xin = gx >= 0 && gx < n;
            const float2 *col = src + sx;
            float2 a0 = col[(r0 - 1) * SX - 1], a1 = col[(r0 - 1) * SX], a2 = col[(r0 - 1) * SX + 1];
            float2 b0 = col[r0 * SX - 1], b1 = col[r0 * SX], b2 = col[r0 * SX + 1];
            for (int sy = r0; sy < r1; ++sy) {
                const float2 *row = col + (sy + 1) * SX;
                const float2 c0 = row[-1], c1 = row[0], c2 = row[1];
                float sh = 0.f, sl = 0.f;
                if (tap2s<P, 1>(0, 0)) ff_acc(0 == kFirst, sh, sl, w.hi[0], w.lo[0], a0.x, a0.y);
                if (tap2s<P, 1>(0, 1)) ff_acc(1 == kFirst, sh, sl, w.hi[1], w.lo[1], a1.x, a1.y);
                if (tap2s<P, 1>(0, 2)) ff_acc(2 == kFirst, sh, sl, w.hi[2], w.lo[2], a2.x, a2.y);
                if (tap2s<P, 1>(1, 0)) ff_acc(3 == kFirst, sh, sl, w.hi[3], w.lo[3], b0.x, b0.y);
                if (tap2s<P, 1>(1, 1)) ff_acc(4 == kFirst, sh, sl, w.hi[4], w.lo[4], b1.x, b1.y);
                if (tap2s<P, 1>(1, 2)) ff_acc(5 == kFirst, sh, sl, w.hi[5], w.lo[5], b2.x, b2.y);
                if (tap2s<P, 1>(2, 0)) ff_acc(6 == kFirst, sh, sl, w.hi[6], w.lo[6], c0.x, c0.y);
                if (tap2s<P, 1>(2, 1)) ff_acc(7 == kFirst, sh, sl, w.hi[7], w.lo[7], c1.x, c1.y);
                if (tap2s<P, 1>(2, 2)) ff_acc(8 == kFirst, sh, sl, w.hi[8], w.lo[8], c2.x, c2.y);
                const int gy = y0 - H + sy;
                const bool inside = xin && gy >= 0 && gy < m;
                const float2 r = inside ? ff_finish(sh, sl) : zero;
                if (t < T) dst[sy * SX + sx] = r;
                else if (inside) out[(long long)gy * ld + gx] = r;
                a0 = b0, a1 = b1, a2 = b2;
                b0 = c0, b1 = c1, b2 = c2;
            }
        }
        if (t < T) __syncthreads();
    }
}

template <int R, int T>
__global__ void __launch_bounds__(256) k1d_ff_tb(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                 long long n, FW<2 * R + 1> w)
{
    constexpr int TX = 1024, H = R * T, SX = TX + 2 * H;
    __shared__ float2 buf[2][SX];
    const long long x0 = (long long)blockIdx.x * TX;
    for (int i = threadIdx.x; i < SX; i += blockDim.x) {
        const long long gx = x0 - H + i;
        buf[0][i] = (gx >= 0 && gx < n) ? in[gx] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int t = 1; t <= T; ++t) {
        const float2 *src = buf[(t - 1) & 1];
        float2 *dst = buf[t & 1];
        const int lo = t * R, rx = SX - 2 * lo;
        for (int k = threadIdx.x; k < rx; k += blockDim.x) {
            const int sx = lo + k;
            const long long gx = x0 - H + sx;
            float sh = 0.f, sl = 0.f;
#pragma unroll
            for (int j = 0; j < 2 * R + 1; ++j) {
                const float2 v = src[sx - R + j];
                ff_acc(j == 0, sh, sl, w.hi[j], w.lo[j], v.x, v.y);
            }
            const bool inside = gx >= 0 && gx < n;
            const float2 r = inside ? ff_finish(sh, sl) : make_float2(0.f, 0.f);
            if (t < T) dst[sx] = r;
            else if (inside) out[gx] = r;
        }
        if (t < T) __syncthreads();
    }
}

// ------------------------------------------------------- tensor-core form
// Persistent: each CTA walks tiles tile = blockIdx.x, +gridDim.x, ...; the
// weight digits are turned into per-lane B fragments once per CTA and kept in
// shared memory (one conflict-free LDS.64 per digit and k-step), which leaves
// registers for three resident CTAs per SM.
__global__ void __launch_bounds__(256, 3) k2d_mma(const float2 *__restrict__ in,
                                                  float2 *__restrict__ out, int m, int n,
                                                  long long ld, int tiles_x, int tiles,
                                                  SliceWeights sw)
{
    __shared__ __align__(16) __half sl[kDigits][SL_PLANE];
    __shared__ __align__(16) uint2 bsm[kDigits][5][32];
    __shared__ __half wd[kDigits * 49];
    __shared__ float red[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;

    for (int i = tid; i < kDigits * 49; i += blockDim.x) wd[i] = sw.d[i / 49][i % 49];
    __syncthreads();
    // B fragments (weights' digits) for lane (g, t): column n = g of the 2x4
    // block (a = g/4, b = g%4), rows kk = 16s + {2t, 2t+1, 2t+8, 2t+9};
    // B[kk][n] = w[r-a][j-b] with kk = 10r + j.
    if (warp == 0) {
        const int a = g >> 2, b = g & 3;
        for (int s = 0; s < 5; ++s) {
            unsigned reg[kDigits][2];
            for (int half = 0; half < 2; ++half) {
                float e[kDigits][2];
                for (int u = 0; u < 2; ++u) {
                    const int kk = 16 * s + 2 * t + 8 * half + u;
                    const int r = kk / 10, j = kk - 10 * r;
                    const int ri = r - a, ci = j - b;
                    const bool in_w = ri >= 0 && ri < 7 && ci >= 0 && ci < 7;
                    for (int l = 0; l < kDigits; ++l)
                        e[l][u] = in_w ? __half2float(wd[l * 49 + ri * 7 + ci]) : 0.f;
                }
                for (int l = 0; l < kDigits; ++l) reg[l][half] = pack_h2(e[l][0], e[l][1]);
            }
            for (int l = 0; l < kDigits; ++l) bsm[l][s][lane] = make_uint2(reg[l][0], reg[l][1]);
        }
    }
    // A-fragment offsets (halves) inside a slice plane for this lane: element
    // (M row = block column g or g+8, K index kk) sits at window (r, j),
    // kk = 10r + j, i.e. plane position (r, 4*block + j).
    int aoff[5][2];
#pragma unroll
    for (int s = 0; s < 5; ++s)
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int kk = 16 * s + 2 * t + 8 * half;
            const int r = kk / 10, j = kk - 10 * r;
            aoff[s][half] = r * SL_PITCH + 4 * g + j;
        }

    constexpr int PAIRS = SL_X / 2;  // 35 column pairs per tile row
    constexpr int NPAIR = SL_Y * PAIRS;
    constexpr int PER = (NPAIR + 255) / 256;

#pragma unroll 1
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
        const int x0 = tx * MT_X, y0 = ty * MT_Y;

        // 1. Load the tile (pairs of columns) and its max |hi|.
        float2 v0[PER], v1[PER];
        float vmax = 0.f;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = tid + q * 256;
            v0[q] = v1[q] = make_float2(0.f, 0.f);
            if (idx < NPAIR) {
                const int sy = idx / PAIRS, px = idx - sy * PAIRS;
                const int gy = y0 - 3 + sy, gx = x0 - 3 + 2 * px;
                if (gy < m + 3) {
                    const float2 *row = in + (long long)gy * ld;
                    if (gx < n + 3) v0[q] = row[gx];
                    if (gx + 1 < n + 3) v1[q] = row[gx + 1];
                }
                vmax = fmaxf(vmax, fmaxf(fabsf(v0[q].x), fabsf(v1[q].x)));
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        __syncthreads();  // previous tile's MMA phase is done with `sl` and `red`
        if (lane == 0) red[warp] = vmax;
        __syncthreads();
        vmax = red[0];
#pragma unroll
        for (int i = 1; i < 8; ++i) vmax = fmaxf(vmax, red[i]);
        const int ex = split::tile_exponent(vmax);
        // 2. Slice into the digit planes.
        const float to_digits = ldexpf(1.0f, kDigitBits - ex);
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = tid + q * 256;
            if (idx < NPAIR) {
                const int sy = idx / PAIRS, px = idx - sy * PAIRS;
                float d0[kDigits], d1[kDigits];
                slice_digits(v0[q].x * to_digits, v0[q].y * to_digits, d0);
                slice_digits(v1[q].x * to_digits, v1[q].y * to_digits, d1);
                unsigned *dst = reinterpret_cast<unsigned *>(&sl[0][sy * SL_PITCH + 2 * px]);
#pragma unroll
                for (int k = 0; k < kDigits; ++k) dst[k * (SL_PLANE / 2)] = pack_h2(d0[k], d1[k]);
            }
        }
        __syncthreads();

        // 3. Two M-tiles (block rows) per warp.
        const float out_scale = ldexpf(1.0f, ex + sw.ew - 2 * kDigitBits);
#pragma unroll 1
        for (int mt = 0; mt < 2; ++mt) {
            const int br = warp * 2 + mt;  // block row: output rows 2br, 2br+1
            float acc[kDigits][4];         // one exact accumulator per level k + l
#pragma unroll
            for (int lv = 0; lv < kDigits; ++lv) acc[lv][0] = acc[lv][1] = acc[lv][2] = acc[lv][3] = 0.f;
            const int rowbase = (2 * br) * SL_PITCH;
#pragma unroll
            for (int s = 0; s < 5; ++s) {
                unsigned af[kDigits][4];
#pragma unroll
                for (int k = 0; k < kDigits; ++k) {
                    const __half *plane = sl[k] + rowbase;
                    af[k][0] = *reinterpret_cast<const unsigned *>(plane + aoff[s][0]);
                    af[k][1] = *reinterpret_cast<const unsigned *>(plane + aoff[s][0] + 32);
                    af[k][2] = *reinterpret_cast<const unsigned *>(plane + aoff[s][1]);
                    af[k][3] = *reinterpret_cast<const unsigned *>(plane + aoff[s][1] + 32);
                }
                uint2 bf[kDigits];
#pragma unroll
                for (int l = 0; l < kDigits; ++l) bf[l] = bsm[l][s][lane];
#pragma unroll
                for (int lv = 0; lv < kDigits; ++lv)
#pragma unroll
                    for (int k = 0; k <= lv; ++k) mma16816(acc[lv], af[k], bf[lv - k].x, bf[lv - k].y);
            }
            // 4. Recombine T = sum_lv acc[lv] * 2^(-9 lv) (levels 0..2 through
            //    error-free sums; levels 3, 4 are below 2^-27 of level 0), and
            //    y = T * 2^(ex + ew - 18).
            float2 res[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float h1, e1, h2, e2, hi, lo;
                two_sum(acc[0][c], acc[1][c] * 0x1p-9f, h1, e1);
                two_sum(h1, acc[2][c] * 0x1p-18f, h2, e2);
                const float tail = fmaf(acc[3][c], 0x1p-27f, acc[4][c] * 0x1p-36f);
                two_sum(h2, (e1 + e2) + tail, hi, lo);
                res[c] = make_float2(hi * out_scale, lo * out_scale);
            }
            // C fragment: c0,c1 -> block g, outputs n = 2t, 2t+1; c2,c3 -> block g+8.
            const int yy = y0 + 2 * br + (t >> 1);
#pragma unroll
            for (int hb = 0; hb < 2; ++hb) {
                const int xx = x0 + 4 * (g + 8 * hb) + 2 * (t & 1);
                if (yy < m) {
                    float2 *o = out + (long long)yy * ld + xx;
                    if (xx + 1 < n) {
                        *reinterpret_cast<float4 *>(o) = make_float4(res[2 * hb].x, res[2 * hb].y,
                                                                     res[2 * hb + 1].x, res[2 * hb + 1].y);
                    } else if (xx < n) {
                        o[0] = res[2 * hb];
                    }
                }
            }
        }
    }
}

// ------------------------------------------------------------ conversions
__global__ void k_from_fp64(const double *__restrict__ src, float2 *__restrict__ dst, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = src[i];
        const float hi = __double2float_rn(v);
        const float lo = __double2float_rn(v - (double)hi);
        dst[i] = make_float2(hi, lo);
    }
}

__global__ void k_to_fp64(const float2 *__restrict__ src, double *__restrict__ dst, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 v = src[i];
        dst[i] = (double)v.x + (double)v.y;
    }
}

// In-place format changes of one buffer (FP64 re-anchor sweeps): element i
// is read and rewritten by one thread, 8 bytes either way.
__global__ void k_split_to_fp64_inplace(unsigned long long *g, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long bits = g[i];
        const float2 v = make_float2(__uint_as_float((unsigned)bits), __uint_as_float((unsigned)(bits >> 32)));
        g[i] = (unsigned long long)__double_as_longlong((double)v.x + (double)v.y);
    }
}

__global__ void k_fp64_to_split_inplace(unsigned long long *g, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double x = __longlong_as_double((long long)g[i]);
        const float hi = __double2float_rn(x);
        const float lo = __double2float_rn(x - (double)hi);
        g[i] = ((unsigned long long)__float_as_uint(lo) << 32) | __float_as_uint(hi);
    }
}

unsigned grid_for(long long n)
{
    long long b = (n + 255) / 256;
    return (unsigned)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

template <int R>
cudaError_t go1d(const GridView &g, const Weights &w, const float2 *in, float2 *out, cudaStream_t st)
{
    k1d_ff<R><<<ceil_div(g.ext[0], 1024), 256, 0, st>>>(in, out, g.ext[0], pack_ff<2 * R + 1>(w));
    return cudaGetLastError();
}

template <int R, int P>
cudaError_t go2d(const GridView &g, const Weights &w, const float2 *in, float2 *out, cudaStream_t st)
{
    constexpr int K = 2 * R + 1;
    dim3 grid(ceil_div(g.ext[1], 64), ceil_div(g.ext[0], 32));
    k2d_ff<R, P><<<grid, 256, 0, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], g.pitch[0],
                                        pack_ff<K * K>(w));
    return cudaGetLastError();
}

}  // namespace

bool split_tb_supported(int dims, int radius, int pattern)
{
    return (dims == 2 && radius == 1) || (dims == 1 && (radius == 1 || radius == 2));
}

cudaError_t launch_split_sweep_tb(const GridView &g, int R, int P, int T, const Weights &w,
                                  const float2 *in, float2 *out, cudaStream_t st)
{
    note_launch();
    if (g.dims == 1) {
        const unsigned grid = ceil_div(g.ext[0], 1024);
#define CS_TB1(RR, TT)                                                                        \
    if (R == RR && T == TT) {                                                                 \
        k1d_ff_tb<RR, TT><<<grid, 256, 0, st>>>(in, out, g.ext[0], pack_ff<2 * RR + 1>(w));   \
        return cudaGetLastError();                                                            \
    }
        CS_TB1(1, 2) CS_TB1(1, 3) CS_TB1(1, 4) CS_TB1(2, 2) CS_TB1(2, 3) CS_TB1(2, 4)
#undef CS_TB1
    } else if (g.dims == 2 && R == 1) {
#define CS_TB2(PP, TT)                                                                        \
    if (P == PP && T == TT) {                                                                 \
        dim3 grid(ceil_div(g.ext[1], 64 - 2 * TT), ceil_div(g.ext[0], 32));                   \
        k2d_ff_tb<PP, TT><<<grid, 256, 0, st>>>(in, out, (int)g.ext[0], (int)g.ext[1],         \
                                                 g.pitch[0], pack_ff<9>(w));                  \
        return cudaGetLastError();                                                            \
    }
        CS_TB2(PAT_STAR, 2) CS_TB2(PAT_STAR, 3) CS_TB2(PAT_STAR, 4)
        CS_TB2(PAT_DENSE, 2) CS_TB2(PAT_DENSE, 3) CS_TB2(PAT_DENSE, 4)
#undef CS_TB2
    }
    return cudaErrorInvalidValue;
}

bool split_supported(int dims, int radius, int pattern)
{
    if (dims == 1) return radius >= 1 && radius <= 4;
    if (dims == 2) return radius >= 1 && radius <= 3;
    if (dims == 3) return radius == 1 || radius == 3;
    return false;
}

bool split_mma_layout_ok(const GridView &g, long long origin)
{
    // float4 stores need even element offsets; the tile reads 3 halo columns.
    return g.dims == 2 && (origin % 2) == 0 && (g.pitch[0] % 2) == 0;
}

cudaError_t launch_split_sweep(const GridView &g, int R, int P, const Weights &w, int algo_mma,
                               const float2 *in, float2 *out, cudaStream_t st)
{
    note_launch();
    if (algo_mma) {
        const int tiles_x = (int)ceil_div(g.ext[1], MT_X);
        const int tiles = tiles_x * (int)ceil_div(g.ext[0], MT_Y);
        const int grid = std::min(tiles, 3 * sm_count());
        k2d_mma<<<grid, 256, 0, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], g.pitch[0], tiles_x,
                                      tiles, split::slice_weights(w));
        return cudaGetLastError();
    }
    if (g.dims == 1) {
        switch (R) {
        case 1: return go1d<1>(g, w, in, out, st);
        case 2: return go1d<2>(g, w, in, out, st);
        case 3: return go1d<3>(g, w, in, out, st);
        case 4: return go1d<4>(g, w, in, out, st);
        }
    } else if (g.dims == 2) {
        if (R == 1) {
            if (P == PAT_STAR) return go2d<1, PAT_STAR>(g, w, in, out, st);
            return go2d<1, PAT_DENSE>(g, w, in, out, st);
        }
        if (R == 2) {
            if (P == PAT_STAR) return go2d<2, PAT_STAR>(g, w, in, out, st);
            if (P == PAT_DIAMOND) return go2d<2, PAT_DIAMOND>(g, w, in, out, st);
            return go2d<2, PAT_DENSE>(g, w, in, out, st);
        }
        if (R == 3) {
            if (P == PAT_STAR) return go2d<3, PAT_STAR>(g, w, in, out, st);
            if (P == PAT_DIAMOND) return go2d<3, PAT_DIAMOND>(g, w, in, out, st);
            return go2d<3, PAT_DENSE>(g, w, in, out, st);
        }
    } else if (g.dims == 3) {
        return launch_split_sweep_3d(g, R, P, w, in, out, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_split_from_fp64(long long n, const double *src, float2 *dst, cudaStream_t st)
{
    note_launch();
    k_from_fp64<<<grid_for(n), 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_split_to_fp64(long long n, const float2 *src, double *dst, cudaStream_t st)
{
    note_launch();
    k_to_fp64<<<grid_for(n), 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_split_to_fp64_inplace(long long n, void *grid, cudaStream_t st)
{
    note_launch();
    k_split_to_fp64_inplace<<<grid_for(n), 256, 0, st>>>((unsigned long long *)grid, n);
    return cudaGetLastError();
}

cudaError_t launch_fp64_to_split_inplace(long long n, void *grid, cudaStream_t st)
{
    note_launch();
    k_fp64_to_split_inplace<<<grid_for(n), 256, 0, st>>>((unsigned long long *)grid, n);
    return cudaGetLastError();
}

}  // namespace cs
