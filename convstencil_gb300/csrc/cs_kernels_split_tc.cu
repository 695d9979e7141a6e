// cs_kernels_split_tc.cu — split-precision sweep for dense 7x7 kernels on
// the fifth-generation tensor cores (tcgen05.mma, accumulators in TMEM).
//
// Arithmetic: as in the mma.sync slice kernel (cs_kernels_split.cu). Every
// input (hi, lo) pair of a tile is scaled by a power of two and cut into five
// balanced 9-bit digits held exactly in FP16; the weights are cut the same
// way. Products of digit k of x and digit e of w with k + e = L land in one
// FP32 accumulator per level L. Every product is an integer below 2^16 and a
// level sums at most 49 * 5 of them, so each level is exact (< 2^24) whatever
// the summation order; the five levels are recombined error-free into a new
// (hi, lo) pair.
//
// Mapping onto tcgen05 (M = 128, K = 16, N = 32 per level):
//   * A CTA owns a 64 x 64 output tile: 16 row groups of 4 rows, 8 blocks
//     of 8 columns. Its input window (70 x 72 points, columns x0-4 ..
//     x0+67) arrives by one 2D TMA load and is cut into five digit planes
//     in shared memory, one row of 72 halves (144 bytes) per window row.
//   * Row m of the A operand is the 16-wide window of block b = m % 8 in
//     row group r = m / 8. A K-major, non-swizzled shared-memory descriptor
//     with a 16-byte K-chunk stride and a stride of four plane rows between
//     8-row groups reads exactly that sliding window out of the plane in
//     place: element (m, k) sits at plane row 4r, column 8b + k. Window row
//     offset i (0..9) is the same descriptor started i plane rows lower, so
//     no im2col copy exists.
//   * Column n of B_i is output (row 4r + rho, column 8b + c), n = 8 rho + c;
//     B_i[k][n] = w[i - rho][k - c - 1] where that tap exists, else 0.
//   * For input digit d the B operand is [B_i(e=0) | ... | B_i(e=4-d)] (the
//     first 32 (5-d) rows of one K-major matrix) and the accumulator starts
//     at TMEM column 32 d, so one MMA feeds levels d..4 at once: per tile
//     10 offsets x 5 digits = 50 MMAs into 160 FP32 columns.
//   * The tile shape serves as many outputs per MMA as shared memory allows:
//     4 rows per group give 4096 outputs per 50 MMAs (2 rows: 2048 per 40).
//     The issuing thread stalls on each MMA until the tensor core accepts
//     it, so the 50 MMAs are unrolled with compile-time descriptor offsets
//     (measured on GB300: 56 cycles per MMA for this N = 160..32 sequence,
//     70 with the descriptors computed in the loop).
//   * One persistent CTA per SM (about 188 KB of shared memory) with warp
//     roles joined by mbarriers: one warp issues the TMA window loads, one
//     thread issues the MMAs (tcgen05.mma issue blocks while the tensor
//     core is busy, so it must not sit in anyone else's barrier), eight
//     warps read a window into registers, release the stage to the next
//     load and cut the digit planes, and eight warps drain the accumulators,
//     recombine and store. Two accumulators (TMEM columns 0 and 256) and two
//     sets of digit planes let slicing of tile t+1, the MMAs of tile t and
//     the stores of tile t-1 run at the same time.
//
// Every mbarrier wait is bounded (2 s of %globaltimer). An expired wait is
// counted in g_tc_wait_timeouts; the CTA then waits, again bounded, for the
// TMA copy and the MMAs it still has in flight, frees its TMEM and leaves.
#include "cs_internal.h"
#include "cs_split_common.cuh"
#include "cs_tc_common.cuh"

#include <cuda.h>

#include <algorithm>
#include <mutex>

namespace cs {

__device__ unsigned int g_tc_wait_timeouts;

namespace {

using split::kDigitBits;
using split::kDigits;
using split::SliceWeights;
using split::slice_digits;
using split::two_sum;
using namespace tc;

// Warp roles.
constexpr int kSliceWarps = 8, kEpiWarps = 8;
constexpr int kWarpTma = 0, kWarpMma = 1, kWarpSlice0 = 2, kWarpEpi0 = kWarpSlice0 + kSliceWarps;
constexpr int kThreads = 32 * (kWarpEpi0 + kEpiWarps);  // 576
constexpr int kSliceThreads = 32 * kSliceWarps;
constexpr int kSliceBarrier = 1;           // named barrier of the slicer warps

constexpr int R = 4;                       // output rows per row group (N dimension)
constexpr int G = 16;                      // row groups per tile (M = G x 8 blocks = 128)
constexpr int TX = 64, TY = G * R;         // output tile 64 x 64
constexpr int ST_X = TX + 8, ST_Y = TY + 6;  // window: columns x0-4 .. x0+67, rows y0-3 .. y0+66
constexpr int PL = ST_X * ST_Y;            // halves per digit plane (10,080 bytes)
constexpr unsigned kRowBytes = ST_X * 2;   // 144
constexpr int NOFF = R + 6;                // window row offsets per row group
constexpr int NLV = 8 * R;                 // accumulator columns per level
constexpr int NCOL = NLV * kDigits;        // 160: level L at NLV * L
constexpr int kAccStride = 256;            // TMEM columns between the two accumulators
constexpr int kTmemCols = 512;
constexpr unsigned kStageBytes = ST_X * ST_Y * sizeof(float2);  // 40,320
constexpr int PAIRS = ST_X / 2, NPAIR = ST_Y * PAIRS;           // 36, 2,520
constexpr int PER = (NPAIR + kSliceThreads - 1) / kSliceThreads;  // 10
static_assert(kEpiWarps == 2 * 4 && R == 4, "two epilogue warps per TMEM lane quarter, two rows each");

struct Smem {
    float2 stage[ST_Y * ST_X];                 // TMA destination
    __half planes[2][kDigits][PL];             // digit planes, two tiles
    __half bmat[NOFF][NCOL * 16];              // B_i, K-major 8x16-byte core matrices
    unsigned long long stage_full, stage_empty;
    unsigned long long planes_full[2], planes_empty[2];
    unsigned long long acc_full[2], acc_empty[2];
    unsigned tmem;                             // TMEM base column
    int abort;                                 // set by the first expired wait
    int wait_ok[2];                            // slicer leader's wait results
    int scale_exp[4];                          // per-tile input scale, ring of 4
    float red[kSliceWarps];
};

// The MMAs of one tile: window row offset I, input digit D. Descriptor
// addresses advance in 16-byte units: digit planes are PL halves apart, row
// offsets one plane row, B_i matrices NCOL * 16 halves.
template <int I, int D>
__device__ __forceinline__ void tile_mma(unsigned d_base, unsigned long long a0, unsigned long long b0)
{
    constexpr unsigned long long a_off = ((unsigned long long)D * PL * 2 + I * kRowBytes) >> 4;
    constexpr unsigned long long b_off = ((unsigned long long)I * NCOL * 16 * 2) >> 4;
    static_assert(((unsigned long long)D * PL * 2 + I * kRowBytes) % 16 == 0 && (NCOL * 16 * 2) % 16 == 0,
                  "descriptor offsets must be 16-byte multiples");
    mma_f16(d_base + (unsigned)(NLV * D), a0 + a_off, b0 + b_off, instr_desc(NLV * (kDigits - D)),
            (I | D) != 0 ? 1u : 0u);
    if constexpr (D + 1 < kDigits)
        tile_mma<I, D + 1>(d_base, a0, b0);
    else if constexpr (I + 1 < NOFF)
        tile_mma<I + 1, 0>(d_base, a0, b0);
}

__device__ __forceinline__ void issue_tile_mmas(unsigned d_base, unsigned long long a0, unsigned long long b0)
{
    tile_mma<0, 0>(d_base, a0, b0);
}

__global__ void __launch_bounds__(kThreads, 1)
    k2d_tc(const __grid_constant__ CUtensorMap tmap, float2 *__restrict__ out, int m, int n,
           long long ld, int tiles_x, int tiles, int map_x, int map_y, SliceWeights sw)
{
    extern __shared__ unsigned char smem_raw[];
    Smem &S = *reinterpret_cast<Smem *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int my_tiles = (int)blockIdx.x < tiles ? (tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    volatile int *abort = &S.abort;
    const unsigned stage_full = smem_addr(&S.stage_full), stage_empty = smem_addr(&S.stage_empty);
    auto bar2 = [](unsigned long long (&b)[2], int i) { return smem_addr(&b[i]); };
    auto wait = [abort](unsigned bar, unsigned parity) {
        return mbar_wait(bar, parity, abort, &g_tc_wait_timeouts);
    };

    int issued = 0, committed = 0;  // window loads issued / MMA batches committed (one thread each)
    if (tid == 0) {
        mbar_init(stage_full, 1);
        mbar_init(stage_empty, kSliceWarps);
        for (int i = 0; i < 2; ++i) {
            mbar_init(bar2(S.planes_full, i), kSliceWarps);
            mbar_init(bar2(S.planes_empty, i), 1);
            mbar_init(bar2(S.acc_full, i), 1);
            mbar_init(bar2(S.acc_empty, i), kEpiWarps);
        }
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (my_tiles > 0) {  // the first window load overlaps the set-up below
            const int ty = (int)blockIdx.x / tiles_x;
            const int x0 = ((int)blockIdx.x - ty * tiles_x) * TX, y0 = ty * TY;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(stage_full),
                         "r"(kStageBytes)
                         : "memory");
            tma_load_2d(smem_addr(S.stage), &tmap, map_x + x0 - 4, map_y + y0 - 3, stage_full);
            issued = 1;
        }
    }
    if (warp == kWarpTma) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&S.tmem)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // B_i: N row nn = NLV e + 8 rho + c (digit e of w, output row rho of the
    // group, column c of the block), K index k.
    for (int idx = tid; idx < NOFF * NCOL * 16; idx += kThreads) {
        const int i = idx / (NCOL * 16), rem = idx - i * (NCOL * 16);
        const int nn = rem >> 4, k = rem & 15;
        const int e = nn / NLV, rho = (nn % NLV) >> 3, c = nn & 7;
        const int ti = i - rho, tj = k - c - 1;
        const __half v = (ti >= 0 && ti < 7 && tj >= 0 && tj < 7) ? sw.d[e][ti * 7 + tj] : __float2half(0.f);
        S.bmat[i][(nn >> 3) * 128 + (nn & 7) * 8 + (k >> 3) * 64 + (k & 7)] = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = S.tmem;
    auto tile_origin = [&](int it, int &x0, int &y0) {
        const int tile = blockIdx.x + it * gridDim.x;
        const int ty = tile / tiles_x;
        x0 = (tile - ty * tiles_x) * TX;
        y0 = ty * TY;
    };

    if (warp == kWarpTma) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            for (int it = issued; it < my_tiles; ++it) {
                if (!wait(stage_empty, (it & 1) ^ 1)) break;
                int x0, y0;
                tile_origin(it, x0, y0);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(stage_full),
                             "r"(kStageBytes)
                             : "memory");
                tma_load_2d(smem_addr(S.stage), &tmap, map_x + x0 - 4, map_y + y0 - 3, stage_full);
                issued = it + 1;
            }
        }
    } else if (warp == kWarpMma) {
        // ------------------------------------------------ MMA issuer
        const unsigned long long a_desc_buf0 = smem_desc(smem_addr(S.planes[0][0]), 16, R * kRowBytes);
        const unsigned long long a_desc_buf1 = smem_desc(smem_addr(S.planes[1][0]), 16, R * kRowBytes);
        const unsigned long long b_desc0 = smem_desc(smem_addr(S.bmat[0]), 128, 256);
        if (lane == 0) {
            for (int it = 0; it < my_tiles; ++it) {
                const int buf = it & 1, use = it >> 1;
                if (!wait(bar2(S.planes_full, buf), use & 1)) break;
                if (!wait(bar2(S.acc_empty, buf), (use & 1) ^ 1)) break;
                tc_fence_after();
                // The issuing thread stalls on every MMA until the tensor core
                // takes it, so nothing else sits between them: all 50 are
                // unrolled, each descriptor one add of a compile-time offset.
                issue_tile_mmas(tmem + (unsigned)(kAccStride * buf), buf ? a_desc_buf1 : a_desc_buf0, b_desc0);
                mma_commit(bar2(S.planes_empty, buf));  // planes may be overwritten
                mma_commit(bar2(S.acc_full, buf));      // accumulator ready
                committed = it + 1;
            }
        }
    } else if (warp < kWarpEpi0) {
        // ------------------------------------------------ slicers
        const int st = tid - 32 * kWarpSlice0;
        const bool leader = st == 0;
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it & 1, use = it >> 1;
            // (a) window landed? One thread waits, the barrier shares the answer.
            if (leader) S.wait_ok[0] = wait(stage_full, it & 1);
            asm volatile("bar.sync %0, %1;" ::"n"(kSliceBarrier), "n"(kSliceThreads) : "memory");
            if (!S.wait_ok[0]) break;
            // (b) window -> registers, then release the stage to the next load.
            const float4 *stg = reinterpret_cast<const float4 *>(S.stage);
            float4 v[PER];
            float vmax = 0.f;
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int idx = st + q * kSliceThreads;
                v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (idx < NPAIR) {
                    v[q] = stg[idx];
                    vmax = fmaxf(vmax, fmaxf(fabsf(v[q].x), fabsf(v[q].z)));
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
            __syncwarp();
            if (lane == 0) {
                S.red[warp - kWarpSlice0] = vmax;
                mbar_arrive(stage_empty);
            }
            // (c) planes of this buffer free (MMAs two tiles back done)?
            if (leader) S.wait_ok[1] = wait(bar2(S.planes_empty, buf), (use & 1) ^ 1);
            asm volatile("bar.sync %0, %1;" ::"n"(kSliceBarrier), "n"(kSliceThreads) : "memory");
            const bool go = S.wait_ok[1];
            vmax = S.red[0];
#pragma unroll
            for (int i = 1; i < kSliceWarps; ++i) vmax = fmaxf(vmax, S.red[i]);
            // (d) every slicer has read wait_ok[1] and red[] before they are reused
            asm volatile("bar.sync %0, %1;" ::"n"(kSliceBarrier), "n"(kSliceThreads) : "memory");
            if (!go) break;
            const int ex = split::tile_exponent(vmax);
            if (leader) S.scale_exp[it & 3] = ex;
            const float to_digits = ldexpf(1.0f, kDigitBits - ex);
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int idx = st + q * kSliceThreads;
                if (idx < NPAIR) {
                    float d0[kDigits], d1[kDigits];
                    slice_digits(v[q].x * to_digits, v[q].y * to_digits, d0);
                    slice_digits(v[q].z * to_digits, v[q].w * to_digits, d1);
                    unsigned *dst = reinterpret_cast<unsigned *>(&S.planes[buf][0][0]) + idx;
#pragma unroll
                    for (int k = 0; k < kDigits; ++k) dst[k * (PL / 2)] = split::pack_h2(d0[k], d1[k]);
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(bar2(S.planes_full, buf));
        }
    } else {
        // ------------------------------------------------ epilogue
        // Warp w reads TMEM lanes 32 (w % 4) ..; lane -> D row m = (row group
        // er, block eb); the two warps of a quarter store rows 2h, 2h+1 of the
        // group, columns 8 eb .. 8 eb + 7.
        const int quarter = warp & 3, h = (warp - kWarpEpi0) >> 2;
        const int mrow = 32 * quarter + lane;
        const int er = mrow >> 3, eb = mrow & 7;
        const unsigned lane_bits = (unsigned)(32 * quarter) << 16;
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it & 1, use = it >> 1;
            if (!wait(bar2(S.acc_full, buf), use & 1)) break;
            tc_fence_after();
            int x0, y0;
            tile_origin(it, x0, y0);
            const float scale = ldexpf(1.0f, S.scale_exp[it & 3] + sw.ew - 2 * kDigitBits);
            const int xb = x0 + 8 * eb;
#pragma unroll 1
            for (int pass = 0; pass < 2; ++pass) {
                const int rho = 2 * h + pass;
                float acc[kDigits][8];
#pragma unroll
                for (int L = 0; L < kDigits; ++L)
                    tmem_ld8(tmem + lane_bits + (unsigned)(kAccStride * buf + NLV * L + 8 * rho), acc[L]);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (pass == 1) {  // accumulator drained: hand it back to the MMA warp
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(bar2(S.acc_empty, buf));
                }
                const int yy = y0 + R * er + rho;
                if (yy < m) {
                    float2 res[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float h1, e1, h2, e2, hi, lo;
                        two_sum(acc[0][j], acc[1][j] * 0x1p-9f, h1, e1);
                        two_sum(h1, acc[2][j] * 0x1p-18f, h2, e2);
                        const float tail = fmaf(acc[3][j], 0x1p-27f, acc[4][j] * 0x1p-36f);
                        two_sum(h2, (e1 + e2) + tail, hi, lo);
                        res[j] = make_float2(hi * scale, lo * scale);
                    }
                    float2 *o = out + (long long)yy * ld + xb;
#pragma unroll
                    for (int j = 0; j < 8; j += 2) {
                        if (xb + j + 1 < n)
                            *reinterpret_cast<float4 *>(o + j) =
                                make_float4(res[j].x, res[j].y, res[j + 1].x, res[j + 1].y);
                        else if (xb + j < n)
                            o[j] = res[j];
                    }
                }
            }
        }
    }

    // Exit: every role is done or has given up. Let the last window load and
    // the last MMA batch finish (they have normally finished already) before
    // the shared memory and TMEM are released.
    tc_fence_before();
    __syncthreads();
    if (warp == kWarpTma && lane == 0 && issued > 0)
        mbar_drain(stage_full, (issued - 1) & 1, &g_tc_wait_timeouts);
    if (warp == kWarpMma && lane == 0 && committed > 0)
        mbar_drain(bar2(S.acc_full, (committed - 1) & 1), ((committed - 1) >> 1) & 1, &g_tc_wait_timeouts);
    __syncthreads();
    tc_fence_after();
    if (warp == kWarpTma)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

cudaError_t launch_split_sweep_tc(const GridView &g, const Weights &w, long long origin,
                                  long long elements, const float2 *in_base, float2 *out_base,
                                  cudaStream_t st)
{
    const long long ld = g.pitch[0];
    CUtensorMap map;
    cudaError_t e = encode_split_window_map(&map, in_base, ld, elements / ld, ST_X, ST_Y);
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(Smem) + 128;
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [smem] {
        attr_err = cudaFuncSetAttribute(k2d_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    if (attr_err != cudaSuccess) return attr_err;
    const int tiles_x = (int)((g.ext[1] + TX - 1) / TX);
    const int tiles = tiles_x * (int)((g.ext[0] + TY - 1) / TY);
    // One CTA per SM (its shared-memory footprint admits no second one, so
    // the TMEM allocation never waits).
    const int grid = std::min(tiles, device_sm_count());
    note_launch();
    k2d_tc<<<grid, kThreads, smem, st>>>(map, out_base + origin, (int)g.ext[0], (int)g.ext[1], ld,
                                        tiles_x, tiles, (int)(origin % ld), (int)(origin / ld),
                                        split::slice_weights(w));
    return cudaGetLastError();
}

cudaError_t split_tc_wait_timeouts(unsigned *count, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(count, g_tc_wait_timeouts, sizeof(unsigned));
    if (e != cudaSuccess || !reset) return e;
    const unsigned zero = 0;
    return cudaMemcpyToSymbol(g_tc_wait_timeouts, &zero, sizeof(unsigned));
}

}  // namespace cs
