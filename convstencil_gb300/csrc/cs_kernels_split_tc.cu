// cs_kernels_split_tc.cu — dense 7x7 sweeps on the fifth-generation tensor
// cores (tcgen05.mma, accumulators in TMEM), in two number formats that share
// one pipeline:
//
//   * split precision (FmtSplit): grids of FP32 (hi, lo) pairs. Every input
//     pair of a tile is scaled by a power of two and cut into five balanced
//     9-bit digits held exactly in FP16; the weights likewise. Products of
//     digit k of x and digit e of w with k + e = L land in one FP32
//     accumulator per level L. Every product is an integer below 2^16 and a
//     level sums at most 49 * 5 of them, so each level is exact (< 2^24)
//     whatever the summation order; the five levels are recombined
//     error-free into a new (hi, lo) pair.
//   * FP64 (FmtF64): FP64 grids, the drop-in form. Each FP64 input is turned
//     into a 52-bit fixed-point integer relative to its tile's largest
//     exponent and cut into six balanced 9-bit digits with integer
//     operations only (no FP64 instruction: this GPU's FP64 pipe runs at
//     about 1/1000 of its FP16 tensor rate); the weights into six digits of a
//     fixed point below 1/4, so the top digits of both stay within 128.
//     Levels 0..5 (21 digit pairs per tap) are kept: level L sums at most
//     49 * (4 * 2^16 + 2 * 2^15) < 2^24, so each is again exact. The levels
//     are combined into one 64-bit integer and rounded once to FP64 by
//     integer operations. Error per sweep: the inputs carry 52 bits below
//     the tile maximum, the weights 53 below the largest weight, and the
//     dropped levels >= 6 weigh below 2^-48 of (tile max x largest weight)
//     in the worst case (about 2^-53 for data without adversarial digits).
//
// Mapping onto tcgen05 (M = 128, K = 16, N = 32 per level):
//   * A CTA owns a 64 x 64 output tile: 16 row groups of 4 rows, 8 blocks
//     of 8 columns. Its input window (70 x 72 points, columns x0-4 ..
//     x0+67) arrives by one 2D TMA load and is cut into digit planes in
//     shared memory, one row of 72 halves (144 bytes) per window row.
//   * Row m of the A operand is the 16-wide window of block b = m % 8 in
//     row group r = m / 8. A K-major, non-swizzled shared-memory descriptor
//     with a 16-byte K-chunk stride and a stride of four plane rows between
//     8-row groups reads exactly that sliding window out of the plane in
//     place: element (m, k) sits at plane row 4r, column 8b + k. Window row
//     offset i (0..9) is the same descriptor started i plane rows lower, so
//     no im2col copy exists.
//   * Column n of B_i is output (row 4r + rho, column 8b + c), n = 8 rho + c;
//     B_i[k][n] = w[i - rho][k - c - 1] where that tap exists, else 0.
//   * For input digit d the B operand is [B_i(e=0) | ... | B_i(e=D-1-d)]
//     (the first 32 (D-d) rows of one K-major matrix) and the accumulator
//     starts at TMEM column 32 d, so one MMA feeds levels d..D-1 at once:
//     per tile 10 offsets x D digits MMAs (50 split, 60 FP64) into 32 D FP32
//     columns.
//   * The tile shape serves as many outputs per MMA as shared memory allows:
//     4 rows per group give 4096 outputs per tile (2 rows: 2048 per 40
//     MMAs). The issuing thread stalls on each MMA until the tensor core
//     accepts it, so the MMAs are unrolled with compile-time descriptor
//     offsets (measured on GB300: 56 cycles per MMA for the split N =
//     160..32 sequence, 70 with the descriptors computed in the loop).
//   * One persistent CTA per SM (about 188 KB of shared memory split, 218 KB
//     FP64) with warp roles joined by mbarriers: one warp issues the TMA
//     window loads, one thread issues the MMAs (tcgen05.mma issue blocks
//     while the tensor core is busy, so it must not sit in anyone else's
//     barrier), eight warps read a window into registers, release the stage
//     to the next load and cut the digit planes, and four (split) or eight
//     (FP64) warps drain the accumulators, recombine and store. Two accumulators (TMEM columns 0 and
//     256) and two sets of digit planes let slicing of tile t+1, the MMAs of
//     tile t and the stores of tile t-1 run at the same time.
//
// Every mbarrier wait is bounded (WaitCfg, 2 s by default). An expired wait
// is counted in g_tc_wait_timeouts; the CTA then waits, again bounded, for
// the TMA copy and the MMAs it still has in flight, frees its TMEM and
// leaves.
#include "cs_internal.h"
#include "cs_split_common.cuh"
#include "cs_tc_common.cuh"
#include "cs_tc_f64.cuh"

#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>

namespace cs {

__device__ unsigned int g_tc_wait_timeouts;

namespace {

using split::kDigitBits;
using split::slice_digits;
using split::two_sum;
using namespace tc;

// Number formats.
// kEpiWarps: epilogue warps, one or two per TMEM lane quarter. Every warp the
// epilogue runs takes issue slots from the slicers, which bound the split
// kernel, so its light recombination runs on four warps (8192^2 on GB300:
// 192 -> 204 GStencil/s against eight); the FP64 recombination (integer
// operations) needs eight (120 GStencil/s on four, 169 on eight).
struct FmtSplit {
    static constexpr bool kF64 = false;
    static constexpr int kDigits = split::kDigits;  // 5
    static constexpr int kEpiWarps = 4;
    using Out = float2;
    using Digits = split::SliceWeights;
};

struct FmtF64 {
    static constexpr bool kF64 = true;
    static constexpr int kDigits = 6;
    static constexpr int kEpiWarps = 8;
    using Out = double;
    using Digits = F64Weights;
};

// Warp roles.
constexpr int kSliceWarps = 8;
constexpr int kWarpTma = 0, kWarpMma = 1, kWarpSlice0 = 2, kWarpEpi0 = kWarpSlice0 + kSliceWarps;
template <class F>
constexpr int kThreads = 32 * (kWarpEpi0 + F::kEpiWarps);  // 448 split, 576 FP64
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
constexpr int kAccStride = 256;            // TMEM columns between the two accumulators
constexpr int kTmemCols = 512;
constexpr unsigned kStageBytes = ST_X * ST_Y * 8;  // 40,320 (8-byte points)
// 1D row view: a tile's 70 window rows of 72 points lie in 71 array rows of 64
constexpr int kSpanRows = ST_Y + 1;
constexpr unsigned kSpanBytes = TX * kSpanRows * 8;  // 36,352
static_assert(kSpanBytes <= kStageBytes, "the span fits the stage");
constexpr int PAIRS = ST_X / 2, NPAIR = ST_Y * PAIRS;           // 36, 2,520
constexpr int PER = (NPAIR + kSliceThreads - 1) / kSliceThreads;  // 10
static_assert(FmtSplit::kEpiWarps == 4 && FmtF64::kEpiWarps == 8 && R == 4,
              "one or two epilogue warps per TMEM lane quarter, R / (warps per quarter) rows each");

template <class F>
struct Smem {
    static constexpr int D = F::kDigits;
    static constexpr int NCOL = NLV * D;       // level L at NLV * L
    static_assert(NCOL <= kAccStride, "an accumulator must fit between the two TMEM bases");
    uint4 stage[NPAIR];                        // TMA destination: pairs of 8-byte points
    __half planes[2][D][PL];                   // digit planes, two tiles
    __half bmat[NOFF][NCOL * 16];              // B_i, K-major 8x16-byte core matrices
    unsigned long long stage_full, stage_empty;
    unsigned long long planes_full[2], planes_empty[2];
    unsigned long long acc_full[2], acc_empty[2];
    unsigned tmem;                             // TMEM base column
    int abort;                                 // set by the first expired wait
    int wait_ok[2];                            // slicer leader's wait results
    int scale_exp[4];                          // per-tile input scale, ring of 4
    float red[kSliceWarps];                    // split: per-warp max |hi|
    int redi[kSliceWarps];                     // FP64: per-warp max biased exponent
};

static_assert(sizeof(Smem<FmtF64>) + 128 <= 232448 && sizeof(Smem<FmtSplit>) + 128 <= 232448,
              "shared memory of one CTA must stay within 227 KB");

// The MMAs of one tile: window row offset I, input digit DG. Descriptor
// addresses advance in 16-byte units: digit planes are PL halves apart, row
// offsets one plane row, B_i matrices NCOL * 16 halves.
template <int D, int I, int DG>
__device__ __forceinline__ void tile_mma(unsigned d_base, unsigned long long a0, unsigned long long b0)
{
    constexpr int NCOL = NLV * D;
    constexpr unsigned long long a_off = ((unsigned long long)DG * PL * 2 + I * kRowBytes) >> 4;
    constexpr unsigned long long b_off = ((unsigned long long)I * NCOL * 16 * 2) >> 4;
    static_assert(((unsigned long long)DG * PL * 2 + I * kRowBytes) % 16 == 0 && (NCOL * 16 * 2) % 16 == 0,
                  "descriptor offsets must be 16-byte multiples");
    mma_f16(d_base + (unsigned)(NLV * DG), a0 + a_off, b0 + b_off, instr_desc(NLV * (D - DG)),
            (I | DG) != 0 ? 1u : 0u);
    if constexpr (DG + 1 < D)
        tile_mma<D, I, DG + 1>(d_base, a0, b0);
    else if constexpr (I + 1 < NOFF)
        tile_mma<D, I + 1, 0>(d_base, a0, b0);
}

// One grid of a batch (batch mode): its tensor map, output, sizes, tile
// numbering and weight digits. Records live in a device array.
template <class F>
struct alignas(128) TcGrid {
    CUtensorMap map;          // window map over the source buffer
    typename F::Out *out;     // interior point (0, 0) of the destination
    long long ld;
    int m, n, tiles_x, tile_begin, map_x, map_y;
    int digits_id;            // grids with the same id have the same weights
    typename F::Digits digits;
};

// B_i: N row nn = NLV e + 8 rho + c (digit e of w, output row rho of the
// group, column c of the block), K index k; threads t0, t0 + nt, ... fill it.
template <class F>
__device__ __forceinline__ void build_bmat(Smem<F> &S, const typename F::Digits &sw, int t0, int nt)
{
    constexpr int NCOL = NLV * F::kDigits;
    for (int idx = t0; idx < NOFF * NCOL * 16; idx += nt) {
        const int i = idx / (NCOL * 16), rem = idx - i * (NCOL * 16);
        const int nn = rem >> 4, k = rem & 15;
        const int e = nn / NLV, rho = (nn % NLV) >> 3, c = nn & 7;
        const int ti = i - rho, tj = k - c - 1;
        const __half v = (ti >= 0 && ti < 7 && tj >= 0 && tj < 7) ? sw.d[e][ti * 7 + tj] : __float2half(0.f);
        S.bmat[i][(nn >> 3) * 128 + (nn & 7) * 8 + (k >> 3) * 64 + (k & 7)] = v;
    }
}

// Batch mode: the grid of global tile `tile` (last record whose tile_begin
// is not above it).
template <class F>
__device__ __forceinline__ int grid_of(const TcGrid<F> *grids, int ngrids, int tile)
{
    int lo = 0, hi = ngrids - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (grids[mid].tile_begin <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One grid (BATCH = false: kernel parameters describe it, tiles are dealt
// round-robin) or a batch of grids (BATCH = true: `grids` describes them,
// each CTA takes a contiguous run of the batch's tiles, and the MMA warp
// rebuilds its B matrices when the run crosses into the next grid, after
// the MMAs of the previous tile have completed).
template <class F, bool BATCH, bool ROWS1D = false>
__global__ void __launch_bounds__(kThreads<F>, 1)
    k2d_tc(const __grid_constant__ CUtensorMap tmap, typename F::Out *__restrict__ out, int m, int n,
           long long ld, int tiles_x, int tiles, int map_x, int map_y, typename F::Digits sw, WaitCfg wc,
           const TcGrid<F> *__restrict__ grids, int ngrids)
{
    constexpr int D = F::kDigits;
    using SM = Smem<F>;
    extern __shared__ unsigned char smem_raw[];
    SM &S = *reinterpret_cast<SM *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    pdl_allow_dependents();
    int my_tiles, first = 0;
    if constexpr (BATCH) {
        const int per = tiles / (int)gridDim.x, extra = tiles % (int)gridDim.x, b = (int)blockIdx.x;
        first = b * per + min(b, extra);
        my_tiles = per + (b < extra ? 1 : 0);
    } else {
        my_tiles = (int)blockIdx.x < tiles ? (tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    }
    // Where tile `it` of this CTA lies: its grid and output origin.
    auto tile_at = [&](int it, int &g, int &x0, int &y0) {
        if constexpr (BATCH) {
            const int tile = first + it;
            g = grid_of(grids, ngrids, tile);
            const int local = tile - grids[g].tile_begin, tx = grids[g].tiles_x;
            const int ty = local / tx;
            x0 = (local - ty * tx) * TX;
            y0 = ty * TY;
        } else {
            const int tile = blockIdx.x + it * gridDim.x;
            const int ty = tile / tiles_x;
            g = 0;
            x0 = (tile - ty * tiles_x) * TX;
            y0 = ty * TY;
        }
    };
    auto load_window = [&](int it, unsigned bar) {
        int g, x0, y0;
        tile_at(it, g, x0, y0);
        const CUtensorMap *map = &tmap;
        int mx = map_x, my = map_y;
        if constexpr (BATCH) {
            map = &grids[g].map;
            mx = grids[g].map_x;
            my = grids[g].map_y;
        }
        if constexpr (ROWS1D) {
            // 1D row view: the span of 71 array rows of 64 points from view
            // row y0 - 3 (rows outside the map read as zero)
            mbar_expect_tx(bar, kSpanBytes);
            tma_load_2d(smem_addr(S.stage), map, 0, y0 - 3, bar);
            return;
        }
        mbar_expect_tx(bar, kStageBytes);
        tma_load_2d(smem_addr(S.stage), map, mx + x0 - 4, my + y0 - 3, bar);
    };
    volatile int *abort = &S.abort;
    const unsigned stage_full = smem_addr(&S.stage_full), stage_empty = smem_addr(&S.stage_empty);
    auto bar2 = [](unsigned long long (&b)[2], int i) { return smem_addr(&b[i]); };
    const unsigned long long limit = wc.limit_ns;
    auto wait = [abort, limit](unsigned bar, unsigned parity) {
        return mbar_wait(bar, parity, abort, &g_tc_wait_timeouts, limit);
    };

    int issued = 0, committed = 0;  // window loads issued / MMA batches committed (one thread each)
    if (tid == 0) {
        mbar_init(stage_full, 1);
        mbar_init(stage_empty, kSliceWarps);
        for (int i = 0; i < 2; ++i) {
            mbar_init(bar2(S.planes_full, i), kSliceWarps);
            mbar_init(bar2(S.planes_empty, i), 1);
            mbar_init(bar2(S.acc_full, i), 1);
            mbar_init(bar2(S.acc_empty, i), F::kEpiWarps);
        }
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (my_tiles > 0 && !wc.skip_loads) {  // the first window load overlaps the set-up below
            pdl_wait();
            load_window(0, stage_full);
            issued = 1;
        }
    }
    if (warp == kWarpTma) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&S.tmem)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // B matrices of the first tile's grid (batch mode: the MMA warp rebuilds
    // them whenever its run of tiles enters another grid).
    int g_bmat = 0;
    if constexpr (BATCH) {
        if (my_tiles > 0) {
            int x0, y0;
            tile_at(0, g_bmat, x0, y0);
            build_bmat<F>(S, grids[g_bmat].digits, tid, kThreads<F>);
        }
    } else {
        build_bmat<F>(S, sw, tid, kThreads<F>);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = S.tmem;

    if (warp == kWarpTma) {
        // ------------------------------------------------ TMA producer
        if (lane == 0 && !wc.skip_loads) {
            for (int it = issued; it < my_tiles; ++it) {
                if (!wait(stage_empty, (it & 1) ^ 1)) break;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                load_window(it, stage_full);
                issued = it + 1;
            }
        }
    } else if (warp == kWarpMma) {
        // ------------------------------------------------ MMA issuer
        const unsigned long long a_desc_buf0 = smem_desc(smem_addr(S.planes[0][0]), 16, R * kRowBytes);
        const unsigned long long a_desc_buf1 = smem_desc(smem_addr(S.planes[1][0]), 16, R * kRowBytes);
        const unsigned long long b_desc0 = smem_desc(smem_addr(S.bmat[0]), 128, 256);
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it & 1, use = it >> 1;
            if constexpr (BATCH) {
                int g, x0, y0;
                tile_at(it, g, x0, y0);
                if (g != g_bmat) {
                    // New grid with other weights: once the MMAs of the
                    // previous tile (and so all earlier ones) are done reading
                    // B, the warp rewrites it. Grids that share the weights
                    // (the same digits_id) keep it.
                    if (grids[g].digits_id != grids[g_bmat].digits_id) {
                        int ok = 1;
                        if (lane == 0 && it > 0) ok = wait(bar2(S.acc_full, (it - 1) & 1), ((it - 1) >> 1) & 1);
                        if (!__shfl_sync(0xffffffffu, ok, 0)) break;
                        tc_fence_after();
                        build_bmat<F>(S, grids[g].digits, lane, 32);
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        __syncwarp();
                    }
                    g_bmat = g;
                }
            }
            int ok = 1;
            if (lane == 0) {
                ok = wait(bar2(S.planes_full, buf), use & 1) && wait(bar2(S.acc_empty, buf), (use & 1) ^ 1);
                if (ok) {
                    tc_fence_after();
                    // The issuing thread stalls on every MMA until the tensor
                    // core takes it, so nothing else sits between them: all
                    // MMAs are unrolled, each descriptor one add of a
                    // compile-time offset.
                    tile_mma<D, 0, 0>(tmem + (unsigned)(kAccStride * buf), buf ? a_desc_buf1 : a_desc_buf0,
                                      b_desc0);
                    mma_commit(bar2(S.planes_empty, buf));  // planes may be overwritten
                    mma_commit(bar2(S.acc_full, buf));      // accumulator ready
                    committed = it + 1;
                }
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) break;
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
            uint4 v[PER];
            float vmax = 0.f;   // split: largest |hi|
            unsigned emax = 0;  // FP64: largest biased exponent
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int idx = st + q * kSliceThreads;
                v[q] = make_uint4(0u, 0u, 0u, 0u);
                if (idx < NPAIR) {
                    // 1D row view: window row r (pairs 36 r ..) starts at pair
                    // 32 r of the span, the 72 points from view row y0 - 3 + r
                    if constexpr (ROWS1D)
                        v[q] = S.stage[idx - 4 * (idx / PAIRS)];
                    else
                        v[q] = S.stage[idx];
                    if constexpr (F::kF64)
                        emax = max(emax, max((v[q].y >> 20) & 0x7FFu, (v[q].w >> 20) & 0x7FFu));
                    else
                        vmax = fmaxf(vmax, fmaxf(fabsf(__uint_as_float(v[q].x)), fabsf(__uint_as_float(v[q].z))));
                }
            }
            if constexpr (F::kF64) {
                emax = __reduce_max_sync(0xffffffffu, emax);
            } else {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
            }
            __syncwarp();
            if (lane == 0) {
                if constexpr (F::kF64)
                    S.redi[warp - kWarpSlice0] = (int)emax;
                else
                    S.red[warp - kWarpSlice0] = vmax;
                mbar_arrive(stage_empty);
            }
            // (c) planes of this buffer free (MMAs two tiles back done)?
            if (leader) S.wait_ok[1] = wait(bar2(S.planes_empty, buf), (use & 1) ^ 1);
            asm volatile("bar.sync %0, %1;" ::"n"(kSliceBarrier), "n"(kSliceThreads) : "memory");
            const bool go = S.wait_ok[1];
            int ex;
            if constexpr (F::kF64) {
                int eb = S.redi[0];
#pragma unroll
                for (int i = 1; i < kSliceWarps; ++i) eb = max(eb, S.redi[i]);
                ex = max(eb, 1);
            } else {
                vmax = S.red[0];
#pragma unroll
                for (int i = 1; i < kSliceWarps; ++i) vmax = fmaxf(vmax, S.red[i]);
                ex = split::tile_exponent(vmax);
            }
            // (d) every slicer has read wait_ok[1] and the maxima before they are reused
            asm volatile("bar.sync %0, %1;" ::"n"(kSliceBarrier), "n"(kSliceThreads) : "memory");
            if (!go) break;
            if (leader) S.scale_exp[it & 3] = (F::kF64 && ex == 2047) ? kNonFiniteTile : ex;
            unsigned *dst0 = reinterpret_cast<unsigned *>(&S.planes[buf][0][0]);
            if constexpr (F::kF64) {
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int idx = st + q * kSliceThreads;
                    if (idx < NPAIR) {
                        const unsigned long long ya = f64_biased_fixed(v[q].x, v[q].y, ex);
                        const unsigned long long yb = f64_biased_fixed(v[q].z, v[q].w, ex);
                        unsigned *dst = dst0 + idx;
                        dst[0 * (PL / 2)] = f64_digit_pair<0>(ya, yb);
                        dst[1 * (PL / 2)] = f64_digit_pair<1>(ya, yb);
                        dst[2 * (PL / 2)] = f64_digit_pair<2>(ya, yb);
                        dst[3 * (PL / 2)] = f64_digit_pair<3>(ya, yb);
                        dst[4 * (PL / 2)] = f64_digit_pair<4>(ya, yb);
                        dst[5 * (PL / 2)] = f64_digit_pair<5>(ya, yb);
                    }
                }
            } else {
                const float to_digits = ldexpf(1.0f, kDigitBits - ex);
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    const int idx = st + q * kSliceThreads;
                    if (idx < NPAIR) {
                        split::f2x a, b, s2;
                        asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "r"(v[q].x), "r"(v[q].z));
                        asm("mov.b64 %0, {%1, %2};" : "=l"(b) : "r"(v[q].y), "r"(v[q].w));
                        asm("mov.b64 %0, {%1, %1};" : "=l"(s2) : "f"(to_digits));
                        unsigned wd[D];
                        split::slice_digit_pairs_x2(split::f2_mul(a, s2), split::f2_mul(b, s2), wd);
                        unsigned *dst = dst0 + idx;
#pragma unroll
                        for (int k = 0; k < D; ++k) dst[k * (PL / 2)] = wd[k];
                    }
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(bar2(S.planes_full, buf));
        }
    } else {
        // ------------------------------------------------ epilogue
        // Warp w reads TMEM lanes 32 (w % 4) ..; lane -> D row m = (row group
        // er, block eb); warp h of a quarter (one warp per quarter split,
        // two FP64) stores rows kRowsPerWarp h .. of the group, columns
        // 8 eb .. 8 eb + 7.
        const int quarter = warp & 3, h = (warp - kWarpEpi0) >> 2;
        const int mrow = 32 * quarter + lane;
        const int er = mrow >> 3, eb = mrow & 7;
        const unsigned lane_bits = (unsigned)(32 * quarter) << 16;
        for (int it = 0; it < my_tiles; ++it) {
            const int buf = it & 1, use = it >> 1;
            if (!wait(bar2(S.acc_full, buf), use & 1)) break;
            tc_fence_after();
            int g, x0, y0;
            tile_at(it, g, x0, y0);
            typename F::Out *o_base = out;
            long long o_ld = ld;
            int o_m = m, o_n = n, ew = sw.ew;
            if constexpr (BATCH) {
                o_base = grids[g].out;
                o_ld = grids[g].ld;
                o_m = grids[g].m;
                o_n = grids[g].n;
                ew = grids[g].digits.ew;
            }
            const int ex = S.scale_exp[it & 3];
            const int xb = x0 + 8 * eb;
            constexpr int kRowsPerWarp = R * 4 / F::kEpiWarps;  // 4 split, 2 FP64
#pragma unroll 1
            for (int pass = 0; pass < kRowsPerWarp; ++pass) {
                const int rho = kRowsPerWarp * h + pass;
                float acc[D][8];
#pragma unroll
                for (int L = 0; L < D; ++L)
                    tmem_ld8(tmem + lane_bits + (unsigned)(kAccStride * buf + NLV * L + 8 * rho), acc[L]);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (pass == kRowsPerWarp - 1) {  // accumulator drained: hand it back to the MMA warp
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(bar2(S.acc_empty, buf));
                }
                const int yy = y0 + R * er + rho;
                if (yy >= o_m) continue;
                if constexpr (F::kF64) {
                    // value = T 2^c with T from the levels (f64_combine) and
                    // c = (input scale) + (weight scale) - 1080.
                    const int c = ex + ew - 1080;
                    double res[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const float lv[6] = {acc[0][j], acc[1][j], acc[2][j], acc[3][j], acc[4][j], acc[5][j]};
                        res[j] = ex == kNonFiniteTile ? __longlong_as_double(0x7FF8000000000000ll)
                                                      : f64_from_fixed(f64_combine(lv), c);
                    }
                    double *o = reinterpret_cast<double *>(o_base) + (long long)yy * o_ld + xb;
#pragma unroll
                    for (int j = 0; j < 8; j += 2) {
                        if (xb + j + 1 < o_n)
                            *reinterpret_cast<double2 *>(o + j) = make_double2(res[j], res[j + 1]);
                        else if (xb + j < o_n)
                            o[j] = res[j];
                    }
                } else {
                    const float scale = ldexpf(1.0f, ex + ew - 2 * kDigitBits);
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
                    float2 *o = reinterpret_cast<float2 *>(o_base) + (long long)yy * o_ld + xb;
#pragma unroll
                    for (int j = 0; j < 8; j += 2) {
                        if (xb + j + 1 < o_n)
                            *reinterpret_cast<float4 *>(o + j) =
                                make_float4(res[j].x, res[j].y, res[j + 1].x, res[j + 1].y);
                        else if (xb + j < o_n)
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

template <class F, bool BATCH, bool ROWS1D = false>
cudaError_t set_smem_attr()
{
    static const cudaError_t err = cudaFuncSetAttribute(
        k2d_tc<F, BATCH, ROWS1D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(Smem<F>) + 128));
    return err;
}

template <class F>
cudaError_t launch_tc(const GridView &g, const typename F::Digits &digits, long long origin, long long elements,
                      const void *in_base, void *out_base, const WaitCfg &wc, cudaStream_t st)
{
    const long long ld = g.pitch[0];
    CUtensorMap map;
    // The map copies 8-byte points whatever they hold ((hi, lo) pairs or FP64).
    cudaError_t e = encode_split_window_map(&map, reinterpret_cast<const float2 *>(in_base), ld, elements / ld,
                                            ST_X, ST_Y);
    if (e != cudaSuccess) return e;
    if ((e = set_smem_attr<F, false>()) != cudaSuccess) return e;
    const int tiles_x = (int)((g.ext[1] + TX - 1) / TX);
    const int tiles = tiles_x * (int)((g.ext[0] + TY - 1) / TY);
    // One CTA per SM (its shared-memory footprint admits no second one, so
    // the TMEM allocation never waits).
    const int grid = std::min(tiles, device_sm_count());
    note_launch();
    return launch_programmatic(k2d_tc<F, false>, grid, kThreads<F>, sizeof(Smem<F>) + 128, st, map,
                               reinterpret_cast<typename F::Out *>(out_base) + origin, (int)g.ext[0],
                               (int)g.ext[1], ld, tiles_x, tiles, (int)(origin % ld), (int)(origin / ld), digits,
                               wc, static_cast<const TcGrid<F> *>(nullptr), 0);
}

template <class F>
cudaError_t fill_record(void *rec, const GridView &g, const Weights &w, long long origin, long long elements,
                        const void *in_base, void *out_base, int tile_begin, int digits_id, int *tiles,
                        typename F::Digits (*slice)(const Weights &))
{
    TcGrid<F> r;
    std::memset(&r, 0, sizeof r);
    const long long ld = g.pitch[0];
    cudaError_t e = encode_split_window_map(&r.map, reinterpret_cast<const float2 *>(in_base), ld, elements / ld,
                                            ST_X, ST_Y);
    if (e != cudaSuccess) return e;
    r.out = reinterpret_cast<typename F::Out *>(out_base) + origin;
    r.ld = ld;
    r.m = (int)g.ext[0];
    r.n = (int)g.ext[1];
    r.tiles_x = (int)((g.ext[1] + TX - 1) / TX);
    r.tile_begin = tile_begin;
    r.map_x = (int)(origin % ld);
    r.map_y = (int)(origin / ld);
    r.digits_id = digits_id;
    r.digits = slice(w);
    *tiles = r.tiles_x * (int)((g.ext[0] + TY - 1) / TY);
    std::memcpy(rec, &r, sizeof r);
    return cudaSuccess;
}

template <class F>
cudaError_t launch_batch(const void *records, int ngrids, int total, const WaitCfg &wc, cudaStream_t st)
{
    cudaError_t e = set_smem_attr<F, true>();
    if (e != cudaSuccess) return e;
    CUtensorMap unused;
    std::memset(&unused, 0, sizeof unused);
    const int grid = std::min(total, device_sm_count());
    note_launch();
    // The records were written before the previous kernel of the stream ran,
    // so the set-up may read them before pdl_wait().
    return launch_programmatic(k2d_tc<F, true>, grid, kThreads<F>, sizeof(Smem<F>) + 128, st, unused,
                               static_cast<typename F::Out *>(nullptr), 0, 0, 0LL, 0, total, 0, 0,
                               typename F::Digits{}, wc, reinterpret_cast<const TcGrid<F> *>(records), ngrids);
}

split::SliceWeights split_digits(const Weights &w) { return split::slice_weights(w); }
F64Weights f64_digits(const Weights &w) { return f64_slice_weights(w); }

}  // namespace

cudaError_t launch_split_sweep_tc(const GridView &g, const Weights &w, long long origin,
                                  long long elements, const float2 *in_base, float2 *out_base,
                                  const TcWait &wt, cudaStream_t st)
{
    return launch_tc<FmtSplit>(g, split::slice_weights(w), origin, elements, in_base, out_base,
                               WaitCfg{wt.limit_ns, wt.skip_loads}, st);
}

cudaError_t launch_fp64_sweep_tc(const GridView &g, const Weights &w, long long origin, long long elements,
                                 const double *in_base, double *out_base, const TcWait &wt, cudaStream_t st)
{
    return launch_tc<FmtF64>(g, f64_slice_weights(w), origin, elements, in_base, out_base,
                             WaitCfg{wt.limit_ns, wt.skip_loads}, st);
}

cudaError_t launch_fp64_sweep_tc_rows1d(long long n, const Weights &w7, long long origin, long long elements,
                                        const double *in_base, double *out_base, const TcWait &wt, cudaStream_t st)
{
    // Row r of the view starts at point origin - 4 + 64 r and is 72 points
    // wide: its outputs (columns 4..67) are the interior points
    // origin + 64 r .. + 63, and columns 0..3 and 68..71 their neighbours on
    // either side. The kernel sees an R x 64 grid (pitch 64); rows of the view
    // overlap by 8 points, which a tensor map cannot describe, so a tile loads
    // the span of 71 array rows of 64 points (from origin - 4, not
    // overlapping) that holds its 70 window rows, and the slicers read window
    // row r at point 64 r of the span. The taps sit in row 3 of the 7x7, so
    // the window's other rows meet zero weights. The last tile's span reaches
    // array row R (points origin + n - 4 .. origin + n + 59), so the array
    // holds 60 points after the interior; the map covers its whole rows.
    if (n % TX != 0 || n < 8 * TX || origin < 4 || origin % 2 != 0 || elements < origin + n + 60 ||
        reinterpret_cast<uintptr_t>(in_base) % 16 != 0 || reinterpret_cast<uintptr_t>(out_base) % 16 != 0)
        return cudaErrorInvalidValue;
    const long long rows = n / TX;
    CUtensorMap map;
    cudaError_t e = encode_split_window_map(&map, reinterpret_cast<const float2 *>(in_base + origin - 4), TX,
                                            (elements - (origin - 4)) / TX, TX, kSpanRows);
    if (e != cudaSuccess) return e;
    if ((e = set_smem_attr<FmtF64, false, true>()) != cudaSuccess) return e;
    const int tiles = (int)((rows + TY - 1) / TY);
    const int grid = std::min(tiles, device_sm_count());
    note_launch();
    return launch_programmatic(k2d_tc<FmtF64, false, true>, grid, kThreads<FmtF64>, sizeof(Smem<FmtF64>) + 128, st,
                               map, out_base + origin, (int)rows, TX, (long long)TX, 1, tiles, 0, 0,
                               f64_slice_weights(w7), WaitCfg{wt.limit_ns, wt.skip_loads},
                               static_cast<const TcGrid<FmtF64> *>(nullptr), 0);
}

size_t tc_batch_record_bytes(bool fp64) { return fp64 ? sizeof(TcGrid<FmtF64>) : sizeof(TcGrid<FmtSplit>); }

cudaError_t tc_batch_fill_record(bool fp64, void *rec, const GridView &g, const Weights &w, long long origin,
                                 long long elements, const void *in_base, void *out_base, int tile_begin,
                                 int digits_id, int *tiles)
{
    return fp64 ? fill_record<FmtF64>(rec, g, w, origin, elements, in_base, out_base, tile_begin, digits_id, tiles,
                                      f64_digits)
                : fill_record<FmtSplit>(rec, g, w, origin, elements, in_base, out_base, tile_begin, digits_id,
                                        tiles, split_digits);
}

cudaError_t launch_tc_batch(bool fp64, const void *records, int ngrids, int total_tiles, const TcWait &wt,
                            cudaStream_t st)
{
    const WaitCfg wc{wt.limit_ns, wt.skip_loads};
    return fp64 ? launch_batch<FmtF64>(records, ngrids, total_tiles, wc, st)
                : launch_batch<FmtSplit>(records, ngrids, total_tiles, wc, st);
}

cudaError_t split_tc_wait_timeouts(unsigned *count, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(count, g_tc_wait_timeouts, sizeof(unsigned));
    if (e != cudaSuccess || !reset) return e;
    const unsigned zero = 0;
    return cudaMemcpyToSymbol(g_tc_wait_timeouts, &zero, sizeof(unsigned));
}

}  // namespace cs
