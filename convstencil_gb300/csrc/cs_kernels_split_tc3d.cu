// cs_kernels_split_tc3d.cu — split-precision sweep for dense 3x3x3 (27-point)
// kernels on the fifth-generation tensor cores (tcgen05.mma, TMEM).
//
// Arithmetic: as in the 2D tcgen05 kernel (cs_kernels_split_tc.cu). Inputs
// (hi, lo) are scaled by a power of two per input plane of a tile and cut
// into five balanced 9-bit digits held exactly in FP16; the weights are cut
// the same way with one scale. Products of digit k of x and digit e of w with
// k + e = L land in one FP32 accumulator per level L, input plane and output
// plane; such a level sums at most 9 * 5 products below 2^16, so it is exact
// in any order, and the levels are recombined error-free into (hi, lo).
//
// Mapping (M = 128, K = 16):
//   * A work item is a column of output tiles, 16 rows x 64 columns on zc
//     consecutive planes. The CTA loads each input plane of the column once
//     (planes z0-1 .. z0+zc), by one 3D TMA load of rows y0-1 .. y0+16 and
//     columns x0-4 .. x0+67, and cuts it into five digit planes (18 rows of
//     72 halves).
//   * Row m of A is the 16-wide window of block b = m % 8 (8 output columns)
//     in output row r = m / 8: a K-major, non-swizzled descriptor with a
//     16-byte K-chunk stride and a stride of one plane row between 8-row
//     groups reads it out of the digit plane in place; window row offset i
//     (0..2) is the same descriptor started i rows lower.
//   * Input plane P feeds output planes P+1, P and P-1 as their z taps
//     dz = 0, 1, 2, and its MMAs serve all three at once: column n of B_i is
//     (weight digit e, tap plane dz, column c), n = 32 e + 8 dz + c, with
//     B[k][n] = w_e[dz][i][k - c - 3] (n with dz = 3 is zero padding that
//     keeps every level 32 columns wide). For input digit d one MMA with
//     N = 32 (5 - d) feeds levels d..4 of the plane's TMEM block: 3 row
//     offsets x 5 digits = 15 MMAs per input plane and 1024 outputs.
//   * Each input plane has its own 160-column TMEM block (ring of three,
//     columns 0, 160, 320), so every plane keeps its own scale. The epilogue
//     reads a block once, as soon as its MMAs are done, hands it back, and
//     adds its three tap-plane parts to the running sums of output planes
//     P+1 (dz = 0), P (dz = 1) and P-1 (dz = 2, its last: stored). Parts of
//     one output with the same plane scale (the usual case) are added as
//     exact level sums and recombined once; otherwise as (hi, lo) pairs
//     relative to the largest scale.
//   * Roles: one warp issues the window loads (six stage buffers), one
//     thread issues the MMAs, three groups of four warps cut every third
//     input plane into digit planes (ring of seven; a plane is too small for
//     many warps to share without waiting on each other; only the window
//     columns that meet nonzero weights are cut), and eight warps (a TMEM
//     lane quarter and half of the 8 columns each) drain the blocks,
//     recombine, scale once and store. No slicer shares the MMA thread's
//     warp scheduler.
//
// Every mbarrier wait is bounded (WaitCfg, 2 s by default). An expired wait is
// counted in g_tc3d_wait_timeouts; the CTA then waits, again bounded, for the
// TMA copies and the MMAs it still has in flight, frees its TMEM and leaves.
#include "cs_internal.h"
#include "cs_split_common.cuh"
#include "cs_tc_common.cuh"
#include "cs_tc_f64.cuh"

#include <algorithm>

namespace cs {

__device__ unsigned int g_tc3d_wait_timeouts;

namespace {

using split::kDigitBits;
using split::SliceWeights;
using split::slice_digits;
using split::two_sum;
using namespace tc;

// Number formats: split (FP32 (hi, lo) grids, five digits, a ring of three
// 160-column TMEM blocks) and FP64 (FP64 grids, six digits cut with integer
// operations as in the 2D kernel, a ring of two 192-column blocks: three do
// not fit in the 512 columns).
struct F3Split {
    static constexpr bool kF64 = false;
    static constexpr int D = split::kDigits;  // 5
    static constexpr int NBLK = 3;
    using Out = float2;
    using Digits = SliceWeights;
};
struct F3F64 {
    static constexpr bool kF64 = true;
    static constexpr int D = 6;
    static constexpr int NBLK = 2;
    using Out = double;
    using Digits = F64Weights;
};

// Warp roles. Warp w issues from the SM's scheduler w % 4, and an epilogue
// warp can read only TMEM lanes 32 (w % 4) .. + 31, so each scheduler hosts
// two epilogue warps. The MMA thread stalls on every tcgen05.mma until the
// tensor core takes it, so every issue slot it loses to a busy neighbour
// stretches the MMA stream: it shares scheduler 1 with the TMA warp, the two
// epilogue warps of lane quarter 1 and two idle warps, and the twelve slicer
// warps sit on schedulers 0, 2 and 3 (box3d1r 512^3 on GB300: 135 -> 148
// GStencil/s against slicers spread over all four). 24 warps, six per
// scheduler, leave 80 registers a thread.
constexpr int kGroups = 3, kGroupWarps = 4;  // slicer groups of four warps take every third plane
constexpr int kSliceWarps = kGroups * kGroupWarps, kEpiWarps = 8;
constexpr int kWarpTma = 1, kWarpMma = 5;
constexpr unsigned kEpiMask = (1u << 0) | (1u << 2) | (1u << 3) | (1u << 4) | (1u << 6) | (1u << 7) | (1u << 9) |
                              (1u << 13);
constexpr unsigned kSliceMask = (1u << 8) | (1u << 10) | (1u << 11) | (1u << 12) | (1u << 14) | (1u << 15) |
                                (1u << 16) | (1u << 18) | (1u << 19) | (1u << 20) | (1u << 22) | (1u << 23);
constexpr int kThreads = 32 * 24;  // warps 17 and 21 idle
constexpr int kGroupThreads = 32 * kGroupWarps;
static_assert(__builtin_popcount(kSliceMask) == kSliceWarps && __builtin_popcount(kEpiMask) == kEpiWarps &&
                  (kSliceMask & kEpiMask) == 0 && ((kSliceMask | kEpiMask) & ((1u << kWarpTma) | (1u << kWarpMma))) == 0,
              "warp roles overlap");
static_assert((kSliceMask & 0x22222222u) == 0 && (kWarpMma & 3) == 1, "no slicer beside the MMA thread");
constexpr int kSliceBarrier = 1;             // named barriers 1 .. kGroups: one per slicer group

constexpr int G = 16;                        // output rows per tile (M = G x 8 blocks = 128)
constexpr int TX = 64, TY = G;               // output tile 16 x 64
constexpr int ST_X = TX + 8, ST_Y = TY + 2;  // window: columns x0-4 .. x0+67, rows y0-1 .. y0+16
constexpr int PL = ST_X * ST_Y;              // halves per digit plane (2,592 bytes)
constexpr unsigned kRowBytes = ST_X * 2;     // 144
constexpr int NOFF = 3;                      // window row offsets
constexpr int NLV = 32;                      // TMEM columns per level: 4 tap planes (3 + padding) x 8
template <class F>
constexpr int kNcol = NLV * F::D;            // columns per input-plane block: 160 split, 192 FP64
constexpr int kTmemCols = 512;
constexpr int kStages = 2 * kGroups;         // TMA window buffers (two per slicer group)
constexpr int NPL = 7;                       // digit-plane sets (ring); also keeps one CTA per SM
constexpr int kScaleRing = 32;               // per-input-plane scale exponents (ring)
constexpr unsigned kStageBytes = ST_X * ST_Y * 8;  // 10,368 (8-byte points)
// Column pairs of a window row. Only window columns 3..68 meet a nonzero
// weight (block b reads columns 8b .. 8b+15, taps at k = c+3 .. c+5), so the
// slicers cut pairs 1..34 (columns 2..69); the digit planes' columns 0, 1, 70
// and 71 keep the zeros they are initialised with (the MMAs multiply them by
// zero weights, so they only need to be finite).
constexpr int PAIRS = ST_X / 2, CUT0 = 1, NCUTX = 34, NCUT = ST_Y * NCUTX;  // 36, 612
constexpr int PER = (NCUT + kGroupThreads - 1) / kGroupThreads;            // 5
static_assert(F3Split::NBLK * kNcol<F3Split> <= kTmemCols && F3F64::NBLK * kNcol<F3F64> <= kTmemCols,
              "TMEM blocks exceed the allocation");
static_assert(kEpiWarps == 8, "two epilogue warps per TMEM lane quarter, four columns each");
static_assert(kStageBytes % 128 == 0, "TMA destinations stay 128-byte aligned");

template <class F>
struct Smem {
    uint4 stage[kStages][ST_Y * PAIRS];        // TMA destinations: pairs of 8-byte points
    __half planes[NPL][F::D][PL];              // digit planes of input planes (ring)
    __half bmat[NOFF][kNcol<F> * 16];          // B_i, K-major 8x16-byte core matrices
    unsigned long long stage_full[kStages], stage_empty[kStages];
    unsigned long long planes_full[NPL], planes_empty[NPL];
    unsigned long long blk_full[F::NBLK], blk_empty[F::NBLK];
    unsigned tmem;                             // TMEM base column
    int abort;                                 // set by the first expired wait
    int wait_ok[kGroups][2];                   // slicer group leaders' wait results
    int scale_exp[kScaleRing];                 // input-plane scale exponents by plane sequence
    float red[kGroups][kGroupWarps];           // split: per-warp max |hi|
    int redi[kGroups][kGroupWarps];            // FP64: per-warp max biased exponent
};
static_assert(sizeof(Smem<F3F64>) + 128 <= 232448 && sizeof(Smem<F3Split>) + 128 <= 232448,
              "shared memory of one CTA must stay within 227 KB");

// The MMAs of one input plane: window row offset I, input digit D. `a`
// addresses digit 0, row 0 of the plane's digit planes; descriptor
// addresses advance in 16-byte units.
template <class F, int I, int D>
__device__ __forceinline__ void plane_mma(unsigned d_base, unsigned long long a, unsigned long long b0)
{
    constexpr int NCOL = kNcol<F>;
    constexpr unsigned long long a_off = ((unsigned long long)D * PL * 2 + I * kRowBytes) >> 4;
    constexpr unsigned long long b_off = ((unsigned long long)I * NCOL * 16 * 2) >> 4;
    static_assert(((unsigned long long)D * PL * 2 + I * kRowBytes) % 16 == 0 && (NCOL * 16 * 2) % 16 == 0,
                  "descriptor offsets must be 16-byte multiples");
    mma_f16(d_base + (unsigned)(NLV * D), a + a_off, b0 + b_off, instr_desc(NLV * (F::D - D)),
            (I | D) != 0 ? 1u : 0u);
    if constexpr (D + 1 < F::D)
        plane_mma<F, I, D + 1>(d_base, a, b0);
    else if constexpr (I + 1 < NOFF)
        plane_mma<F, I + 1, 0>(d_base, a, b0);
}

// Work item `item` of the sweep: output tile column (x0, y0) on planes
// zs .. zs + zn - 1. Items run x fastest, then y, then the plane chunk, so
// CTAs working at the same time share window rows in L2.
struct Item {
    int x0, y0, zs, zn;
};

__device__ __forceinline__ Item item_of(int item, int tiles_x, int tiles_y, int zc, int h)
{
    const int txy = tiles_x * tiles_y;
    const int chunk = item / txy, rem = item - chunk * txy;
    const int ty = rem / tiles_x;
    Item it;
    it.x0 = (rem - ty * tiles_x) * TX;
    it.y0 = ty * TY;
    it.zs = chunk * zc;
    it.zn = min(zc, h - it.zs);
    return it;
}

__device__ __forceinline__ void tmem_ld4(unsigned taddr, float (&v)[4])
{
    unsigned r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = __uint_as_float(r[j]);
}

// Recombines five exact level sums (level L in units of 2^-9L) into a
// double-float pair.
__device__ __forceinline__ void recombine(const float (&acc)[split::kDigits], float &hi, float &lo)
{
    float h1, e1, h2, e2;
    two_sum(acc[0], acc[1] * 0x1p-9f, h1, e1);
    two_sum(h1, acc[2] * 0x1p-18f, h2, e2);
    const float tail = fmaf(acc[3], 0x1p-27f, acc[4] * 0x1p-36f);
    two_sum(h2, (e1 + e2) + tail, hi, lo);
}

template <class F>
__global__ void __launch_bounds__(kThreads, 1)
    k3d_tc(const __grid_constant__ CUtensorMap tmap, typename F::Out *__restrict__ out, int h, int m, int n,
           long long ldy, long long ldz, int tiles_x, int tiles_y, int zc, int items, int map_x, int map_y,
           int map_z, typename F::Digits sw, WaitCfg wc)
{
    constexpr int D = F::D, NBLK = F::NBLK, NCOL = kNcol<F>;
    extern __shared__ unsigned char smem_raw[];
    Smem<F> &S = *reinterpret_cast<Smem<F> *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    pdl_allow_dependents();
    volatile int *abort = &S.abort;
    auto bar = [](unsigned long long *b, int i) { return smem_addr(&b[i]); };
    const unsigned long long limit = wc.limit_ns;
    auto wait = [abort, limit](unsigned b, unsigned parity) {
        return mbar_wait(b, parity, abort, &g_tc3d_wait_timeouts, limit);
    };
    const int first = blockIdx.x, step = gridDim.x;

    int issued = 0, committed = 0;  // window loads issued / input planes committed (one thread each)
    if (tid == 0) {
        for (int i = 0; i < kStages; ++i) {
            mbar_init(bar(S.stage_full, i), 1);
            mbar_init(bar(S.stage_empty, i), kGroupWarps);
        }
        for (int i = 0; i < NPL; ++i) {
            mbar_init(bar(S.planes_full, i), kGroupWarps);
            mbar_init(bar(S.planes_empty, i), 1);
        }
        for (int i = 0; i < NBLK; ++i) {
            mbar_init(bar(S.blk_full, i), 1);
            mbar_init(bar(S.blk_empty, i), kEpiWarps);
        }
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == kWarpTma) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&S.tmem)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // B_i: N row nn = NLV e + 8 dz + c (digit e of w, z tap dz, column c of
    // the block; dz = 3 is padding), K index k.
    for (int idx = tid; idx < NOFF * NCOL * 16; idx += kThreads) {
        const int i = idx / (NCOL * 16), rem = idx - i * (NCOL * 16);
        const int nn = rem >> 4, k = rem & 15;
        const int e = nn / NLV, dz = (nn % NLV) >> 3, c = nn & 7;
        const int tj = k - c - 3;
        const __half v = (dz < 3 && tj >= 0 && tj < 3) ? sw.d[e][(dz * 3 + i) * 3 + tj] : __float2half(0.f);
        S.bmat[i][(nn >> 3) * 128 + (nn & 7) * 8 + (k >> 3) * 64 + (k & 7)] = v;
    }
    for (int i = tid; i < NPL * D * PL / 2; i += kThreads)
        reinterpret_cast<unsigned *>(&S.planes[0][0][0])[i] = 0u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = S.tmem;

    if (warp == kWarpTma) {
        // ------------------------------------------------ TMA producer
        if (lane == 0 && !wc.skip_loads) {
            pdl_wait();  // the previous sweep has finished with both buffers
            int q = 0;  // input-plane sequence number
            bool ok = true;
            for (int item = first; item < items && ok; item += step) {
                const Item wi = item_of(item, tiles_x, tiles_y, zc, h);
                for (int p = 0; p < wi.zn + 2; ++p, ++q) {
                    const int sb = q % kStages;
                    if (!(ok = wait(bar(S.stage_empty, sb), ((q / kStages) & 1) ^ 1))) break;
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_expect_tx(bar(S.stage_full, sb), kStageBytes);
                    tma_load_3d(smem_addr(S.stage[sb]), &tmap, map_x + wi.x0 - 4, map_y + wi.y0 - 1,
                                map_z + wi.zs - 1 + p, bar(S.stage_full, sb));
                    issued = q + 1;
                }
            }
        }
    } else if (warp == kWarpMma) {
        // ------------------------------------------------ MMA issuer
        const unsigned long long a_desc0 = smem_desc(smem_addr(S.planes[0][0]), 16, kRowBytes);
        constexpr unsigned long long kSetUnits = (unsigned long long)D * PL * 2 / 16;
        const unsigned long long b_desc0 = smem_desc(smem_addr(S.bmat[0]), 128, 256);
        if (lane == 0) {
            int q = 0;
            bool ok = true;
            for (int item = first; item < items && ok; item += step) {
                const Item wi = item_of(item, tiles_x, tiles_y, zc, h);
                for (int p = 0; p < wi.zn + 2; ++p, ++q) {
                    const int slot = q % NPL, blk = q % NBLK;
                    if (!(ok = wait(bar(S.planes_full, slot), (q / NPL) & 1) &&
                               wait(bar(S.blk_empty, blk), ((q / NBLK) & 1) ^ 1)))
                        break;
                    tc_fence_after();
                    plane_mma<F, 0, 0>(tmem + (unsigned)(NCOL * blk), a_desc0 + kSetUnits * slot, b_desc0);
                    mma_commit(bar(S.blk_full, blk));       // block ready for the epilogue
                    mma_commit(bar(S.planes_empty, slot));  // digit planes may be overwritten
                    committed = q + 1;
                }
            }
        }
    } else if ((kSliceMask >> warp) & 1u) {
        // ------------------------------------------------ slicers
        // Group grp (four warps) cuts the planes with q % kGroups == grp, from
        // stage buffers grp and grp + kGroups; the groups work on consecutive
        // planes at the same time.
        const int sidx = __popc(kSliceMask & ((1u << warp) - 1u));  // 0 .. kSliceWarps - 1
        const int grp = sidx / kGroupWarps, gw = sidx % kGroupWarps;
        const int st = 32 * gw + lane;
        const bool leader = st == 0;
        int q = 0;
        bool go = true;
        for (int item = first; item < items && go; item += step) {
            const Item wi = item_of(item, tiles_x, tiles_y, zc, h);
            for (int p = 0; p < wi.zn + 2; ++p, ++q) {
                if (q % kGroups != grp) continue;
                const int sb = q % kStages, slot = q % NPL;
                // (a) window landed? One thread waits, the barrier shares the answer.
                if (leader) S.wait_ok[grp][0] = wait(bar(S.stage_full, sb), (q / kStages) & 1);
                asm volatile("bar.sync %0, %1;" ::"r"(kSliceBarrier + grp), "n"(kGroupThreads) : "memory");
                if (!S.wait_ok[grp][0]) {
                    go = false;
                    break;
                }
                // (b) window -> registers, then release the stage to the next load.
                const uint4 *stg = S.stage[sb];
                uint4 v[PER];
                float vmax = 0.f;   // split: largest |hi|
                unsigned emax = 0;  // FP64: largest biased exponent
#pragma unroll
                for (int k = 0; k < PER; ++k) {
                    const int u = st + k * kGroupThreads;
                    v[k] = make_uint4(0u, 0u, 0u, 0u);
                    if (u < NCUT) {
                        v[k] = stg[(u / NCUTX) * PAIRS + CUT0 + u % NCUTX];
                        if constexpr (F::kF64)
                            emax = max(emax, max((v[k].y >> 20) & 0x7FFu, (v[k].w >> 20) & 0x7FFu));
                        else
                            vmax = fmaxf(vmax, fmaxf(fabsf(__uint_as_float(v[k].x)), fabsf(__uint_as_float(v[k].z))));
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
                        S.redi[grp][gw] = (int)emax;
                    else
                        S.red[grp][gw] = vmax;
                    mbar_arrive(bar(S.stage_empty, sb));
                }
                // (c) digit-plane set free (the MMAs that read it are done)?
                if (leader) S.wait_ok[grp][1] = wait(bar(S.planes_empty, slot), ((q / NPL) & 1) ^ 1);
                asm volatile("bar.sync %0, %1;" ::"r"(kSliceBarrier + grp), "n"(kGroupThreads) : "memory");
                go = S.wait_ok[grp][1];
                int ex;
                if constexpr (F::kF64) {
                    int eb = S.redi[grp][0];
#pragma unroll
                    for (int i = 1; i < kGroupWarps; ++i) eb = max(eb, S.redi[grp][i]);
                    ex = max(eb, 1);
                } else {
                    vmax = S.red[grp][0];
#pragma unroll
                    for (int i = 1; i < kGroupWarps; ++i) vmax = fmaxf(vmax, S.red[grp][i]);
                    ex = split::tile_exponent(vmax);
                }
                // (d) every slicer of the group has read wait_ok and the maxima before they are reused
                asm volatile("bar.sync %0, %1;" ::"r"(kSliceBarrier + grp), "n"(kGroupThreads) : "memory");
                if (!go) break;
                if (leader) S.scale_exp[q % kScaleRing] = (F::kF64 && ex == 2047) ? kNonFiniteTile : ex;
                unsigned *dst0 = reinterpret_cast<unsigned *>(&S.planes[slot][0][0]);
                if constexpr (F::kF64) {
#pragma unroll
                    for (int k = 0; k < PER; ++k) {
                        const int u = st + k * kGroupThreads;
                        if (u < NCUT) {
                            const int idx = (u / NCUTX) * PAIRS + CUT0 + u % NCUTX;
                            const unsigned long long ya = f64_biased_fixed(v[k].x, v[k].y, ex);
                            const unsigned long long yb = f64_biased_fixed(v[k].z, v[k].w, ex);
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
                    for (int k = 0; k < PER; ++k) {
                        const int u = st + k * kGroupThreads;
                        if (u < NCUT) {
                            const int idx = (u / NCUTX) * PAIRS + CUT0 + u % NCUTX;
                            float d0[D], d1[D];
                            slice_digits(__uint_as_float(v[k].x) * to_digits, __uint_as_float(v[k].y) * to_digits, d0);
                            slice_digits(__uint_as_float(v[k].z) * to_digits, __uint_as_float(v[k].w) * to_digits, d1);
                            unsigned *dst = dst0 + idx;
#pragma unroll
                            for (int dg = 0; dg < D; ++dg) dst[dg * (PL / 2)] = split::pack_h2(d0[dg], d1[dg]);
                        }
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(S.planes_full, slot));
            }
        }
    } else if ((kEpiMask >> warp) & 1u) {
        // ------------------------------------------------ epilogue
        // Warp w reads TMEM lanes 32 (w % 4) ..; lane -> D row m = (output
        // row er, block eb); of the two warps of a lane quarter (w < 4 and
        // w >= 4 for quarters 0, 2, 3; 9 and 13 for quarter 1) hh = 0, 1
        // takes columns 8 eb + 4 hh .. + 3.
        // Each input plane's block is read once, as soon as its MMAs are
        // done, and handed back at once: its three tap-plane partial sums go
        // to the running sums of the output planes it feeds. Output j of the
        // column receives input plane j (dz = 0), j+1 (dz = 1) and j+2
        // (dz = 2) in that order and is stored after the last.
        const int quarter = warp & 3, hh = (warp >> 2) & 1;
        const int mrow = 32 * quarter + lane;
        const int er = mrow >> 3, eb = mrow & 7;
        const unsigned lane_bits = (unsigned)(32 * quarter) << 16;
        if constexpr (F::kF64) {
        int q0 = 0;  // first input plane of the item
        bool ok = true;
        for (int item = first; item < items && ok; item += step) {
            const Item wi = item_of(item, tiles_x, tiles_y, zc, h);
            const int xb = wi.x0 + 8 * eb + 4 * hh, yy = wi.y0 + er;
            // Running sums of outputs p - 2 (a) and p - 1 (b). A part's six
            // level sums combine into one 64-bit integer T (value T 2^c,
            // c = plane exponent + ew - 1080, as in the 2D kernel); while every
            // part of a sum had the same plane exponent (ea, eb2) the sum stays
            // an exact integer (27 taps: |T| < 2^63), rounded once at the end.
            // A part with another exponent turns the sum into an FP64 value
            // (fa, fb: the bits live in the same words); a part from a window
            // with an Inf or NaN makes the output NaN (na, nb).
            long long a[4], b[4];
            int ea = 0, eb2 = 0;
            bool fa = false, fb = false, na = false, nb = false;
            const int ew = sw.ew;
            auto part_t = [](const float (&acc)[D][4], long long (&t)[4]) {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float lv[6] = {acc[0][c], acc[1][c], acc[2][c], acc[3][c], acc[4][c], acc[5][c]};
                    t[c] = f64_combine_small(lv);  // one z tap: every level below 2^22
                }
            };
            auto add_part = [&](long long (&sm)[4], int &se, bool &fl, bool &nf, const float (&acc)[D][4],
                                int ex) {
                if (nf) return;
                if (ex == kNonFiniteTile) {
                    nf = true;
                    return;
                }
                long long t[4];
                part_t(acc, t);
                if (!fl && ex == se) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) sm[c] += t[c];
                    return;
                }
                if (!fl) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) sm[c] = __double_as_longlong(f64_from_fixed(sm[c], se + ew - 1080));
                    fl = true;
                }
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    sm[c] = __double_as_longlong(__longlong_as_double(sm[c]) + f64_from_fixed(t[c], ex + ew - 1080));
            };
            auto load_part = [&](int q, int dz, float (&acc)[D][4]) {
                const unsigned col = (unsigned)(NCOL * (q % NBLK) + 8 * dz + 4 * hh);
#pragma unroll
                for (int L = 0; L < D; ++L) tmem_ld4(tmem + lane_bits + col + NLV * L, acc[L]);
                tmem_wait_ld();
            };
            for (int p = 0; p < wi.zn + 2; ++p) {
                const int q = q0 + p;
                if (!(ok = wait(bar(S.blk_full, q % NBLK), (q / NBLK) & 1))) break;
                tc_fence_after();
                const int ex = S.scale_exp[q % kScaleRing];
                float acc[D][4];
                // z tap 2 of output p - 2: its last part; store.
                load_part(q, 2, acc);
                if (p >= 2) {
                    add_part(a, ea, fa, na, acc, ex);
                    if (yy < m) {
                        double res[4];
#pragma unroll
                        for (int c = 0; c < 4; ++c)
                            res[c] = na ? __longlong_as_double(0x7FF8000000000000ll)
                                 : fa ? __longlong_as_double(a[c])
                                      : f64_from_fixed(a[c], ea + ew - 1080);
                        double *op = out + (long long)(wi.zs + p - 2) * ldz + (long long)yy * ldy + xb;
#pragma unroll
                        for (int c = 0; c < 4; c += 2) {
                            if (xb + c + 1 < n)
                                *reinterpret_cast<double2 *>(op + c) = make_double2(res[c], res[c + 1]);
                            else if (xb + c < n)
                                op[c] = res[c];
                        }
                    }
                }
                // z tap 1 of output p - 1.
                load_part(q, 1, acc);
                if (p >= 1 && p - 1 < wi.zn) add_part(b, eb2, fb, nb, acc, ex);
                // z tap 0 of output p: its first part. The block is then
                // drained and handed back.
                load_part(q, 0, acc);
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(S.blk_empty, q % NBLK));
#pragma unroll
                for (int c = 0; c < 4; ++c) a[c] = b[c];  // rotate: p - 1 becomes p - 2, p starts
                ea = eb2;
                fa = fb;
                na = nb;
                eb2 = ex;
                fb = false;
                nb = ex == kNonFiniteTile;
                if (!nb) part_t(acc, b);
            }
            q0 += wi.zn + 2;
        }
        } else {
        int q0 = 0;  // first input plane of the item
        bool ok = true;
        for (int item = first; item < items && ok; item += step) {
            const Item wi = item_of(item, tiles_x, tiles_y, zc, h);
            const int xb = wi.x0 + 8 * eb + 4 * hh, yy = wi.y0 + er;
            // Running sums of outputs p - 2 (a) and p - 1 (b). While every
            // part added to a sum had the same plane scale (2^ea, 2^eb2), the
            // sum is kept as level sums: S0, S1, S2 exact (three parts of at
            // most 45 digit products below 2^16 each stay below 2^24) and the
            // tail T = S3 2^-27 + S4 2^-36 (its rounding weighs below 2^-50 of
            // S0's unit); the output is then recombined once. A part with
            // another scale turns the sum into a (hi, lo) pair in [0], [1]
            // relative to the largest scale seen (fa, fb set), which takes its
            // later parts as recombined pairs. Plane scales are the same for
            // the whole CTA, so the choice never diverges.
            float a[4][4], b[4][4];
            int ea = 0, eb2 = 0;
            bool fa = false, fb = false;
            auto tail = [](float s3, float s4) { return fmaf(s3, 0x1p-27f, s4 * 0x1p-36f); };
            // Level sums -> (hi, lo) in [0], [1].
            auto to_pair = [](float (&sm)[4][4]) {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float h1, e1, h2, e2, hi, lo;
                    two_sum(sm[0][c], sm[1][c] * 0x1p-9f, h1, e1);
                    two_sum(h1, sm[2][c] * 0x1p-18f, h2, e2);
                    two_sum(h2, (e1 + e2) + sm[3][c], hi, lo);
                    sm[0][c] = hi;
                    sm[1][c] = lo;
                }
            };
            // Adds a tap plane's part (five levels per column, relative to
            // 2^ex) to a running sum.
            auto add_part = [&](float (&sm)[4][4], int &se, bool &fl, const float (&acc)[D][4], int ex) {
                if (!fl && ex == se) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        sm[0][c] += acc[0][c];
                        sm[1][c] += acc[1][c];
                        sm[2][c] += acc[2][c];
                        sm[3][c] += tail(acc[3][c], acc[4][c]);
                    }
                    return;
                }
                if (!fl) to_pair(sm);
                fl = true;
                float ra = 1.0f, rb = 1.0f;
                if (ex > se) {
                    ra = ldexpf(1.0f, se - ex);
                    se = ex;
                } else {
                    rb = ldexpf(1.0f, ex - se);
                }
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float lv[D], ph, pl, s2, e2;
#pragma unroll
                    for (int L = 0; L < D; ++L) lv[L] = acc[L][c];
                    recombine(lv, ph, pl);
                    two_sum(sm[0][c] * ra, ph * rb, s2, e2);
                    sm[1][c] = sm[1][c] * ra + (e2 + pl * rb);
                    sm[0][c] = s2;
                }
            };
            auto load_part = [&](int q, int dz, float (&acc)[D][4]) {
                const unsigned col = (unsigned)(NCOL * (q % NBLK) + 8 * dz + 4 * hh);
#pragma unroll
                for (int L = 0; L < D; ++L) tmem_ld4(tmem + lane_bits + col + NLV * L, acc[L]);
                tmem_wait_ld();
            };
            for (int p = 0; p < wi.zn + 2; ++p) {
                const int q = q0 + p;
                if (!(ok = wait(bar(S.blk_full, q % NBLK), (q / NBLK) & 1))) break;
                tc_fence_after();
                const int ex = S.scale_exp[q % kScaleRing];
                float acc[D][4];
                // z tap 2 of output p - 2: its last part; store.
                load_part(q, 2, acc);
                if (p >= 2) {
                    add_part(a, ea, fa, acc, ex);
                    if (!fa) to_pair(a);
                    if (yy < m) {
                        const float scale = ldexpf(1.0f, ea + sw.ew - 2 * kDigitBits);
                        float2 res[4];
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            float hi, lo;
                            two_sum(a[0][c], a[1][c], hi, lo);
                            res[c] = make_float2(hi * scale, lo * scale);
                        }
                        float2 *op = out + (long long)(wi.zs + p - 2) * ldz + (long long)yy * ldy + xb;
#pragma unroll
                        for (int c = 0; c < 4; c += 2) {
                            if (xb + c + 1 < n)
                                *reinterpret_cast<float4 *>(op + c) =
                                    make_float4(res[c].x, res[c].y, res[c + 1].x, res[c + 1].y);
                            else if (xb + c < n)
                                op[c] = res[c];
                        }
                    }
                }
                // z tap 1 of output p - 1.
                load_part(q, 1, acc);
                if (p >= 1 && p - 1 < wi.zn) add_part(b, eb2, fb, acc, ex);
                // z tap 0 of output p: its first part. The block is then
                // drained and handed back.
                load_part(q, 0, acc);
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(S.blk_empty, q % NBLK));
#pragma unroll
                for (int c = 0; c < 4; ++c) {  // rotate: p - 1 becomes p - 2, p starts
#pragma unroll
                    for (int k = 0; k < 4; ++k) a[k][c] = b[k][c];
                    b[0][c] = acc[0][c];
                    b[1][c] = acc[1][c];
                    b[2][c] = acc[2][c];
                    b[3][c] = tail(acc[3][c], acc[4][c]);
                }
                ea = eb2;
                fa = fb;
                eb2 = ex;
                fb = false;
            }
            q0 += wi.zn + 2;
        }
        }
    }

    // Exit: every role is done or has given up. Let the last window loads and
    // the last MMA batch finish (they have normally finished already) before
    // the shared memory and TMEM are released.
    tc_fence_before();
    __syncthreads();
    if (warp == kWarpTma && lane == 0)
        for (int l = max(0, issued - kStages); l < issued; ++l)
            mbar_drain(bar(S.stage_full, l % kStages), (l / kStages) & 1, &g_tc3d_wait_timeouts);
    if (warp == kWarpMma && lane == 0 && committed > 0)
        mbar_drain(bar(S.blk_full, (committed - 1) % NBLK), ((committed - 1) / NBLK) & 1,
                   &g_tc3d_wait_timeouts);
    __syncthreads();
    tc_fence_after();
    if (warp == kWarpTma)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

}  // namespace

bool split_tc3d_layout_ok(const GridView &g, long long origin, const void *in_base, const void *out_base)
{
    if (g.dims != 3) return false;
    const long long ldy = g.pitch[1], ldz = g.pitch[0];
    return ldy % 2 == 0 && ldz % 2 == 0 && ldz % ldy == 0 && (origin % ldy) % 2 == 0 &&
           reinterpret_cast<uintptr_t>(in_base) % 16 == 0 && reinterpret_cast<uintptr_t>(out_base) % 16 == 0;
}

namespace {

template <class F>
cudaError_t launch_tc3d(const GridView &g, const typename F::Digits &digits, long long origin, long long elements,
                        const void *in_base, void *out_base, const TcWait &wt, cudaStream_t st)
{
    const long long ldy = g.pitch[1], ldz = g.pitch[0];
    CUtensorMap map;
    // The map copies 8-byte points whatever they hold ((hi, lo) pairs or FP64).
    cudaError_t e = encode_split_window_map_3d(&map, reinterpret_cast<const float2 *>(in_base), ldy, ldz,
                                               elements / ldz, ST_X, ST_Y);
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(Smem<F>) + 128;
    static const cudaError_t attr_err =
        cudaFuncSetAttribute(k3d_tc<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr_err != cudaSuccess) return attr_err;
    const int h = (int)g.ext[0], m = (int)g.ext[1], n = (int)g.ext[2];
    const int tiles_x = (n + TX - 1) / TX, tiles_y = (m + TY - 1) / TY;
    // Planes per work item: a column of zc output planes loads and cuts
    // zc + 2 input planes, and the busiest CTA takes ceil(items / SMs) items,
    // so zc (up to 32) minimises ceil(items / SMs) * (zc + 2).
    const int sms = device_sm_count();
    const long long txy = (long long)tiles_x * tiles_y;
    int zc = 1;
    long long best = -1;
    for (int c = 1; c <= std::min(32, h); ++c) {
        const long long it = txy * ((h + c - 1) / c);
        const long long cost = ((it + sms - 1) / sms) * (c + 2);
        if (best < 0 || cost < best) best = cost, zc = c;
    }
    const int items = (int)(txy * ((h + zc - 1) / zc));
    const int grid = std::min(items, sms);
    note_launch();
    return launch_programmatic(k3d_tc<F>, grid, kThreads, smem, st, map,
                               reinterpret_cast<typename F::Out *>(out_base) + origin, h, m, n, ldy, ldz, tiles_x,
                               tiles_y, zc, items, (int)(origin % ldy), (int)((origin % ldz) / ldy),
                               (int)(origin / ldz), digits, WaitCfg{wt.limit_ns, wt.skip_loads});
}

}  // namespace

cudaError_t launch_split_sweep_tc3d(const GridView &g, const Weights &w, long long origin,
                                    long long elements, const float2 *in_base, float2 *out_base,
                                    const TcWait &wt, cudaStream_t st)
{
    return launch_tc3d<F3Split>(g, split::slice_weights(w, 27), origin, elements, in_base, out_base, wt, st);
}

cudaError_t launch_fp64_sweep_tc3d(const GridView &g, const Weights &w, long long origin, long long elements,
                                   const double *in_base, double *out_base, const TcWait &wt, cudaStream_t st)
{
    return launch_tc3d<F3F64>(g, f64_slice_weights(w, 27), origin, elements, in_base, out_base, wt, st);
}

cudaError_t split_tc3d_wait_timeouts(unsigned *count, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(count, g_tc3d_wait_timeouts, sizeof(unsigned));
    if (e != cudaSuccess || !reset) return e;
    const unsigned zero = 0;
    return cudaMemcpyToSymbol(g_tc3d_wait_timeouts, &zero, sizeof(unsigned));
}

}  // namespace cs
