// cs_kernels_split_tma.cu — TMA-fed split-precision sweep for dense 7x7
// kernels (the tensor-core path of box2d3r and of the reference's fused 2D
// kernels).
//
// The arithmetic is the one of k2d_mma in cs_kernels_split.cu (five exact
// 9-bit FP16 slices per operand, one exact FP32 accumulator per slice level,
// error-free recombination). What changes is how a tile reaches shared
// memory: one thread issues a 2D TMA tile load (cp.async.bulk.tensor) of the
// raw (hi, lo) tile into a staging buffer, completing on an mbarrier. The
// load of tile t+1 is issued as soon as tile t has been cut into digit
// planes, so it is in flight while the warps run tile t's MMAs. Three
// persistent CTAs per SM (about 67 KB of shared memory and 80 registers
// each) overlap one CTA's slicing with another's MMAs.
//
// Every mbarrier wait is bounded (2 s of %globaltimer); an expired wait is
// counted in g_wait_timeouts, the CTA leaves uniformly after waiting (bounded)
// for the TMA copy it issued, so a fault cannot hang the GPU. The host reads
// the counter through split_wait_timeouts().
#include "cs_internal.h"
#include "cs_split_common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

namespace cs {

__device__ unsigned int g_wait_timeouts;

namespace {

using split::kDigitBits;
using split::kDigits;
using split::MT_X;
using split::MT_Y;
using split::SL_PITCH;
using split::SL_PLANE;
using split::SliceWeights;
using split::mma16816;
using split::pack_h2;
using split::slice_digits;
using split::two_sum;

constexpr int kThreads = 256;
// TMA box: columns x0-4 .. x0+67 (x0-4 keeps the start 16-byte aligned),
// rows y0-3 .. y0+34.
constexpr int ST_X = 72, ST_Y = 38;
constexpr unsigned kStageBytes = ST_X * ST_Y * sizeof(float2);  // 21,888
constexpr unsigned long long kWaitNs = 2000000000ull;

struct Smem {
    float2 stage[ST_Y * ST_X];           // TMA destination (128-byte aligned)
    __half planes[kDigits][SL_PLANE];    // digit planes
    uint2 bsm[kDigits][5][32];           // per-lane B fragments
    __half wd[kDigits * 49];             // weight digits
    unsigned long long full;             // TMA landed
    float red[8];
};

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete; gives up after
// kWaitNs and counts the timeout.
__device__ __noinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    for (;;) {
        for (int i = 0; i < 32; ++i)
            if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer() - t0 > kWaitNs) {
            atomicAdd(&g_wait_timeouts, 1u);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap *map, int x, int y,
                                            unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__global__ void __launch_bounds__(kThreads, 3)
    k2d_mma_tma(const __grid_constant__ CUtensorMap tmap, float2 *__restrict__ out, int m, int n,
                long long ld, int tiles_x, int tiles, int map_x, int map_y, SliceWeights sw)
{
    extern __shared__ unsigned char smem_raw[];
    Smem &S = *reinterpret_cast<Smem *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const unsigned full = smem_addr(&S.full);

    auto issue = [&](int tile) {  // thread 0 only
        const int ty = tile / tiles_x;
        const int x0 = (tile - ty * tiles_x) * MT_X, y0 = ty * MT_Y;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_expect_tx(full, kStageBytes);
        tma_load_2d(smem_addr(S.stage), &tmap, map_x + x0 - 4, map_y + y0 - 3, full);
    };
    if (tid == 0) {
        mbar_init(full, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if ((int)blockIdx.x < tiles) issue(blockIdx.x);
    }
    for (int i = tid; i < kDigits * 49; i += blockDim.x) S.wd[i] = sw.d[i / 49][i % 49];
    __syncthreads();
    if (warp == 0) {  // B fragments: column n = g of the 2x4 block, rows kk = 16s + {2t,2t+1,2t+8,2t+9}
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
                        e[l][u] = in_w ? __half2float(S.wd[l * 49 + ri * 7 + ci]) : 0.f;
                }
                for (int l = 0; l < kDigits; ++l) reg[l][half] = pack_h2(e[l][0], e[l][1]);
            }
            for (int l = 0; l < kDigits; ++l) S.bsm[l][s][lane] = make_uint2(reg[l][0], reg[l][1]);
        }
    }
    int aoff[5][2];
#pragma unroll
    for (int s = 0; s < 5; ++s)
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int kk = 16 * s + 2 * t + 8 * half;
            const int r = kk / 10, j = kk - 10 * r;
            aoff[s][half] = r * SL_PITCH + 4 * g + j;
        }

    constexpr int PAIRS = (MT_X + 6) / 2, NPAIR = ST_Y * PAIRS;
    constexpr int PER = (NPAIR + kThreads - 1) / kThreads;
#pragma unroll 1
    for (int it = 0;; ++it) {
        const int tile = blockIdx.x + it * gridDim.x;
        if (tile >= tiles) break;
        const int ty = tile / tiles_x;
        const int x0 = (tile - ty * tiles_x) * MT_X, y0 = ty * MT_Y;
        // 1. Tile landed? (uniform decision across the CTA)
        const bool ok = __syncthreads_and(mbar_wait(full, it & 1));
        if (!ok) {
            if (tid == 0) mbar_wait(full, it & 1);  // bounded: let the copy finish before leaving
            return;
        }
        // 2. Read the stage (plane column p = input column x0-3+p = stage column p+1).
        float2 v0[PER], v1[PER];
        float vmax = 0.f;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = tid + q * kThreads;
            v0[q] = v1[q] = make_float2(0.f, 0.f);
            if (idx < NPAIR) {
                const int sy = idx / PAIRS, pp = idx - sy * PAIRS;
                v0[q] = S.stage[sy * ST_X + 2 * pp + 1];
                v1[q] = S.stage[sy * ST_X + 2 * pp + 2];
                vmax = fmaxf(vmax, fmaxf(fabsf(v0[q].x), fabsf(v1[q].x)));
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        if (lane == 0) S.red[warp] = vmax;
        __syncthreads();  // stage fully read; red[] complete; previous MMAs done with the planes
        if (tid == 0) {
            const int next = tile + gridDim.x;
            if (next < tiles) issue(next);  // in flight during this tile's MMAs
        }
        vmax = S.red[0];
#pragma unroll
        for (int i = 1; i < 8; ++i) vmax = fmaxf(vmax, S.red[i]);
        const int ex = split::tile_exponent(vmax);
        // 3. Slice into the digit planes.
        const float to_digits = ldexpf(1.0f, kDigitBits - ex);
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = tid + q * kThreads;
            if (idx < NPAIR) {
                const int sy = idx / PAIRS, pp = idx - sy * PAIRS;
                float d0[kDigits], d1[kDigits];
                slice_digits(v0[q].x * to_digits, v0[q].y * to_digits, d0);
                slice_digits(v1[q].x * to_digits, v1[q].y * to_digits, d1);
                unsigned *dst = reinterpret_cast<unsigned *>(&S.planes[0][sy * SL_PITCH + 2 * pp]);
#pragma unroll
                for (int k = 0; k < kDigits; ++k) dst[k * (SL_PLANE / 2)] = pack_h2(d0[k], d1[k]);
            }
        }
        __syncthreads();
        // 4. Two M-tiles (block rows) per warp.
        const float out_scale = ldexpf(1.0f, ex + sw.ew - 2 * kDigitBits);
#pragma unroll 1
        for (int mt = 0; mt < 2; ++mt) {
            const int br = warp * 2 + mt;  // block row: output rows 2br, 2br+1
            float acc[kDigits][4];
#pragma unroll
            for (int lv = 0; lv < kDigits; ++lv) acc[lv][0] = acc[lv][1] = acc[lv][2] = acc[lv][3] = 0.f;
            const int rowbase = (2 * br) * SL_PITCH;
#pragma unroll
            for (int s = 0; s < 5; ++s) {
                unsigned af[kDigits][4];
#pragma unroll
                for (int k = 0; k < kDigits; ++k) {
                    const __half *plane = S.planes[k] + rowbase;
                    af[k][0] = *reinterpret_cast<const unsigned *>(plane + aoff[s][0]);
                    af[k][1] = *reinterpret_cast<const unsigned *>(plane + aoff[s][0] + 32);
                    af[k][2] = *reinterpret_cast<const unsigned *>(plane + aoff[s][1]);
                    af[k][3] = *reinterpret_cast<const unsigned *>(plane + aoff[s][1] + 32);
                }
                uint2 bf[kDigits];
#pragma unroll
                for (int l = 0; l < kDigits; ++l) bf[l] = S.bsm[l][s][lane];
#pragma unroll
                for (int lv = 0; lv < kDigits; ++lv)
#pragma unroll
                    for (int k = 0; k <= lv; ++k) mma16816(acc[lv], af[k], bf[lv - k].x, bf[lv - k].y);
            }
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

// ----------------------------------------------------------------- host
PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

}  // namespace

int device_sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

cudaError_t encode_split_window_map(CUtensorMap *map, const float2 *base, long long ld, long long rows,
                                    unsigned box_x, unsigned box_y)
{
    auto encode = encode_fn();
    if (!encode) return cudaErrorNotSupported;
    cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * sizeof(float2))};
    cuuint32_t box[2] = {box_x, box_y};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<float2 *>(base), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// 3D form: planes of `rows` rows of pitch ld, plane pitch ldz; box
// box_x x box_y x 1.
cudaError_t encode_split_window_map_3d(CUtensorMap *map, const float2 *base, long long ld, long long ldz,
                                       long long planes, unsigned box_x, unsigned box_y)
{
    auto encode = encode_fn();
    if (!encode) return cudaErrorNotSupported;
    cuuint64_t dims[3] = {(cuuint64_t)ld, (cuuint64_t)(ldz / ld), (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)(ld * sizeof(float2)), (cuuint64_t)(ldz * sizeof(float2))};
    cuuint32_t box[3] = {box_x, box_y, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<float2 *>(base), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Rows of `width` 8-byte points that start `step` points apart (step <
// width: consecutive rows overlap), `rows` of them: a 1D array seen as a 2D
// grid whose rows carry their neighbours' points as halo. Box width x box_y.
bool split_tma_layout_ok(const GridView &g, long long origin, const void *base)
{
    if (g.dims != 2) return false;
    const long long ld = g.pitch[0];
    const long long col = origin % ld, row = origin / ld;
    return (ld % 2) == 0 && col >= 4 && (col % 2) == 0 && row >= 3 &&
           (reinterpret_cast<uintptr_t>(base) % 16) == 0;
}

cudaError_t launch_split_sweep_tma(const GridView &g, const Weights &w, long long origin,
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
        attr_err = cudaFuncSetAttribute(k2d_mma_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    if (attr_err != cudaSuccess) return attr_err;
    const int tiles_x = (int)((g.ext[1] + MT_X - 1) / MT_X);
    const int tiles = tiles_x * (int)((g.ext[0] + MT_Y - 1) / MT_Y);
    const int grid = std::min(tiles, 3 * device_sm_count());
    note_launch();
    k2d_mma_tma<<<grid, kThreads, smem, st>>>(map, out_base + origin, (int)g.ext[0], (int)g.ext[1], ld,
                                             tiles_x, tiles, (int)(origin % ld), (int)(origin / ld),
                                             split::slice_weights(w));
    return cudaGetLastError();
}

cudaError_t split_wait_timeouts(unsigned *count, bool reset)
{
    cudaError_t e = cudaMemcpyFromSymbol(count, g_wait_timeouts, sizeof(unsigned));
    if (e != cudaSuccess || !reset) return e;
    const unsigned zero = 0;
    return cudaMemcpyToSymbol(g_wait_timeouts, &zero, sizeof(unsigned));
}

}  // namespace cs
