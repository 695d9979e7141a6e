// cs_batch.cu — uneven 2D or 3D grids packed into one persistent launch per
// sweep.
//
// A batch is a set of plans (same dims, radius, tap pattern, precision and
// steps per sweep; any sizes, weights and layouts) with their ping-pong
// buffers. One launch advances every grid of the batch by one sweep: the
// tiles of all grids (2D: 64 x 32 tiles; 3D: 32 x 16 columns of up to eight
// planes) form one list, persistent CTAs walk it, and a device table gives
// each tile its grid (pointers, sizes, pitches) and weights. Per point the
// arithmetic is the single-grid kernels' (same tap order, same FP64 FMA or
// double-float operations), so a grid's result is the same batched or alone
// (bitwise; the 3D 7-point split star alone starts its sums with ff_first,
// equal up to the sign of a zero). 2D radius-3 grids of at least 8 x 8 on
// TMA-compatible layouts run on the tcgen05 kernels instead (split or FP64,
// one record per grid with its tensor map and weight digits; equal to a
// cs_run with CS_ALGO_SPLIT_TC / CS_ALGO_FP64_TC). cs_batch_run of an even
// sweep count on a stream is captured once as a CUDA graph and replayed on
// later calls.
#include "../../include/convstencil.h"
#include "cs_internal.h"
#include "cs_plan_internal.h"
#include "cs_split_ff.cuh"

#include <algorithm>
#include <cstring>
#include <climits>
#include <map>
#include <type_traits>
#include <vector>


namespace {

using cs::GridView;
using cs::PAT_DENSE;
using cs::PAT_DIAMOND;
using cs::PAT_STAR;

struct Item {
    const void *in;  // interior point (0, 0) of the source grid
    void *out;       // interior point (0, 0) of the destination grid
    long long ld;
    int m, n, tiles_x, tile_begin;
    long long sweeps;  // sweeps this grid takes (launches for later sweeps skip its tiles)
};

constexpr int TX = 64, TY = 32, RPT = 8;

using cs::ff::tap2s;

template <class It>
__device__ __forceinline__ int find_item(const It *items, int nitems, int tile)
{
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {  // last item with tile_begin <= tile
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].tile_begin <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// FP64 FMA, the k2d_fma<R,P> body with weights from shared memory.
template <int R, int P>
__global__ void __launch_bounds__(256) k2d_fma_batch(const Item *__restrict__ items, int nitems,
                                                     const double *__restrict__ wtab, int total, long long sweep)
{
    constexpr int K = 2 * R + 1, SX = TX + 2 * R, SY = TY + 2 * R;
    __shared__ double s[SY * SX];
    __shared__ double ws[K * K];
    int cur = -1;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int it = find_item(items, nitems, tile);
        const Item I = items[it];
        if (sweep >= I.sweeps) continue;  // this grid is done (uniform over the CTA)
        const int local = tile - I.tile_begin, ty = local / I.tiles_x;
        const int x0 = (local - ty * I.tiles_x) * TX, y0 = ty * TY;
        const double *in = (const double *)I.in;
        __syncthreads();  // the previous tile is done with s[] and ws[]
        if (it != cur)
            for (int i = threadIdx.x; i < K * K; i += blockDim.x) ws[i] = wtab[it * K * K + i];
        cur = it;
        for (int idx = threadIdx.x; idx < SY * SX; idx += blockDim.x) {
            const int sy = idx / SX, sx = idx - sy * SX;
            const int gy = y0 - R + sy, gx = x0 - R + sx;
            s[idx] = (gy < I.m + R && gx < I.n + R) ? __ldg(in + (long long)gy * I.ld + gx) : 0.0;
        }
        __syncthreads();
        const int c = threadIdx.x & 63, g = threadIdx.x >> 6;
        double acc[RPT];
#pragma unroll
        for (int o = 0; o < RPT; ++o) acc[o] = 0.0;
        const double *col = s + (g * RPT) * SX + c;
#pragma unroll
        for (int ir = 0; ir < RPT + 2 * R; ++ir) {
            double v[K];
#pragma unroll
            for (int j = 0; j < K; ++j) v[j] = col[ir * SX + j];
#pragma unroll
            for (int i = 0; i < K; ++i) {
                const int o = ir - i;
                if (o >= 0 && o < RPT) {
#pragma unroll
                    for (int j = 0; j < K; ++j)
                        if (tap2s<P, R>(i, j)) acc[o] = fma(ws[i * K + j], v[j], acc[o]);
                }
            }
        }
        double *out = (double *)I.out;
#pragma unroll
        for (int o = 0; o < RPT; ++o) {
            const int y = y0 + g * RPT + o, x = x0 + c;
            if (y < I.m && x < I.n) out[(long long)y * I.ld + x] = acc[o];
        }
    }
}

// Split precision, double-float on FP32 cores: the k2d_ff<R,P> body.
template <int R, int P>
__global__ void __launch_bounds__(256) k2d_ff_batch(const Item *__restrict__ items, int nitems,
                                                    const float2 *__restrict__ wtab, int total, long long sweep)
{
    constexpr int K = 2 * R + 1, SX = TX + 2 * R, SY = TY + 2 * R;
    __shared__ float2 s[SY * SX];
    __shared__ float2 ws[K * K];  // (hi, lo) per tap
    int cur = -1;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int it = find_item(items, nitems, tile);
        const Item I = items[it];
        if (sweep >= I.sweeps) continue;  // this grid is done (uniform over the CTA)
        const int local = tile - I.tile_begin, ty = local / I.tiles_x;
        const int x0 = (local - ty * I.tiles_x) * TX, y0 = ty * TY;
        const float2 *in = (const float2 *)I.in;
        __syncthreads();
        if (it != cur)
            for (int i = threadIdx.x; i < K * K; i += blockDim.x) ws[i] = wtab[it * K * K + i];
        cur = it;
        for (int idx = threadIdx.x; idx < SY * SX; idx += blockDim.x) {
            const int sy = idx / SX, sx = idx - sy * SX;
            const int gy = y0 - R + sy, gx = x0 - R + sx;
            s[idx] = (gy < I.m + R && gx < I.n + R) ? in[(long long)gy * I.ld + gx] : make_float2(0.f, 0.f);
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
                        if (tap2s<P, R>(i, j)) {
                            const float2 wv = ws[i * K + j];
                            cs::ff::ff_acc(i * K + j == cs::ff::first_tap2<P, R>(), sh[o], sl[o], wv.x, wv.y,
                                           v[j].x, v[j].y);
                        }
                }
            }
        }
        float2 *out = (float2 *)I.out;
#pragma unroll
        for (int o = 0; o < RPT; ++o) {
            const int y = y0 + g * RPT + o, x = x0 + c;
            if (y < I.m && x < I.n) {
                float h, l;
                cs::split::two_sum(sh[o], sl[o], h, l);
                out[(long long)y * I.ld + x] = make_float2(h, l);
            }
        }
    }
}

// ---- 3D: a work unit is a 32 x 16 column of one grid over zc planes.
struct Item3 {
    const void *in;  // interior point (0, 0, 0) of the source grid
    void *out;
    long long ldy, ldz;
    int h, m, n, tiles_x, tiles_y, zc, tile_begin;
    long long sweeps;  // sweeps this grid takes (launches for later sweeps skip its tiles)
};

constexpr int TX3 = 32, TY3 = 16, ZC3 = 8;

template <int R>
constexpr int k3d_batch_smem(bool split)
{
    return ((2 * R + 1) * (TX3 + 2 * R) * (TY3 + 2 * R) + (2 * R + 1) * (2 * R + 1) * (2 * R + 1)) *
           (split ? (int)sizeof(float2) : (int)sizeof(double));
}

// Per point, the k3d_fma (FP64) or k3d_ff1 (split) sum: taps in (dz, dy, dx)
// order from zero, weights from shared memory.
template <int R, int P, bool SPLIT>
__global__ void __launch_bounds__(256) k3d_batch(const Item3 *__restrict__ items, int nitems,
                                                 const void *__restrict__ wtab, int total, long long sweep)
{
    using T = typename std::conditional<SPLIT, float2, double>::type;
    constexpr int K = 2 * R + 1, SX = TX3 + 2 * R, SY = TY3 + 2 * R, PL = SX * SY, KK = K * K * K;
    extern __shared__ unsigned char b3_raw[];
    T *ring = reinterpret_cast<T *>(b3_raw);
    T *ws = ring + K * PL;
    const T *wt = reinterpret_cast<const T *>(wtab);
    int cur = -1;
    for (int unit = blockIdx.x; unit < total; unit += gridDim.x) {
        const int it = find_item(items, nitems, unit);
        const Item3 I = items[it];
        if (sweep >= I.sweeps) continue;  // this grid is done (uniform over the CTA)
        const int local = unit - I.tile_begin, txy = I.tiles_x * I.tiles_y;
        const int tz = local / txy, rem = local - tz * txy, ty = rem / I.tiles_x;
        const int x0 = (rem - ty * I.tiles_x) * TX3, y0 = ty * TY3, z0 = tz * I.zc;
        const int zend = min(z0 + I.zc, I.h);
        const T *in = reinterpret_cast<const T *>(I.in);
        T *out = reinterpret_cast<T *>(I.out);
        __syncthreads();  // the previous unit is done with ring[] and ws[]
        if (it != cur)
            for (int i = threadIdx.x; i < KK; i += blockDim.x) ws[i] = wt[(long long)it * KK + i];
        cur = it;
        auto load_plane = [&](int gz) {  // gz in [-R, h + R)
            T *dst = ring + ((gz + K) % K) * PL;
            const bool zok = gz < I.h + R;
            for (int idx = threadIdx.x; idx < PL; idx += blockDim.x) {
                const int sy = idx / SX, sx = idx - sy * SX;
                const int gy = y0 - R + sy, gx = x0 - R + sx;
                T v;
                if constexpr (SPLIT)
                    v = make_float2(0.f, 0.f);
                else
                    v = 0.0;
                if (zok && gy < I.m + R && gx < I.n + R) v = in[(long long)gz * I.ldz + (long long)gy * I.ldy + gx];
                dst[idx] = v;
            }
        };
        for (int gz = z0 - R; gz < z0 + R; ++gz) load_plane(gz);
        const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
        for (int z = z0; z < zend; ++z) {
            load_plane(z + R);
            __syncthreads();
#pragma unroll 1
            for (int q = 0; q < 2; ++q) {
                const int ly = ly0 + 8 * q;
                double acc = 0.0;
                float sh = 0.f, sl = 0.f;
#pragma unroll(R == 1 ? K : 1)
                for (int a = 0; a < K; ++a) {
                    const T *pl = ring + ((z - R + a + K) % K) * PL + ly * SX + lx;
#pragma unroll
                    for (int i = 0; i < K; ++i)
#pragma unroll
                        for (int j = 0; j < K; ++j)
                            if (cs::ff::tap3s<P, R>(a, i, j)) {
                                const int t = (a * K + i) * K + j;
                                if constexpr (SPLIT) {
                                    const float2 v = pl[i * SX + j], wv = ws[t];
                                    cs::ff::ff_tap(sh, sl, wv.x, wv.y, v.x, v.y);
                                } else {
                                    acc = fma(ws[t], pl[i * SX + j], acc);
                                }
                            }
                }
                const int y = y0 + ly, x = x0 + lx;
                if (y < I.m && x < I.n) {
                    T r;
                    if constexpr (SPLIT)
                        r = cs::ff::ff_finish(sh, sl);
                    else
                        r = acc;
                    out[(long long)z * I.ldz + (long long)y * I.ldy + x] = r;
                }
            }
            __syncthreads();
        }
    }
}

template <class KernelT>
int persistent_grid(KernelT kernel, int total)
{
    int dev = 0, sms = 1, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, 0);
    return std::max(1, std::min(total, sms * std::max(1, per)));
}

template <int R, int P>
cudaError_t launch_batch(bool split, const Item *items, int nitems, const void *wtab, int total,
                         long long sweep, cudaStream_t st)
{
    cs::note_launch();
    if (split) {
        const int grid = persistent_grid(k2d_ff_batch<R, P>, total);
        k2d_ff_batch<R, P><<<grid, 256, 0, st>>>(items, nitems, (const float2 *)wtab, total, sweep);
    } else {
        const int grid = persistent_grid(k2d_fma_batch<R, P>, total);
        k2d_fma_batch<R, P><<<grid, 256, 0, st>>>(items, nitems, (const double *)wtab, total, sweep);
    }
    return cudaGetLastError();
}

cudaError_t dispatch(int R, int P, bool split, const Item *items, int nitems, const void *wtab, int total,
                     long long sweep, cudaStream_t st)
{
    if (R == 1) return P == PAT_STAR ? launch_batch<1, PAT_STAR>(split, items, nitems, wtab, total, sweep, st)
                                     : launch_batch<1, PAT_DENSE>(split, items, nitems, wtab, total, sweep, st);
    if (R == 2) {
        if (P == PAT_STAR) return launch_batch<2, PAT_STAR>(split, items, nitems, wtab, total, sweep, st);
        if (P == PAT_DIAMOND) return launch_batch<2, PAT_DIAMOND>(split, items, nitems, wtab, total, sweep, st);
        return launch_batch<2, PAT_DENSE>(split, items, nitems, wtab, total, sweep, st);
    }
    if (R == 3) {
        if (P == PAT_STAR) return launch_batch<3, PAT_STAR>(split, items, nitems, wtab, total, sweep, st);
        if (P == PAT_DIAMOND) return launch_batch<3, PAT_DIAMOND>(split, items, nitems, wtab, total, sweep, st);
        return launch_batch<3, PAT_DENSE>(split, items, nitems, wtab, total, sweep, st);
    }
    return cudaErrorInvalidValue;
}

template <int R, int P, bool SPLIT>
cudaError_t launch_batch3(const Item3 *items, int nitems, const void *wtab, int total, long long sweep,
                          cudaStream_t st)
{
    constexpr int smem = k3d_batch_smem<R>(SPLIT);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k3d_batch<R, P, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (attr != cudaSuccess) return attr;
    int dev = 0, sms = 1, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k3d_batch<R, P, SPLIT>, 256, smem);
    const int grid = std::max(1, std::min(total, sms * std::max(1, per)));
    cs::note_launch();
    k3d_batch<R, P, SPLIT><<<grid, 256, smem, st>>>(items, nitems, wtab, total, sweep);
    return cudaGetLastError();
}

template <bool SPLIT>
cudaError_t dispatch3s(int R, int P, const Item3 *items, int nitems, const void *wtab, int total, long long sweep,
                       cudaStream_t st)
{
    if (R == 1) return P == PAT_STAR ? launch_batch3<1, PAT_STAR, SPLIT>(items, nitems, wtab, total, sweep, st)
                                     : launch_batch3<1, PAT_DENSE, SPLIT>(items, nitems, wtab, total, sweep, st);
    if (R == 3) {
        if (P == PAT_STAR) return launch_batch3<3, PAT_STAR, SPLIT>(items, nitems, wtab, total, sweep, st);
        if (P == PAT_DIAMOND) return launch_batch3<3, PAT_DIAMOND, SPLIT>(items, nitems, wtab, total, sweep, st);
        return launch_batch3<3, PAT_DENSE, SPLIT>(items, nitems, wtab, total, sweep, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t dispatch3(int R, int P, bool split, const Item3 *items, int nitems, const void *wtab, int total,
                      long long sweep, cudaStream_t st)
{
    return split ? dispatch3s<true>(R, P, items, nitems, wtab, total, sweep, st)
                 : dispatch3s<false>(R, P, items, nitems, wtab, total, sweep, st);
}

}  // namespace

struct cs_batch {
    int count = 0, dims = 2, radius = 0, pattern = 0, sps = 1, total = 0;
    bool split = false;
    bool tc = false;  // 2D radius-3 grids on the tcgen05 kernels (d_items hold their records)
    cs::TcWait wait;
    void *d_items[2] = {nullptr, nullptr};  // Item or Item3 tables; sweep parity 0: a -> b, 1: b -> a
    void *d_w = nullptr;
    std::map<long long, cudaGraphExec_t> graphs;  // (sweeps, starting parity) -> graph
    int parity = 0;  // which buffer holds the current state of every grid
    cudaStream_t mem_stream = nullptr;  // tables allocated and freed in order on it (server packs)
    bool stream_mem = false;
};

namespace {

cudaError_t table_alloc(cs_batch *bt, void **p, size_t bytes)
{
    return bt->stream_mem ? cudaMallocAsync(p, bytes, bt->mem_stream) : cudaMalloc(p, bytes);
}

cudaError_t table_copy(cs_batch *bt, void *dst, const void *src, size_t bytes)
{
    // Stream-ordered tables come from pageable host vectors: the copy is
    // staged before cudaMemcpyAsync returns, so the vectors may go away.
    return bt->stream_mem ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, bt->mem_stream)
                          : cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
}

}  // namespace

namespace cs {

// cs_batch_create with per-grid sweep counts (NULL: unbounded), the tcgen05
// path optional, and tables allocated in order on `mem_stream` when it is not
// NULL (no device-wide synchronisation; the server's packs).
cs_status batch_create_ex(cs_batch **out, cs_plan *const *plans, void *const *a, void *const *b, int count,
                          const long long *sweeps, bool allow_tc, cudaStream_t mem_stream)
{
    if (!out || !plans || !a || !b || count < 1)
        return cs::set_error(CS_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
    *out = nullptr;
    std::vector<cs::PlanFacts> f(count);
    for (int i = 0; i < count; ++i) {
        if (!plans[i] || !a[i] || !b[i] || a[i] == b[i] || !cs::plan_facts(plans[i], &f[i]))
            return cs::set_error(CS_ERR_INVALID_ARGUMENT, "bad plan or buffer in batch");
        if (reinterpret_cast<uintptr_t>(a[i]) % 8 || reinterpret_cast<uintptr_t>(b[i]) % 8)
            return cs::set_error(CS_ERR_INVALID_ARGUMENT,
                                 "grid buffers must be 8-byte aligned (double / float2 elements)");
        if (f[i].dims != 2 && f[i].dims != 3)
            return cs::set_error(CS_ERR_UNSUPPORTED, "batches pack 2D or 3D grids");
        if (f[i].dims == 3 && f[i].radius != 1 && f[i].radius != 3)
            return cs::set_error(CS_ERR_UNSUPPORTED, "3D batches serve radius 1 and 3");
        if (f[i].dims != f[0].dims || f[i].radius != f[0].radius || f[i].pattern != f[0].pattern || f[i].prec != f[0].prec ||
            f[i].steps_per_sweep != f[0].steps_per_sweep)
            return cs::set_error(CS_ERR_INVALID_ARGUMENT,
                                 "batched plans must share dims, radius, tap pattern, precision and steps per "
                                 "sweep");
    }
    auto *bt = new cs_batch();
    bt->mem_stream = mem_stream;
    bt->stream_mem = mem_stream != nullptr;
    bt->count = count;
    bt->dims = f[0].dims;
    bt->radius = f[0].radius;
    bt->pattern = f[0].pattern;
    bt->sps = f[0].steps_per_sweep;
    bt->split = f[0].prec == CS_PREC_SPLIT;
    // 2D radius-3 grids of at least 8 x 8 on TMA-compatible layouts and
    // 16-byte aligned buffers run on the tcgen05 kernels (split or FP64).
    bt->tc = allow_tc && !sweeps && bt->dims == 2 && bt->radius == 3;
    for (int i = 0; bt->tc && i < count; ++i)
        bt->tc = f[i].view.ext[0] >= 8 && f[i].view.ext[1] >= 8 &&
                 cs::split_tma_layout_ok(f[i].view, f[i].origin, a[i]) &&
                 cs::split_tma_layout_ok(f[i].view, f[i].origin, b[i]) &&
                 reinterpret_cast<uintptr_t>(a[i]) % 16 == 0 && reinterpret_cast<uintptr_t>(b[i]) % 16 == 0;
    if (bt->tc) {
        const size_t rb = cs::tc_batch_record_bytes(!bt->split);
        std::vector<unsigned char> rec[2];
        cudaError_t e = cudaSuccess;
        int total = 0;
        for (int p = 0; p < 2; ++p) rec[p].resize(rb * count);
        for (int i = 0; i < count && e == cudaSuccess; ++i) {
            int tiles = 0, id = i;  // grids with equal weights share their B matrices
            for (int j = 0; j < i; ++j)
                if (std::memcmp(f[j].w, f[i].w, sizeof(cs::Weights)) == 0) {
                    id = j;
                    break;
                }
            e = cs::tc_batch_fill_record(!bt->split, rec[0].data() + rb * i, f[i].view, *f[i].w, f[i].origin,
                                         f[i].elements, a[i], b[i], total, id, &tiles);
            if (e == cudaSuccess)
                e = cs::tc_batch_fill_record(!bt->split, rec[1].data() + rb * i, f[i].view, *f[i].w, f[i].origin,
                                             f[i].elements, b[i], a[i], total, id, &tiles);
            total += tiles;
        }
        for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
            e = table_alloc(bt, &bt->d_items[p], rb * count);
            if (e == cudaSuccess) e = table_copy(bt, bt->d_items[p], rec[p].data(), rb * count);
        }
        bt->total = total;
        if (e != cudaSuccess) {
            cs_batch_destroy(bt);
            return cs::set_error(e == cudaErrorMemoryAllocation ? CS_ERR_OUT_OF_MEMORY : CS_ERR_CUDA,
                                 cudaGetErrorString(e));
        }
        *out = bt;
        return CS_OK;
    }
    const int K = 2 * bt->radius + 1, taps = bt->dims == 3 ? K * K * K : K * K;
    std::vector<Item> items[2];
    std::vector<Item3> items3[2];
    std::vector<double> wd;
    std::vector<float2> wf;
    int total = 0;
    for (int i = 0; i < count; ++i) {
        const GridView &g = f[i].view;
        const size_t esz = bt->split ? sizeof(float2) : sizeof(double);
        char *pa = (char *)a[i] + f[i].origin * esz, *pb = (char *)b[i] + f[i].origin * esz;
        if (bt->dims == 2) {
            Item it{};
            it.ld = g.pitch[0];
            it.m = (int)g.ext[0];
            it.n = (int)g.ext[1];
            it.tiles_x = (int)((g.ext[1] + TX - 1) / TX);
            it.tile_begin = total;
            it.sweeps = sweeps ? sweeps[i] : LLONG_MAX;
            total += it.tiles_x * (int)((g.ext[0] + TY - 1) / TY);
            it.in = pa;
            it.out = pb;
            items[0].push_back(it);
            it.in = pb;
            it.out = pa;
            items[1].push_back(it);
        } else {
            Item3 it{};
            it.ldy = g.pitch[1];
            it.ldz = g.pitch[0];
            it.h = (int)g.ext[0];
            it.m = (int)g.ext[1];
            it.n = (int)g.ext[2];
            it.tiles_x = (int)((g.ext[2] + TX3 - 1) / TX3);
            it.tiles_y = (int)((g.ext[1] + TY3 - 1) / TY3);
            it.zc = (int)std::min<long long>(ZC3, g.ext[0]);
            it.tile_begin = total;
            it.sweeps = sweeps ? sweeps[i] : LLONG_MAX;
            total += it.tiles_x * it.tiles_y * (int)((g.ext[0] + it.zc - 1) / it.zc);
            it.in = pa;
            it.out = pb;
            items3[0].push_back(it);
            it.in = pb;
            it.out = pa;
            items3[1].push_back(it);
        }
        for (int t = 0; t < taps; ++t) {
            const double v = f[i].w->v[t];
            wd.push_back(v);
            const float h = (float)v;
            wf.push_back(make_float2(h, (float)(v - (double)h)));
        }
    }
    bt->total = total;
    const size_t isz = bt->dims == 2 ? sizeof(Item) : sizeof(Item3);
    cudaError_t e = cudaSuccess;
    for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
        e = table_alloc(bt, &bt->d_items[p], isz * count);
        const void *src = bt->dims == 2 ? (const void *)items[p].data() : (const void *)items3[p].data();
        if (e == cudaSuccess) e = table_copy(bt, bt->d_items[p], src, isz * count);
    }
    const size_t wbytes = bt->split ? wf.size() * sizeof(float2) : wd.size() * sizeof(double);
    if (e == cudaSuccess) e = table_alloc(bt, &bt->d_w, wbytes);
    if (e == cudaSuccess)
        e = table_copy(bt, bt->d_w, bt->split ? (const void *)wf.data() : (const void *)wd.data(), wbytes);
    if (e != cudaSuccess) {
        cs_batch_destroy(bt);
        return cs::set_error(e == cudaErrorMemoryAllocation ? CS_ERR_OUT_OF_MEMORY : CS_ERR_CUDA,
                             cudaGetErrorString(e));
    }
    *out = bt;
    return CS_OK;
}

// One launch of sweep `sweep` for every grid with more sweeps than that
// (buffer parity sweep % 2: a -> b for even sweeps). Grids past their sweep
// count keep their state where their last sweep left it.
cs_status batch_sweep(cs_batch *bt, long long sweep, cudaStream_t st)
{
    const int par = (int)(sweep & 1);
    cudaError_t e =
        bt->tc ? cs::launch_tc_batch(!bt->split, bt->d_items[par], bt->count, bt->total, bt->wait, st)
        : bt->dims == 2 ? dispatch(bt->radius, bt->pattern, bt->split, (const Item *)bt->d_items[par], bt->count,
                                   bt->d_w, bt->total, sweep, st)
                        : dispatch3(bt->radius, bt->pattern, bt->split, (const Item3 *)bt->d_items[par], bt->count,
                                    bt->d_w, bt->total, sweep, st);
    if (e != cudaSuccess) return cs::set_error(CS_ERR_CUDA, cudaGetErrorString(e));
    return CS_OK;
}

}  // namespace cs

extern "C" {

CS_API cs_status cs_batch_create(cs_batch **out, cs_plan *const *plans, void *const *a, void *const *b,
                                 int count)
{
    return cs::batch_create_ex(out, plans, a, b, count, nullptr, true, nullptr);
}

CS_API cs_status cs_batch_run(cs_batch *bt, long long steps, void *stream, int *result_in_b)
{
    if (!bt) return cs::set_error(CS_ERR_INVALID_ARGUMENT, "NULL batch");
    if (steps < 0 || steps % bt->sps)
        return cs::set_error(CS_ERR_INVALID_ARGUMENT, "steps must be a non-negative multiple of the fused steps");
    const long long sweeps = steps / bt->sps;
    cudaStream_t st = (cudaStream_t)stream;
    auto issue = [&](long long n) -> cudaError_t {
        int par = bt->parity;
        for (long long i = 0; i < n; ++i) {
            cudaError_t e =
                bt->tc ? cs::launch_tc_batch(!bt->split, bt->d_items[par], bt->count, bt->total, bt->wait, st)
                : bt->dims == 2
                    ? dispatch(bt->radius, bt->pattern, bt->split, (const Item *)bt->d_items[par], bt->count,
                               bt->d_w, bt->total, 0, st)
                    : dispatch3(bt->radius, bt->pattern, bt->split, (const Item3 *)bt->d_items[par], bt->count,
                                bt->d_w, bt->total, 0, st);
            if (e != cudaSuccess) return e;
            par ^= 1;
        }
        return cudaSuccess;
    };
    cudaError_t e = cudaSuccess;
    // An even sweep count returns every grid to its starting buffer, so the
    // captured launches can be replayed as they are.
    if (st && sweeps > 0 && sweeps % 2 == 0) {
        const long long key = sweeps * 2 + bt->parity;  // a graph starts from one parity
        auto it = bt->graphs.find(key);
        if (it == bt->graphs.end()) {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t x = nullptr;
            e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                cudaError_t le = issue(sweeps);
                e = cudaStreamEndCapture(st, &g);
                if (le != cudaSuccess) e = le;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e == cudaSuccess) it = bt->graphs.emplace(key, x).first;
        }
        if (e == cudaSuccess) e = cudaGraphLaunch(it->second, st);
    } else {
        e = issue(sweeps);
    }
    if (e != cudaSuccess) return cs::set_error(CS_ERR_CUDA, cudaGetErrorString(e));
    bt->parity ^= (int)(sweeps & 1);
    if (result_in_b) *result_in_b = bt->parity;
    return CS_OK;
}

CS_API cs_status cs_batch_destroy(cs_batch *bt)
{
    if (!bt) return CS_OK;
    for (auto &kv : bt->graphs) cudaGraphExecDestroy(kv.second);
    for (void *p : bt->d_items)
        if (p) bt->stream_mem ? cudaFreeAsync(p, bt->mem_stream) : cudaFree(p);
    if (bt->d_w) bt->stream_mem ? cudaFreeAsync(bt->d_w, bt->mem_stream) : cudaFree(bt->d_w);
    delete bt;
    return CS_OK;
}

}  // extern "C"
