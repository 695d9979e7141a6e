// cs_batch.cu — uneven 2D grids packed into one persistent launch per sweep.
//
// A batch is a set of plans (same dims, radius, tap pattern, precision and
// steps per sweep; any sizes, weights and layouts) with their ping-pong
// buffers. One launch advances every grid of the batch by one sweep: the
// tiles of all grids form one list, persistent CTAs walk it, and a device
// table gives each tile its grid (pointers, sizes, pitch) and weights. Per
// tile the arithmetic is the single-grid kernels' (same tap order, same
// FP64 FMA or double-float operations), so a grid's result is bitwise the
// same batched or alone. cs_batch_run of an even sweep count on a stream is
// captured once as a CUDA graph and replayed on later calls.
#include "../../include/convstencil.h"
#include "cs_internal.h"
#include "cs_split_ff.cuh"

#include <algorithm>
#include <map>
#include <vector>

struct cs_plan;

namespace cs {

struct PlanFacts {  // read-only view of a plan for the batcher (cs_api.cu)
    int dims, radius, pattern, steps_per_sweep;
    cs_precision prec;
    GridView view;
    long long origin;
    const Weights *w;
};
bool plan_facts(const cs_plan *p, PlanFacts *f);
cs_status set_error(cs_status s, const char *msg);

}  // namespace cs

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
};

constexpr int TX = 64, TY = 32, RPT = 8;

using cs::ff::tap2s;

__device__ __forceinline__ int find_item(const Item *items, int nitems, int tile)
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
                                                     const double *__restrict__ wtab, int total)
{
    constexpr int K = 2 * R + 1, SX = TX + 2 * R, SY = TY + 2 * R;
    __shared__ double s[SY * SX];
    __shared__ double ws[K * K];
    int cur = -1;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int it = find_item(items, nitems, tile);
        const Item I = items[it];
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
                                                    const float2 *__restrict__ wtab, int total)
{
    constexpr int K = 2 * R + 1, SX = TX + 2 * R, SY = TY + 2 * R;
    __shared__ float2 s[SY * SX];
    __shared__ float2 ws[K * K];  // (hi, lo) per tap
    int cur = -1;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int it = find_item(items, nitems, tile);
        const Item I = items[it];
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
                         cudaStream_t st)
{
    cs::note_launch();
    if (split) {
        const int grid = persistent_grid(k2d_ff_batch<R, P>, total);
        k2d_ff_batch<R, P><<<grid, 256, 0, st>>>(items, nitems, (const float2 *)wtab, total);
    } else {
        const int grid = persistent_grid(k2d_fma_batch<R, P>, total);
        k2d_fma_batch<R, P><<<grid, 256, 0, st>>>(items, nitems, (const double *)wtab, total);
    }
    return cudaGetLastError();
}

cudaError_t dispatch(int R, int P, bool split, const Item *items, int nitems, const void *wtab, int total,
                     cudaStream_t st)
{
    if (R == 1) return P == PAT_STAR ? launch_batch<1, PAT_STAR>(split, items, nitems, wtab, total, st)
                                     : launch_batch<1, PAT_DENSE>(split, items, nitems, wtab, total, st);
    if (R == 2) {
        if (P == PAT_STAR) return launch_batch<2, PAT_STAR>(split, items, nitems, wtab, total, st);
        if (P == PAT_DIAMOND) return launch_batch<2, PAT_DIAMOND>(split, items, nitems, wtab, total, st);
        return launch_batch<2, PAT_DENSE>(split, items, nitems, wtab, total, st);
    }
    if (R == 3) {
        if (P == PAT_STAR) return launch_batch<3, PAT_STAR>(split, items, nitems, wtab, total, st);
        if (P == PAT_DIAMOND) return launch_batch<3, PAT_DIAMOND>(split, items, nitems, wtab, total, st);
        return launch_batch<3, PAT_DENSE>(split, items, nitems, wtab, total, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

struct cs_batch {
    int count = 0, radius = 0, pattern = 0, sps = 1, total = 0;
    bool split = false;
    Item *d_items[2] = {nullptr, nullptr};  // sweep parity 0: a -> b, parity 1: b -> a
    void *d_w = nullptr;
    std::map<long long, cudaGraphExec_t> graphs;  // (sweeps, starting parity) -> graph
    int parity = 0;  // which buffer holds the current state of every grid
};

extern "C" {

CS_API cs_status cs_batch_create(cs_batch **out, cs_plan *const *plans, void *const *a, void *const *b,
                                 int count)
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
        if (f[i].dims != 2)
            return cs::set_error(CS_ERR_UNSUPPORTED, "batches pack 2D grids");
        if (f[i].radius != f[0].radius || f[i].pattern != f[0].pattern || f[i].prec != f[0].prec ||
            f[i].steps_per_sweep != f[0].steps_per_sweep)
            return cs::set_error(CS_ERR_INVALID_ARGUMENT,
                                 "batched plans must share radius, tap pattern, precision and steps per sweep");
    }
    auto *bt = new cs_batch();
    bt->count = count;
    bt->radius = f[0].radius;
    bt->pattern = f[0].pattern;
    bt->sps = f[0].steps_per_sweep;
    bt->split = f[0].prec == CS_PREC_SPLIT;
    const int K = 2 * bt->radius + 1, taps = K * K;
    std::vector<Item> items[2];
    std::vector<double> wd;
    std::vector<float2> wf;
    int total = 0;
    for (int i = 0; i < count; ++i) {
        const GridView &g = f[i].view;
        const size_t esz = bt->split ? sizeof(float2) : sizeof(double);
        char *pa = (char *)a[i] + f[i].origin * esz, *pb = (char *)b[i] + f[i].origin * esz;
        Item it{};
        it.ld = g.pitch[0];
        it.m = (int)g.ext[0];
        it.n = (int)g.ext[1];
        it.tiles_x = (int)((g.ext[1] + TX - 1) / TX);
        it.tile_begin = total;
        total += it.tiles_x * (int)((g.ext[0] + TY - 1) / TY);
        it.in = pa;
        it.out = pb;
        items[0].push_back(it);
        it.in = pb;
        it.out = pa;
        items[1].push_back(it);
        for (int t = 0; t < taps; ++t) {
            const double v = f[i].w->v[t];
            wd.push_back(v);
            const float h = (float)v;
            wf.push_back(make_float2(h, (float)(v - (double)h)));
        }
    }
    bt->total = total;
    cudaError_t e = cudaSuccess;
    for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
        e = cudaMalloc(&bt->d_items[p], sizeof(Item) * count);
        if (e == cudaSuccess)
            e = cudaMemcpy(bt->d_items[p], items[p].data(), sizeof(Item) * count, cudaMemcpyHostToDevice);
    }
    const size_t wbytes = bt->split ? wf.size() * sizeof(float2) : wd.size() * sizeof(double);
    if (e == cudaSuccess) e = cudaMalloc(&bt->d_w, wbytes);
    if (e == cudaSuccess)
        e = cudaMemcpy(bt->d_w, bt->split ? (const void *)wf.data() : (const void *)wd.data(), wbytes,
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cs_batch_destroy(bt);
        return cs::set_error(e == cudaErrorMemoryAllocation ? CS_ERR_OUT_OF_MEMORY : CS_ERR_CUDA,
                             cudaGetErrorString(e));
    }
    *out = bt;
    return CS_OK;
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
            cudaError_t e = dispatch(bt->radius, bt->pattern, bt->split, bt->d_items[par], bt->count, bt->d_w,
                                     bt->total, st);
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
    for (Item *p : bt->d_items)
        if (p) cudaFree(p);
    if (bt->d_w) cudaFree(bt->d_w);
    delete bt;
    return CS_OK;
}

}  // extern "C"
