// cs_api.cu — host side of libconvstencil_gb300: plans, layouts, weight
// algebra, the sweep loop, the tuner, and the reference-shaped wrappers.
//
// The reference's host wrappers (src/2d/gpu.cu:245-425, src/1d/gpu_1r.cu:227-302,
// src/1d/gpu_2r.cu:85-159, src/3d/gpu_box.cu:446-536, src/3d/gpu_star.cu:238-332)
// build B matrices and lookup tables, copy one grid in, ping-pong `times`
// launches and copy the result out. Here the weights go to the kernels as
// parameters (no __constant__ symbol, so plans are reentrant and independent
// streams can run different stencils at once), no lookup tables exist (the
// kernels index their tiles directly), and every failure is a status code.
#include "../../include/convstencil.h"
#include "cs_internal.h"
#include "cs_plan_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

namespace cs {

static std::atomic<long long> g_launches{0};
void note_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

constexpr int kGraphBlockSweeps = 32;             // sweeps per replayed graph block (about)
constexpr long long kGraphMaxPoints = 8LL << 20;  // grids of up to 8M points replay graphs

}  // namespace cs

using cs::GridView;
using cs::Weights;

namespace {

thread_local std::string t_err;
thread_local double t_loop_seconds = 0.0;
std::atomic<int> g_verbose{0};

cs_status fail(cs_status s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
    return s;
}

cs_status cuda_fail(cudaError_t e, const char *what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(CS_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return fail(CS_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
    return fail(CS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CS_CUDA(call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);        \
    } while (0)

// Per-shape facts. Fused parameters and steps per fused sweep follow the
// reference CLIs and wrappers: src/1d/main.cu:103-151, src/2d/main.cu:183-303,
// src/3d/main.cu:526-567, src/3d/gpu_star.cu:30-56.
struct ShapeInfo {
    int dims, base_r, n_base, fused_r, n_fused, fused_steps;
    const char *name;
};
const ShapeInfo kShapes[8] = {
    {1, 1, 3, 3, 7, 3, "1d1r"},      {1, 2, 5, 4, 9, 2, "1d2r"},
    {2, 1, 5, 3, 49, 3, "star2d1r"}, {2, 1, 9, 3, 49, 3, "box2d1r"},
    {2, 3, 13, 3, 49, 1, "star2d3r"}, {2, 3, 49, 3, 49, 1, "box2d3r"},
    {3, 1, 7, 3, 44, 3, "star3d1r"}, {3, 1, 27, 3, 196, 3, "box3d1r"},
};

int ipow(int b, int e)
{
    int r = 1;
    while (e--) r *= b;
    return r;
}

// Expand a shape's parameters to a dense (2r+1)^dims row-major kernel.
bool expand_weights(cs_shape shape, cs_semantics sem, const double *p, Weights &w, int &radius)
{
    const ShapeInfo &si = kShapes[shape];
    memset(w.v, 0, sizeof w.v);
    if (sem == CS_SEM_STEP) {
        radius = si.base_r;
        switch (shape) {
        case CS_SHAPE_STAR2D1R: {  // N, W, C, E, S at 3x3 cells 1,3,4,5,7 (src/2d/main.cu:211-217)
            const int cell[5] = {1, 3, 4, 5, 7};
            for (int i = 0; i < 5; ++i) w.v[cell[i]] = p[i];
            return true;
        }
        case CS_SHAPE_STAR2D3R: {  // row-major cells of the radius-3 cross
            int t = 0;
            for (int i = 0; i < 7; ++i)
                for (int j = 0; j < 7; ++j)
                    if (i == 3 || j == 3) w.v[i * 7 + j] = p[t++];
            return true;
        }
        case CS_SHAPE_STAR3D1R: {  // z-1, y-1, x-1, C, x+1, y+1, z+1 (src/3d/main.cu:557-565)
            const int cell[7] = {4, 10, 12, 13, 14, 16, 22};
            for (int i = 0; i < 7; ++i) w.v[cell[i]] = p[i];
            return true;
        }
        default:
            for (int i = 0; i < si.n_base; ++i) w.v[i] = p[i];
            return true;
        }
    }
    radius = si.fused_r;
    if (shape == CS_SHAPE_BOX3D1R) {
        // 4 planes of 49; plane q serves dz = +-(3-q) (src/3d/gpu_box.cu:450-468).
        for (int a = 0; a < 7; ++a) {
            const int q = 3 - std::abs(a - 3);
            for (int t = 0; t < 49; ++t) w.v[a * 49 + t] = p[q * 49 + t];
        }
        return true;
    }
    if (shape == CS_SHAPE_STAR3D1R) {
        // Plane |dz| holds the row-major cells of |dy|+|dx| <= 3-|dz|, blocks at
        // 0, 1, 6, 19 (src/3d/main.cu:42-113, src/3d/gpu_star.cu:30-56).
        const int base[4] = {0, 1, 6, 19};
        for (int a = 0; a < 7; ++a) {
            const int rho = 3 - std::abs(a - 3);
            int t = base[rho];
            for (int i = 0; i < 7; ++i)
                for (int j = 0; j < 7; ++j)
                    if (std::abs(i - 3) + std::abs(j - 3) <= rho) w.v[(a * 7 + i) * 7 + j] = p[t++];
        }
        return true;
    }
    for (int i = 0; i < si.n_fused; ++i) w.v[i] = p[i];
    return true;
}

// Smallest tap pattern covering the non-zero weights.
int classify(const Weights &w, int dims, int r)
{
    if (dims == 1) return cs::PAT_DENSE;
    const int k = 2 * r + 1;
    bool star = true, diamond = true;
    const int n = ipow(k, dims);
    for (int t = 0; t < n; ++t) {
        if (w.v[t] == 0.0) continue;
        int c[3] = {0, 0, 0}, rem = t;
        for (int d = dims - 1; d >= 0; --d) {
            c[d] = rem % k - r;
            rem /= k;
        }
        int nz = 0, l1 = 0;
        for (int d = 0; d < dims; ++d) {
            nz += c[d] != 0;
            l1 += std::abs(c[d]);
        }
        if (nz > 1) star = false;
        if (l1 > r) diamond = false;
    }
    if (star) return cs::PAT_STAR;
    if (diamond) return r == 1 ? cs::PAT_STAR : cs::PAT_DIAMOND;
    return cs::PAT_DENSE;
}

long long round_up(long long v, long long a) { return (v + a - 1) / a * a; }

void native_layout(int dims, int r, const long long *ext, cs_layout &L)
{
    memset(&L, 0, sizeof L);
    L.dims = dims;
    L.halo = r;
    const long long x0 = round_up(r, 2);  // interior rows start 16-byte aligned
    if (dims == 1) {
        // at least 4 points of halo before the interior and 60 after it: the
        // 1D FP64 tcgen05 sweep reads 4 neighbours either side of a row of 64
        // outputs, as whole 64-point rows of the array from origin - 4
        const long long h1 = std::max(x0, 4LL);
        L.extent[0] = ext[0];
        L.pitch[0] = 1;
        L.origin = h1;
        L.elements = round_up(h1 + ext[0] + std::max((long long)r, 60LL), 2);
    } else if (dims == 2) {
        L.extent[0] = ext[0];
        L.extent[1] = ext[1];
        L.pitch[1] = 1;
        L.pitch[0] = round_up(x0 + ext[1] + r, 2);
        L.origin = r * L.pitch[0] + x0;
        L.elements = (ext[0] + 2 * r) * L.pitch[0];
    } else {
        for (int d = 0; d < 3; ++d) L.extent[d] = ext[d];
        L.pitch[2] = 1;
        L.pitch[1] = round_up(x0 + ext[2] + r, 2);
        L.pitch[0] = L.pitch[1] * (ext[1] + 2 * r);
        L.origin = r * L.pitch[0] + r * L.pitch[1] + x0;
        L.elements = (ext[0] + 2 * r) * L.pitch[0];
    }
    L.bytes = (size_t)L.elements * sizeof(double);
}

// The tuner's memory: which algorithm won for a (dims, radius, pattern,
// precision, log2 size) class. Process-wide, guarded by a mutex.
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, int>, int> g_tune;      // -> algorithm
std::map<std::tuple<int, int, int, int, int>, int> g_tune_tb;   // -> steps per launch (split FMA)
std::map<std::tuple<int, int, int, int, int>, int> g_tune_rows; // -> FP64 FMA 2D tile rows

}  // namespace

struct cs_plan {
    cs_shape shape;
    cs_semantics sem;
    cs_precision prec;
    int dims, radius, pattern, steps_per_sweep;
    Weights w;
    Weights w7;  // 2D plans: w at the centre of a 7x7 (the 2D tcgen05 kernels' tap window)
    cs_layout layout;
    GridView view;
    int algo = CS_ALGO_AUTO;
    int last_algo = CS_ALGO_AUTO;  // kernel family the last cs_run used
    int time_block = 0;            // split FMA: steps per launch (0 = tuner)
    int last_time_block = 1;
    int tile_rows = 0;             // FP64 FMA 2D: rows per CTA tile (0 = tuner)
    int active_rows = 0;           // the tile rows launches use now (0 = by grid size)
    long long reanchor = 100;
    cs::TcWait wait;               // bounded waits of the tcgen05 kernels
    // Small grids: blocks of sweeps replayed as CUDA graphs (see cs_run).
    std::mutex graph_mu;
    std::map<std::tuple<const void *, const void *, int, int, int>, cudaGraphExec_t> graphs;
    cudaStream_t capture_stream = nullptr;
    // Host-buffer runs (cs_run_host): the two device grids, allocated by the
    // first call and kept for later ones; a call that finds them in use by
    // another thread allocates its own.
    std::mutex host_mu;
    void *host_bufs[2] = {nullptr, nullptr};
    size_t host_bytes = 0;
    // The band schedule of host-buffer runs on the tcgen05 batch kernel
    // (host_run_banded): the device records of every distinct set of
    // band-sweeps, kept for the bands, sweeps and grids they were made for.
    struct BandSet {
        long long rec;  // first record in the table
        int count, tiles;
    };
    struct BandTable {
        int bands = 0, algo = -1;
        long long sweeps = 0;
        const void *d0 = nullptr, *d1 = nullptr;
        void *tab = nullptr;
        std::vector<BandSet> sets;  // one per set, in launch order
    } band;
    ~cs_plan()
    {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        if (capture_stream) cudaStreamDestroy(capture_stream);
        for (void *b : host_bufs)
            if (b) cudaFree(b);
        if (band.tab) cudaFree(band.tab);
    }
};

namespace {

bool fp64_mma_ok(const cs_plan *p)
{
    return p->prec == CS_PREC_FP64 && p->dims == 2 && p->radius == 3 &&
           p->pattern == cs::PAT_DENSE;
}

// The slice kernel's error is relative to the tile scale times the largest
// weight; on grids smaller than the 8x8 window every output can be formed by
// a few small taps only, so those go to the double-float kernel.
bool split_mma_ok(const cs_plan *p)
{
    return p->prec == CS_PREC_SPLIT && p->dims == 2 && p->radius == 3 &&
           p->view.ext[0] >= 8 && p->view.ext[1] >= 8 &&
           cs::split_mma_layout_ok(p->view, p->layout.origin);
}

// FP64 plans of 2D stencils of radius up to 3 (their weights at the centre of
// the 7x7, w7) also run on the tcgen05 digit pipeline; like the split slice
// kernels its error is relative to the tile's scale, so grids smaller than
// the 8x8 window stay on FP64 FMA.
bool fp64_tc_geometry_ok(const cs_plan *p)
{
    return p->dims == 2 && p->radius <= 3 && p->view.ext[0] >= 8 && p->view.ext[1] >= 8 &&
           cs::split_mma_layout_ok(p->view, p->layout.origin);
}

// Buffers and layout the 2D FP64 tcgen05 sweep can read by TMA: even pitch
// and interior column (the window's first column, 4 to the left of a tile,
// must be 16-byte aligned), 16-byte aligned bases. Window rows and columns
// outside the buffer (a halo narrower than 3 rows or 4 columns) are read as
// zero by the TMA unit; those inside it but outside the plan's own halo meet
// zero weights of the 7x7.
bool fp64_tc_window_ok(const GridView &v, long long off, const void *in_base, const void *out_base)
{
    const long long ld = v.pitch[0];
    return v.dims == 2 && ld % 2 == 0 && (off % ld) % 2 == 0 && reinterpret_cast<uintptr_t>(in_base) % 16 == 0 &&
           reinterpret_cast<uintptr_t>(out_base) % 16 == 0;
}

bool fp64_tc_ok(const cs_plan *p) { return p->prec == CS_PREC_FP64 && fp64_tc_geometry_ok(p); }

// FP64 plans of 3D radius-1 stencils run on the 3D tcgen05 digit pipeline
// (the same work items as the split 3D kernel, six digits per point). The
// plan holds the 3x3x3 weights with zeros outside its pattern, and the
// pipeline's cost does not depend on how many taps are nonzero, so the
// 7-point star takes it too.
bool fp64_tc3d_geometry_ok(const cs_plan *p) { return p->dims == 3 && p->radius == 1; }
bool fp64_tc3d_ok(const cs_plan *p) { return p->prec == CS_PREC_FP64 && fp64_tc3d_geometry_ok(p); }

// 1D plans of radius up to 3 on the 2D tcgen05 digit kernel through a row
// view (launch_fp64_sweep_tc_rows1d): rows of 64 outputs, so the interior
// must be a whole number of rows (at least 8), with an even origin, 4 points
// of halo before it and 60 points of the array after it.
bool fp64_tc1d_geometry_ok(const cs_plan *p)
{
    const long long n = p->view.ext[0], o = p->layout.origin;
    return p->dims == 1 && p->radius <= 3 && n % 64 == 0 && n >= 512 && o >= 4 && o % 2 == 0 &&
           p->layout.elements >= o + n + 60;
}
bool fp64_tc1d_ok(const cs_plan *p) { return p->prec == CS_PREC_FP64 && fp64_tc1d_geometry_ok(p); }

// Split plans of 3D radius-1 stencils (27 weights) also run on the tcgen05
// slice kernel.
bool split_tc3d_ok(const cs_plan *p)
{
    return p->prec == CS_PREC_SPLIT && p->dims == 3 && p->radius == 1;
}

// One sweep over the slabs [row0, row0 + rows) of the slowest axis (rows of
// a 2D grid, planes of a 3D one). The slabs on either side are read as the
// grid's own data, so a sweep may be split into bands this way; the
// temporally blocked kernels, which treat everything outside their grid as
// zero, are never launched here.
cudaError_t launch_sweep_rows(const cs_plan *p, int algo, const void *in_base, void *out_base, long long row0,
                              long long rows, cudaStream_t st)
{
    GridView v = p->view;
    v.ext[0] = rows;
    const long long off = p->layout.origin + row0 * p->view.pitch[0];
    if (p->prec == CS_PREC_FP64) {
        const double *in = (const double *)in_base + off;
        double *out = (double *)out_base + off;
        if (algo == CS_ALGO_FP64_MMA) return cs::launch_fp64_mma_2d(v, p->w, in, out, st);
        if (algo == CS_ALGO_FP64_TC && fp64_tc1d_ok(p) && row0 == 0 && rows == p->view.ext[0] &&
            reinterpret_cast<uintptr_t>(in_base) % 16 == 0 && reinterpret_cast<uintptr_t>(out_base) % 16 == 0)
            return cs::launch_fp64_sweep_tc_rows1d(rows, p->w7, p->layout.origin, p->layout.elements,
                                                   (const double *)in_base, (double *)out_base, p->wait, st);
        if (algo == CS_ALGO_FP64_TC && fp64_tc3d_ok(p) && cs::split_tc3d_layout_ok(v, off, in_base, out_base))
            return cs::launch_fp64_sweep_tc3d(v, p->w, off, p->layout.elements, (const double *)in_base,
                                              (double *)out_base, p->wait, st);
        if (algo == CS_ALGO_FP64_TC && fp64_tc_ok(p) && fp64_tc_window_ok(v, off, in_base, out_base))
            return cs::launch_fp64_sweep_tc(v, p->w7, off, p->layout.elements, (const double *)in_base,
                                            (double *)out_base, p->wait, st);
        return cs::launch_fp64_fma(v, p->radius, p->pattern, p->w, in, out, st, p->active_rows);
    }
    // The tensor-core split kernels store float4 (two points) at even element
    // offsets, so they need a 16-byte aligned output base; the TMA-fed ones
    // also a 16-byte aligned input base. Otherwise the double-float kernel
    // (8-byte accesses only) runs.
    const bool out16 = (reinterpret_cast<uintptr_t>(out_base) % 16) == 0;
    if (p->dims == 3) {
        if (algo == CS_ALGO_SPLIT_TC && split_tc3d_ok(p) &&
            cs::split_tc3d_layout_ok(v, off, in_base, out_base))
            return cs::launch_split_sweep_tc3d(v, p->w, off, p->layout.elements,
                                               (const float2 *)in_base, (float2 *)out_base, p->wait, st);
        algo = CS_ALGO_SPLIT_FMA;
    }
    const bool tma_ok = out16 && cs::split_tma_layout_ok(v, off, in_base);
    if (algo == CS_ALGO_SPLIT_TC && tma_ok)
        return cs::launch_split_sweep_tc(v, p->w, off, p->layout.elements,
                                         (const float2 *)in_base, (float2 *)out_base, p->wait, st);
    if (algo == CS_ALGO_SPLIT_MMA_TMA && tma_ok)
        return cs::launch_split_sweep_tma(v, p->w, off, p->layout.elements,
                                          (const float2 *)in_base, (float2 *)out_base, st);
    if (algo == CS_ALGO_SPLIT_MMA_TMA || algo == CS_ALGO_SPLIT_TC)
        algo = CS_ALGO_SPLIT_MMA;  // buffer not TMA-aligned
    if (algo == CS_ALGO_SPLIT_MMA && !out16) algo = CS_ALGO_SPLIT_FMA;
    const float2 *in = (const float2 *)in_base + off;
    float2 *out = (float2 *)out_base + off;
    return cs::launch_split_sweep(v, p->radius, p->pattern, p->w, algo == CS_ALGO_SPLIT_MMA,
                                  in, out, st);
}

cudaError_t launch_sweep(const cs_plan *p, int algo, const void *in_base, void *out_base, cudaStream_t st)
{
    return launch_sweep_rows(p, algo, in_base, out_base, 0, p->view.ext[0], st);
}

int size_class(const cs_plan *p)
{
    long long pts = 1;
    for (int d = 0; d < p->dims; ++d) pts *= p->view.ext[d];
    int c = 0;
    while (pts > 1) {
        pts >>= 2;
        ++c;
    }
    return c;
}

// Picks the algorithm for a plan. With CS_ALGO_AUTO and more than one
// candidate, the first sweep of the first run is timed once per candidate
// (every candidate computes the same sweep a -> b, so the extra work changes
// no result) and the winner is remembered for plans of the same class.
cs_status choose_algo(cs_plan *p, const void *a, void *b, cudaStream_t st, int *out, bool may_time = true)
{
    int cand[4];
    int nc = 0;
    if (p->prec == CS_PREC_SPLIT && split_tc3d_ok(p)) {
        // The 7-point star keeps its own double-float kernel; a pinned
        // algorithm is either the tcgen05 kernel or the double-float one.
        if (p->algo != CS_ALGO_AUTO || p->pattern != cs::PAT_DENSE) {
            *out = p->algo == CS_ALGO_SPLIT_TC ? CS_ALGO_SPLIT_TC : CS_ALGO_SPLIT_FMA;
            return CS_OK;
        }
        cand[nc++] = CS_ALGO_SPLIT_TC;
        cand[nc++] = CS_ALGO_SPLIT_FMA;
    } else if (p->prec == CS_PREC_SPLIT) {
        if (p->algo != CS_ALGO_AUTO || !split_mma_ok(p)) {
            *out = split_mma_ok(p) ? p->algo : CS_ALGO_SPLIT_FMA;
            return CS_OK;
        }
        cand[nc++] = CS_ALGO_SPLIT_TC;
        cand[nc++] = CS_ALGO_SPLIT_MMA;
        cand[nc++] = CS_ALGO_SPLIT_MMA_TMA;
        cand[nc++] = CS_ALGO_SPLIT_FMA;
    } else {
        const bool tc = fp64_tc_ok(p) || fp64_tc3d_ok(p) || fp64_tc1d_ok(p);
        if ((p->algo == CS_ALGO_FP64_MMA && fp64_mma_ok(p)) || (p->algo == CS_ALGO_FP64_TC && tc)) {
            *out = p->algo;
            return CS_OK;
        }
        if (p->algo != CS_ALGO_AUTO || (!fp64_mma_ok(p) && !tc)) {
            *out = CS_ALGO_FP64_FMA;
            return CS_OK;
        }
        cand[nc++] = CS_ALGO_FP64_FMA;
        if (fp64_mma_ok(p)) cand[nc++] = CS_ALGO_FP64_MMA;
        if (tc) cand[nc++] = CS_ALGO_FP64_TC;
    }
    auto key = std::make_tuple(p->dims, p->radius, p->pattern, (int)p->prec, size_class(p));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            *out = it->second;
            return CS_OK;
        }
    }
    if (!may_time) {  // the caller cannot afford a timing run now
        *out = -1;
        return CS_OK;
    }
    float best_ms = 1e30f;
    int best = cand[0];
    cudaEvent_t e0, e1;
    CS_CUDA(cudaEventCreate(&e0));
    CS_CUDA(cudaEventCreate(&e1));
    for (int rep = 0; rep < 2; ++rep) {  // rep 0 warms up
        for (int ci = 0; ci < nc; ++ci) {
            const int c = cand[ci];
            CS_CUDA(cudaEventRecord(e0, st));
            CS_CUDA(launch_sweep(p, c, a, b, st));
            CS_CUDA(cudaEventRecord(e1, st));
            CS_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            CS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep == 1 && ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = best;
    }
    *out = best;
    return CS_OK;
}

// Steps per launch for the double-float split kernels (temporal blocking).
// With time_block 0 the first run times T = 1..4 once (one launch each on
// a -> b; every candidate computes the same sweeps) and remembers the fastest
// per step for plans of the same class.
cs_status choose_time_block(cs_plan *p, int algo, const void *a, void *b, cudaStream_t st, int *out)
{
    *out = 1;
    if (p->prec != CS_PREC_SPLIT || algo != CS_ALGO_SPLIT_FMA ||
        !cs::split_tb_supported(p->dims, p->radius, p->pattern))
        return CS_OK;
    if (p->time_block > 0) {
        *out = p->time_block;
        return CS_OK;
    }
    auto key = std::make_tuple(p->dims, p->radius, p->pattern, (int)p->prec, size_class(p));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_tb.find(key);
        if (it != g_tune_tb.end()) {
            *out = it->second;
            return CS_OK;
        }
    }
    const long long off = p->layout.origin;
    const float2 *in = (const float2 *)a + off;
    float2 *o = (float2 *)b + off;
    cudaEvent_t e0, e1;
    CS_CUDA(cudaEventCreate(&e0));
    CS_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_t = 1;
    for (int rep = 0; rep < 2; ++rep) {
        for (int t = 1; t <= 4; ++t) {
            CS_CUDA(cudaEventRecord(e0, st));
            cudaError_t e = t == 1 ? cs::launch_split_sweep(p->view, p->radius, p->pattern, p->w, 0, in, o, st)
                                   : cs::launch_split_sweep_tb(p->view, p->radius, p->pattern, t, p->w, in, o,
                                                               st);
            if (e != cudaSuccess) return cuda_fail(e, "time-block tuning launch");
            CS_CUDA(cudaEventRecord(e1, st));
            CS_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            CS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep == 1 && ms / t < best) {
                best = ms / t;
                best_t = t;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_tb[key] = best_t;
    }
    *out = best_t;
    return CS_OK;
}

// Tile rows of the FP64 FMA 2D kernel (16 or 32 rows per CTA tile): with
// tile_rows 0 the first run times both once on a -> b (bitwise the same
// sweep) and remembers the faster for plans of the same class.
cs_status choose_tile_rows(cs_plan *p, int algo, const void *a, void *b, cudaStream_t st, int *out)
{
    *out = 0;
    if (p->prec != CS_PREC_FP64 || algo != CS_ALGO_FP64_FMA || p->dims != 2) return CS_OK;
    if (p->tile_rows > 0) {
        *out = p->tile_rows;
        return CS_OK;
    }
    auto key = std::make_tuple(p->dims, p->radius, p->pattern, (int)p->prec, size_class(p));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_rows.find(key);
        if (it != g_tune_rows.end()) {
            *out = it->second;
            return CS_OK;
        }
    }
    const long long off = p->layout.origin;
    cudaEvent_t e0, e1;
    CS_CUDA(cudaEventCreate(&e0));
    CS_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_rows = 32;
    for (int rep = 0; rep < 2; ++rep) {
        for (int rows : {16, 32}) {
            CS_CUDA(cudaEventRecord(e0, st));
            cudaError_t e = cs::launch_fp64_fma(p->view, p->radius, p->pattern, p->w, (const double *)a + off,
                                                (double *)b + off, st, rows);
            if (e != cudaSuccess) return cuda_fail(e, "tile-rows tuning launch");
            CS_CUDA(cudaEventRecord(e1, st));
            CS_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            CS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep == 1 && ms < best) {
                best = ms;
                best_rows = rows;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_rows[key] = best_rows;
    }
    *out = best_rows;
    return CS_OK;
}

}  // namespace

namespace cs {

// FP64 re-anchor sweep of a split plan: the (hi, lo) state in `src` is
// turned into FP64 in place, one sweep runs in FP64 arithmetic (the tcgen05
// digit pipeline for 2D radius-3 plans where the buffers allow it, else FP64
// FMA) into `dst`, and `dst` is turned back into (hi, lo) pairs in place. The
// halos read the same either way (0.0 has the bits of (0, 0)); `src` is left
// holding FP64 values, like any consumed ping-pong buffer.
// One FP64 sweep of the plan's stencil between FP64 buffers.
cudaError_t fp64_anchor_sweep_fp64_in(const cs_plan *p, const void *src, void *dst, cudaStream_t st)
{
    const long long n = p->layout.elements, off = p->layout.origin;
    if (fp64_tc_geometry_ok(p) && fp64_tc_window_ok(p->view, off, src, dst))
        return launch_fp64_sweep_tc(p->view, p->w7, off, n, (const double *)src, (double *)dst, p->wait, st);
    if (fp64_tc3d_geometry_ok(p) && split_tc3d_layout_ok(p->view, off, src, dst))
        return launch_fp64_sweep_tc3d(p->view, p->w, off, n, (const double *)src, (double *)dst, p->wait, st);
    if (fp64_tc1d_geometry_ok(p) && reinterpret_cast<uintptr_t>(src) % 16 == 0 &&
        reinterpret_cast<uintptr_t>(dst) % 16 == 0)
        return launch_fp64_sweep_tc_rows1d(p->view.ext[0], p->w7, off, n, (const double *)src, (double *)dst,
                                           p->wait, st);
    return launch_fp64_fma(p->view, p->radius, p->pattern, p->w, (const double *)src + off, (double *)dst + off, st);
}

cudaError_t fp64_anchor_sweep(const cs_plan *p, void *src, void *dst, cudaStream_t st)
{
    const long long n = p->layout.elements;
    cudaError_t e = launch_split_to_fp64_inplace(n, src, st);
    if (e == cudaSuccess) e = fp64_anchor_sweep_fp64_in(p, src, dst, st);
    if (e == cudaSuccess) e = launch_fp64_to_split_inplace(n, dst, st);
    return e;
}

// cs_run with the sweeps numbered from first_sweep: split plans run sweep k
// in FP64 when (k + 1) is a multiple of the re-anchor interval, so a run cut
// into chunks (the server) re-anchors where one whole run would.
cs_status run_from(cs_plan *p, void *a, void *b, long long first_sweep, long long steps, cudaStream_t st,
                   int *result_in_b)
{
    if (!p || !a || !b) return fail(CS_ERR_INVALID_ARGUMENT, "NULL plan or buffer");
    if (a == b) return fail(CS_ERR_INVALID_ARGUMENT, "ping-pong buffers must differ");
    if (reinterpret_cast<uintptr_t>(a) % 8 || reinterpret_cast<uintptr_t>(b) % 8)
        return fail(CS_ERR_INVALID_ARGUMENT, "grid buffers must be 8-byte aligned (double / float2 elements)");
    long long sweeps = 0;
    cs_status s = cs_plan_sweeps(p, steps, &sweeps);
    if (s != CS_OK) return s;
    int algo = CS_ALGO_FP64_FMA, tb = 1;
    if (sweeps > 0) {
        s = choose_algo(p, a, b, st, &algo);
        if (s != CS_OK) return s;
        s = choose_time_block(p, algo, a, b, st, &tb);
        if (s != CS_OK) return s;
        int rows = 0;
        s = choose_tile_rows(p, algo, a, b, st, &rows);
        if (s != CS_OK) return s;
        p->last_algo = algo;
        p->last_time_block = tb;
        p->active_rows = rows;
    }
    void *buf[2] = {a, b};
    int cur = 0;
    const long long off = p->layout.origin;
    // One launch of t sweeps from buf[c] to buf[c ^ 1] on stream `on`.
    auto one_launch = [&](int t, int c, cudaStream_t on) -> cudaError_t {
        if (t >= 2)
            return cs::launch_split_sweep_tb(p->view, p->radius, p->pattern, t, p->w,
                                             (const float2 *)buf[c] + off, (float2 *)buf[c ^ 1] + off, on);
        return launch_sweep(p, algo, buf[c], buf[c ^ 1], on);
    };
    // Sweep i of this call is an FP64 re-anchor sweep.
    auto anchor = [&](long long i) {
        return p->prec == CS_PREC_SPLIT && p->reanchor > 0 && (first_sweep + i + 1) % p->reanchor == 0;
    };
    // Small grids spend a noticeable share of each sweep on launch gaps, so
    // blocks of an even number of launches are captured once as a CUDA graph
    // and replayed: same kernels, same order, same re-anchoring points, so the
    // result is bitwise the one of plain launches. Not used while the caller
    // is itself capturing `stream` (its capture records plain launches).
    long long pts = 1;
    for (int d = 0; d < p->dims; ++d) pts *= p->view.ext[d];
    const int glaunches = std::max(2, (cs::kGraphBlockSweeps / tb) & ~1);
    const long long gsweeps = (long long)glaunches * tb;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const bool graphs = pts <= cs::kGraphMaxPoints && sweeps >= 3 * gsweeps &&
                        cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone;
    // The graph of a block starting at buf[c], captured on the plan's private
    // stream the first time and cached in the plan.
    auto block_graph = [&](int c, cudaGraphExec_t *out) -> cs_status {
        std::lock_guard<std::mutex> lk(p->graph_mu);
        const auto key = std::make_tuple((const void *)buf[c], (const void *)buf[c ^ 1], algo, tb * 64 + p->active_rows,
                                         glaunches);
        auto it = p->graphs.find(key);
        if (it != p->graphs.end()) {
            *out = it->second;
            return CS_OK;
        }
        if (!p->capture_stream)
            CS_CUDA(cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking));
        CS_CUDA(cudaStreamBeginCapture(p->capture_stream, cudaStreamCaptureModeThreadLocal));
        const long long before = cs::g_launches.load();
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < glaunches && e == cudaSuccess; ++k)
            e = one_launch(tb, c ^ (k & 1), p->capture_stream);
        cs::note_launch(before - cs::g_launches.load());  // captured, not run: counted at each replay
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(p->capture_stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(e != cudaSuccess ? e : e2, "sweep capture");
        }
        cudaGraphExec_t ge = nullptr;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
        p->graphs[key] = ge;
        *out = ge;
        return CS_OK;
    };
    for (long long i = 0; i < sweeps;) {
        if (anchor(i)) {  // this sweep in FP64 (same buffer parity as any sweep)
            cudaError_t e = fp64_anchor_sweep(p, buf[cur], buf[cur ^ 1], st);
            if (e != cudaSuccess) return cuda_fail(e, "re-anchor sweep");
            cur ^= 1;
            ++i;
            continue;
        }
        // The first launch of a run is always plain, so any first-launch
        // set-up of a kernel has happened before a capture.
        if (graphs && i > 0 && sweeps - i >= gsweeps) {
            bool clean = true;  // no re-anchor sweep inside the block
            for (long long k = i; k < i + gsweeps; ++k)
                if (anchor(k)) clean = false;
            if (clean) {
                cudaGraphExec_t ge = nullptr;
                cs_status gs = block_graph(cur, &ge);
                if (gs != CS_OK) return gs;
                cudaError_t e = cudaGraphLaunch(ge, st);
                if (e != cudaSuccess) return cuda_fail(e, "graph launch");
                cs::note_launch(glaunches);
                i += gsweeps;  // even launch count: back in buf[cur]
                continue;
            }
        }
        // A temporally blocked launch stops short of the next re-anchor sweep.
        int t = (int)std::min<long long>(tb, sweeps - i);
        for (int k = 1; k < t; ++k)
            if (anchor(i + k)) {
                t = k;
                break;
            }
        cudaError_t e = one_launch(t, cur, st);
        if (e != cudaSuccess) return cuda_fail(e, "sweep launch");
        cur ^= 1;
        i += t;
    }
    if (result_in_b) *result_in_b = cur;
    return CS_OK;
}


}  // namespace cs

extern "C" {

CS_API const char *cs_status_string(cs_status s)
{
    switch (s) {
    case CS_OK: return "ok";
    case CS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CS_ERR_UNSUPPORTED: return "unsupported";
    case CS_ERR_CUDA: return "CUDA error";
    case CS_ERR_OUT_OF_MEMORY: return "out of memory";
    case CS_ERR_TIMEOUT: return "timeout";
    case CS_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

CS_API const char *cs_last_error(void) { return t_err.c_str(); }
CS_API void cs_set_verbose(int on) { g_verbose.store(on); }
CS_API double cs_last_loop_seconds(void) { return t_loop_seconds; }
CS_API long long cs_kernel_launch_count(void) { return cs::g_launches.load(); }
CS_API const char *cs_version(void) { return "convstencil_gb300 0.1 (sm_103a)"; }

CS_API cs_status cs_device_wait_timeouts(unsigned *count, int reset)
{
    if (!count) return fail(CS_ERR_INVALID_ARGUMENT, "count is NULL");
    unsigned a = 0, b = 0;
    CS_CUDA(cs::split_wait_timeouts(&a, reset != 0));
    CS_CUDA(cs::split_tc_wait_timeouts(&b, reset != 0));
    unsigned c3 = 0;
    CS_CUDA(cs::split_tc3d_wait_timeouts(&c3, reset != 0));
    b += c3;
    *count = a + b;
    return CS_OK;
}

CS_API cs_status cs_plan_create(cs_plan **out, cs_shape shape, cs_semantics sem, cs_precision prec,
                                const long long *extent, const double *weights, int n_weights,
                                const cs_layout *layout)
{
    if (!out) return fail(CS_ERR_INVALID_ARGUMENT, "plan pointer is NULL");
    *out = nullptr;
    if ((int)shape < 0 || (int)shape > 7) return fail(CS_ERR_INVALID_ARGUMENT, "unknown shape %d", (int)shape);
    if (sem != CS_SEM_STEP && sem != CS_SEM_FUSED)
        return fail(CS_ERR_INVALID_ARGUMENT, "unknown semantics %d", (int)sem);
    if (prec != CS_PREC_FP64 && prec != CS_PREC_SPLIT)
        return fail(CS_ERR_INVALID_ARGUMENT, "unknown precision %d", (int)prec);
    if (!extent || !weights) return fail(CS_ERR_INVALID_ARGUMENT, "extent or weights is NULL");
    const ShapeInfo &si = kShapes[shape];
    const int need = sem == CS_SEM_STEP ? si.n_base : si.n_fused;
    if (n_weights != need)
        return fail(CS_ERR_INVALID_ARGUMENT, "%s (%s) takes %d weights, got %d", si.name,
                    sem == CS_SEM_STEP ? "step" : "fused", need, n_weights);
    for (int i = 0; i < need; ++i)
        if (!std::isfinite(weights[i]))
            return fail(CS_ERR_INVALID_ARGUMENT, "weight %d is not finite", i);
    for (int d = 0; d < si.dims; ++d)
        if (extent[d] < 1 || extent[d] > (1LL << 31) - 1)
            return fail(CS_ERR_INVALID_ARGUMENT, "extent[%d] = %lld out of range", d, extent[d]);
    cs_plan *p = new (std::nothrow) cs_plan();
    if (!p) return fail(CS_ERR_OUT_OF_MEMORY, "plan allocation");
    p->shape = shape;
    p->sem = sem;
    p->prec = prec;
    p->dims = si.dims;
    p->steps_per_sweep = sem == CS_SEM_STEP ? 1 : si.fused_steps;
    expand_weights(shape, sem, weights, p->w, p->radius);
    p->pattern = classify(p->w, p->dims, p->radius);
    memset(p->w7.v, 0, sizeof p->w7.v);
    if (p->dims == 2 && p->radius <= 3) {
        const int k = 2 * p->radius + 1, o = 3 - p->radius;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) p->w7.v[(i + o) * 7 + j + o] = p->w.v[i * k + j];
    } else if (p->dims == 1 && p->radius <= 3) {  // the taps in row 3 of the 7x7
        for (int j = 0; j <= 2 * p->radius; ++j) p->w7.v[3 * 7 + 3 - p->radius + j] = p->w.v[j];
    }
    if (layout) {
        const cs_layout &L = *layout;
        bool ok = L.dims == si.dims && L.halo >= p->radius && L.pitch[si.dims - 1] == 1;
        for (int d = 0; ok && d < si.dims; ++d) ok = L.extent[d] == extent[d] && L.pitch[d] >= 1;
        if (ok && si.dims >= 2) ok = L.pitch[si.dims - 2] >= L.extent[si.dims - 1] + 2 * p->radius;
        if (ok && si.dims == 3) ok = L.pitch[0] >= L.pitch[1] * (L.extent[1] + 2 * p->radius);
        if (ok) {
            // every point within the radius of the interior (the box around
            // it) lies in the buffer: the kernels read all of them
            __int128 lo = L.origin, hi = L.origin;
            for (int d = 0; d < si.dims; ++d) {
                lo -= (__int128)p->radius * L.pitch[d];
                hi += (__int128)(L.extent[d] - 1 + p->radius) * L.pitch[d];
            }
            ok = lo >= 0 && hi < (__int128)L.elements;
        }
        if (!ok) {
            const int r = p->radius;
            delete p;
            return fail(CS_ERR_INVALID_ARGUMENT, "layout does not fit the grid with halo %d", r);
        }
        p->layout = L;
        p->layout.bytes = (size_t)L.elements * sizeof(double);
    } else {
        native_layout(si.dims, p->radius, extent, p->layout);
    }
    p->view.dims = si.dims;
    for (int d = 0; d < 3; ++d) {
        p->view.ext[d] = d < si.dims ? p->layout.extent[d] : 1;
        p->view.pitch[d] = d < si.dims ? p->layout.pitch[d] : 1;
    }
    const bool supported = prec == CS_PREC_FP64
                               ? cs::fp64_fma_supported(p->dims, p->radius, p->pattern)
                               : cs::split_supported(p->dims, p->radius, p->pattern);
    if (!supported) {
        const int r = p->radius, pat = p->pattern;
        delete p;
        return fail(CS_ERR_UNSUPPORTED, "no kernel for dims=%d radius=%d pattern=%d precision=%d", si.dims, r, pat,
                    (int)prec);
    }
    *out = p;
    return CS_OK;
}

CS_API cs_status cs_plan_set_option(cs_plan *p, cs_option opt, long long v)
{
    if (!p) return fail(CS_ERR_INVALID_ARGUMENT, "plan is NULL");
    switch (opt) {
    case CS_OPT_ALGO:
        if (v < CS_ALGO_AUTO || v > CS_ALGO_FP64_TC) return fail(CS_ERR_INVALID_ARGUMENT, "bad algo");
        if ((v == CS_ALGO_SPLIT_MMA || v == CS_ALGO_SPLIT_FMA || v == CS_ALGO_SPLIT_MMA_TMA ||
             v == CS_ALGO_SPLIT_TC) &&
            p->prec != CS_PREC_SPLIT)
            return fail(CS_ERR_INVALID_ARGUMENT, "split algo needs a split-precision plan");
        if ((v == CS_ALGO_FP64_FMA || v == CS_ALGO_FP64_MMA || v == CS_ALGO_FP64_TC) && p->prec != CS_PREC_FP64)
            return fail(CS_ERR_INVALID_ARGUMENT, "FP64 algo needs an FP64 plan");
        if (v == CS_ALGO_FP64_MMA && !fp64_mma_ok(p))
            return fail(CS_ERR_UNSUPPORTED, "FP64 MMA serves 2D radius-3 dense FP64 plans only");
        if (v == CS_ALGO_FP64_TC && !fp64_tc_ok(p) && !fp64_tc3d_ok(p) && !fp64_tc1d_ok(p))
            return fail(CS_ERR_UNSUPPORTED,
                        "FP64 tcgen05 serves 2D FP64 plans of radius up to 3 and at least 8x8 on even-aligned "
                        "layouts, 3D radius-1 FP64 plans and 1D FP64 plans of radius up to 3 whose length is a "
                        "multiple of 64 (at least 512) with 4 points of halo before and 60 after the interior");
        if (v == CS_ALGO_SPLIT_TC && split_tc3d_ok(p)) {
            p->algo = (int)v;
            return CS_OK;
        }
        if ((v == CS_ALGO_SPLIT_MMA || v == CS_ALGO_SPLIT_MMA_TMA || v == CS_ALGO_SPLIT_TC) &&
            !split_mma_ok(p))
            return fail(CS_ERR_UNSUPPORTED,
                        "split MMA serves 2D radius-3 plans of at least 8x8 on even-aligned layouts "
                        "(and tcgen05 also 3D radius-1 plans)");
        p->algo = (int)v;
        return CS_OK;
    case CS_OPT_REANCHOR_INTERVAL:
        if (v < 0) return fail(CS_ERR_INVALID_ARGUMENT, "negative re-anchor interval");
        p->reanchor = v;
        return CS_OK;
    case CS_OPT_TIME_BLOCK:
        if (v < 0 || v > 4) return fail(CS_ERR_INVALID_ARGUMENT, "time block must be 0 (tuner) or 1..4");
        if (v > 1 && !(p->prec == CS_PREC_SPLIT && cs::split_tb_supported(p->dims, p->radius, p->pattern)))
            return fail(CS_ERR_UNSUPPORTED,
                        "temporal blocking serves split-precision 2D radius-1 and 1D plans");
        p->time_block = (int)v;
        return CS_OK;
    case CS_OPT_TILE_ROWS:
        if (v != 0 && v != 16 && v != 32) return fail(CS_ERR_INVALID_ARGUMENT, "tile rows must be 0 (tuner), 16 or 32");
        if (v != 0 && !(p->prec == CS_PREC_FP64 && p->dims == 2))
            return fail(CS_ERR_UNSUPPORTED, "tile rows apply to FP64 2D plans (FMA kernel)");
        p->tile_rows = (int)v;
        return CS_OK;
    case CS_OPT_WAIT_LIMIT_US:
        if (v < 1 || v > 60000000LL)
            return fail(CS_ERR_INVALID_ARGUMENT, "wait limit must be 1 .. 60,000,000 microseconds");
        p->wait.limit_ns = (unsigned long long)v * 1000ull;
        return CS_OK;
    case CS_OPT_WAIT_TEST_SKIP_LOADS:
        if (v != 0 && v != 1) return fail(CS_ERR_INVALID_ARGUMENT, "skip-loads test hook is 0 or 1");
        p->wait.skip_loads = (int)v;
        return CS_OK;
    }
    return fail(CS_ERR_INVALID_ARGUMENT, "unknown option %d", (int)opt);
}

CS_API cs_status cs_plan_get_layout(const cs_plan *p, cs_layout *out)
{
    if (!p || !out) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = p->layout;
    return CS_OK;
}

CS_API cs_status cs_plan_sweeps(const cs_plan *p, long long steps, long long *sweeps)
{
    if (!p || !sweeps) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (steps < 0) return fail(CS_ERR_INVALID_ARGUMENT, "negative step count");
    if (steps % p->steps_per_sweep)
        return fail(CS_ERR_INVALID_ARGUMENT, "%lld steps is not a multiple of the %d steps of a fused sweep",
                    steps, p->steps_per_sweep);
    *sweeps = steps / p->steps_per_sweep;
    return CS_OK;
}

CS_API cs_status cs_plan_get_algo(const cs_plan *p, int *algo)
{
    if (!p || !algo) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    *algo = p->last_algo;
    return CS_OK;
}

CS_API cs_status cs_plan_get_tile_rows(const cs_plan *p, int *rows)
{
    if (!p || !rows) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    *rows = p->active_rows;
    return CS_OK;
}

CS_API cs_status cs_plan_get_time_block(const cs_plan *p, int *steps_per_launch)
{
    if (!p || !steps_per_launch) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    *steps_per_launch = p->last_time_block;
    return CS_OK;
}

CS_API cs_status cs_plan_destroy(cs_plan *p)
{
    delete p;
    return CS_OK;
}

CS_API cs_status cs_run(cs_plan *p, void *a, void *b, long long steps, void *stream, int *result_in_b)
{
    return cs::run_from(p, a, b, 0, steps, (cudaStream_t)stream, result_in_b);
}

CS_API cs_status cs_split_from_fp64(const cs_plan *p, const double *src, void *dst, void *stream)
{
    if (!p || !src || !dst) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    // Converts the whole buffer (interior and halo) so halos stay exact.
    CS_CUDA(cs::launch_split_from_fp64(p->layout.elements, src, (float2 *)dst, (cudaStream_t)stream));
    return CS_OK;
}

CS_API cs_status cs_split_to_fp64(const cs_plan *p, const void *src, double *dst, void *stream)
{
    if (!p || !src || !dst) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    CS_CUDA(cs::launch_split_to_fp64(p->layout.elements, (const float2 *)src, dst, (cudaStream_t)stream));
    return CS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------
// Host-buffer runs (the reference wrappers' contract).
namespace {

struct DevBuf {
    void *p = nullptr;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
};

// in_elems doubles from host_in into buffer 0 (buffer 1 zero), `sweeps`
// sweeps, then out_elems doubles from result + out_offset to host_out.
// Host-buffer run with the copies overlapped: the grid goes to the device in
// row bands (slabs of the slowest axis) on one stream while the sweeps run
// as a wavefront over the bands on another (sweep s of band k once sweep
// s - 1 of bands k - 1 .. k + 1 is done, band k + 1 of the input having
// arrived for the first sweep), and each band goes back as soon as its last
// sweep is done. Launches are issued diagonal by diagonal on one stream, so
// sweep s of band k always precedes sweep s + 1 of band k - 1, which
// overwrites rows that it reads. Used when the kernel is known without a
// timing run, no temporal blocking and no re-anchor sweep is involved, and
// the whole grid goes both ways.
// Whether the band-sweeps of a host-buffer run go to the tcgen05 batch
// kernel: 2D split plans on SPLIT_TC (the 2D radius-3 tile geometry). On
// GB300, 20 sweeps of 8192^2 with the copies: 10.3 ms in 32 bands of batched
// sets against 11.7 in 8 bands of one launch each; FP64 plans gain nothing
// from the batches (12.1 against 11.9 ms), whose kernel runs 5 % slower than
// the one-grid kernel, and keep one launch per band-sweep.
bool band_batch_ok(const cs_plan *p, int algo)
{
    return p->prec == CS_PREC_SPLIT && algo == CS_ALGO_SPLIT_TC && p->radius == 3 && fp64_tc_geometry_ok(p);
}

// `kept`: the run uses the plan's kept grids (batched sets allowed).
bool banded_ok(cs_plan *p, long long sweeps, bool kept, int *algo, int *bands)
{
    if (p->dims < 2 || sweeps < 1) return false;
    if (p->prec == CS_PREC_SPLIT && cs::split_tb_supported(p->dims, p->radius, p->pattern) && p->time_block != 1)
        return false;
    if (p->prec == CS_PREC_SPLIT && p->reanchor > 0 && sweeps >= p->reanchor) return false;
    if (choose_algo(p, nullptr, nullptr, nullptr, algo, false) != CS_OK || *algo < 0) return false;
    const long long slabs = p->view.ext[0];
    if (kept && band_batch_ok(p, *algo)) {
        *bands = (int)std::min<long long>(32, slabs / 256);  // one batch launch per set
    } else {
        const long long per = p->dims == 2 ? 1024 : 64;  // slabs per band at least
        *bands = (int)std::min<long long>(8, slabs / per);
    }
    return *bands >= 2;
}

// Band-sweep (k, s) is sweep s (0-based) of the interior slabs of band k: it
// reads level s of bands k-1 .. k+1 (grid s % 2) and writes level s+1 of band
// k (grid (s+1) % 2). Its inputs come from (k-1, s-1), (k, s-1), (k+1, s-1),
// and the level s-1 it overwrites was last read by the same three, so with
// c = 2s + k every dependency points from set c to sets c-1, c-2, c-3: the
// band-sweeps of one set are independent (neighbouring bands are never in
// the same set, and bands are taller than the halo), and the sets in order
// c = 0, 1, ... form a wavefront that starts on the first bands while later
// ones are still arriving. Set c needs band c + 1 on the device when c < K.
struct BandMember {
    int k;
    long long s;
};
static std::vector<BandMember> band_set(int bands, long long sweeps, long long c)
{
    std::vector<BandMember> m;
    for (long long sw = std::max(0LL, (c - bands + 2) / 2); sw <= std::min(sweeps - 1, c / 2); ++sw) {
        const long long k = c - 2 * sw;
        if (k >= 0 && k < bands) m.push_back({(int)k, sw});
    }
    return m;
}

// The batch records of every set (sets whose members have the same bands
// and grid parities share them: in the middle of a long run the pattern
// repeats every four sets), uploaded once per bands, sweeps and grids.
static cs_status band_table(cs_plan *p, int algo, int bands, long long sweeps, void *const d[2],
                            const std::vector<long long> &b)
{
    auto &T = p->band;
    if (T.tab && T.bands == bands && T.sweeps == sweeps && T.algo == algo && T.d0 == d[0] && T.d1 == d[1])
        return CS_OK;
    if (T.tab) cudaFree(T.tab), T.tab = nullptr;
    T.sets.clear();
    const bool fp64 = p->prec == CS_PREC_FP64;
    const size_t rb = cs::tc_batch_record_bytes(fp64);
    std::vector<unsigned char> rec;
    std::map<std::vector<long long>, cs_plan::BandSet> seen;
    const long long nsets = 2 * (sweeps - 1) + bands;
    for (long long c = 0; c < nsets; ++c) {
        const auto mem = band_set(bands, sweeps, c);
        std::vector<long long> sig;
        for (const auto &x : mem) sig.push_back(2 * x.k + (x.s & 1));
        auto it = seen.find(sig);
        if (it == seen.end()) {
            cs_plan::BandSet bs{(long long)(rec.size() / rb), (int)mem.size(), 0};
            for (const auto &x : mem) {
                GridView v = p->view;
                v.ext[0] = b[x.k + 1] - b[x.k];
                const long long off = p->layout.origin + b[x.k] * p->view.pitch[0];
                rec.resize(rec.size() + rb);
                int tiles = 0;
                const cudaError_t e = cs::tc_batch_fill_record(fp64, rec.data() + rec.size() - rb, v, p->w, off,
                                                               p->layout.elements, d[x.s & 1], d[(x.s + 1) & 1],
                                                               bs.tiles, 0, &tiles);
                if (e != cudaSuccess) return fail(CS_ERR_CUDA, "band record: %s", cudaGetErrorString(e));
                bs.tiles += tiles;
            }
            it = seen.emplace(sig, bs).first;
        }
        T.sets.push_back(it->second);
    }
    CS_CUDA(cudaMalloc(&T.tab, rec.size()));
    CS_CUDA(cudaMemcpy(T.tab, rec.data(), rec.size(), cudaMemcpyHostToDevice));
    T.bands = bands;
    T.sweeps = sweeps;
    T.algo = algo;
    T.d0 = d[0];
    T.d1 = d[1];
    return CS_OK;
}

// `kept`: d are the plan's kept grids and the caller holds host_mu, so the
// plan's cached band records (p->band) may be used and rebuilt; a call on
// grids of its own (another thread holds the kept ones) launches its
// band-sweeps one by one and leaves the cache alone.
cs_status host_run_banded(cs_plan *p, int algo, int bands, const double *host_in, double *host_out,
                          long long sweeps, void *const d[2], bool kept, double *loop_seconds)
{
    const long long ld0 = p->view.pitch[0];        // elements per slab
    const long long total = p->layout.elements / ld0;  // slabs in the buffer, halo included
    const long long first = p->layout.origin / ld0;    // halo slabs before the interior
    const long long slabs = p->view.ext[0];
    const long long align = p->dims == 2 ? 64 : 8;
    std::vector<long long> b(bands + 1);  // interior slab boundaries of the bands
    for (int k = 0; k <= bands; ++k) b[k] = std::min(slabs, (slabs * k / bands + align - 1) / align * align);
    b[bands] = slabs;
    std::vector<long long> c(bands + 1);  // buffer slab boundaries of the copy chunks
    for (int k = 0; k <= bands; ++k) c[k] = k == 0 ? 0 : k == bands ? total : first + b[k];
    // The tcgen05 batch kernel takes a whole set per launch when every band
    // meets its layout conditions; otherwise each band-sweep is a launch.
    bool batch = kept && band_batch_ok(p, algo) && reinterpret_cast<uintptr_t>(d[0]) % 16 == 0 &&
                 reinterpret_cast<uintptr_t>(d[1]) % 16 == 0;
    for (int k = 0; k < bands && batch; ++k) {
        GridView v = p->view;
        v.ext[0] = b[k + 1] - b[k];
        const long long off = p->layout.origin + b[k] * ld0;
        batch = cs::split_tma_layout_ok(v, off, d[0]) && cs::split_tma_layout_ok(v, off, d[1]);
    }
    if (batch) {
        const cs_status st = band_table(p, algo, bands, sweeps, d, b);
        if (st != CS_OK) return st;
    }
    struct Streams {
        cudaStream_t s[3] = {nullptr, nullptr, nullptr};
        std::vector<cudaEvent_t> ev;
        ~Streams()
        {
            for (cudaEvent_t e : ev) cudaEventDestroy(e);
            for (cudaStream_t x : s)
                if (x) cudaStreamDestroy(x);
        }
    } S;
    for (auto &x : S.s) CS_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
    cudaStream_t sc = S.s[0], sh = S.s[1], sd = S.s[2];
    S.ev.resize(2 * bands + 2);
    for (auto &e : S.ev) CS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDefault));
    cudaEvent_t *in_ev = S.ev.data(), *out_ev = S.ev.data() + bands, e0 = S.ev[2 * bands], e1 = S.ev[2 * bands + 1];
    const size_t slab_bytes = (size_t)ld0 * sizeof(double);
    CS_CUDA(cudaMemsetAsync(d[1], 0, (size_t)p->layout.bytes, sc));  // the second grid's halo reads as zero
    // The copies in go back to back on their own stream; a split plan's band
    // is converted to (hi, lo) on the sweep stream just before its first use
    // (on the copy stream, each conversion held up the next copy while the
    // sweep kernel filled the SMs: 8192^2 in 4.1 ms instead of 2.6).
    for (int k = 0; k < bands; ++k) {
        const long long cnt = (c[k + 1] - c[k]) * ld0;
        char *dst = (char *)d[0] + c[k] * slab_bytes;
        CS_CUDA(cudaMemcpyAsync(dst, host_in + c[k] * ld0, (size_t)cnt * sizeof(double), cudaMemcpyHostToDevice, sh));
        CS_CUDA(cudaEventRecord(in_ev[k], sh));
    }
    CS_CUDA(cudaEventRecord(e0, sc));
    int arrived = 0;  // bands copied and converted, as the sweep stream sees them
    auto arrive = [&](int upto) -> cs_status {  // bands 0 .. upto on the device, converted
        for (; arrived <= upto; ++arrived) {
            CS_CUDA(cudaStreamWaitEvent(sc, in_ev[arrived], 0));
            if (p->prec == CS_PREC_SPLIT)
                CS_CUDA(cs::launch_fp64_to_split_inplace((c[arrived + 1] - c[arrived]) * ld0,
                                                         (char *)d[0] + c[arrived] * slab_bytes, sc));
        }
        return CS_OK;
    };
    void *f = d[sweeps & 1];  // final grid
    const bool fp64 = p->prec == CS_PREC_FP64;
    const size_t rb = batch ? cs::tc_batch_record_bytes(fp64) : 0;
    auto band_done = [&](int k) -> cs_status {  // band k is final: back to the host now
        const long long cnt = (c[k + 1] - c[k]) * ld0;
        char *src = (char *)f + c[k] * slab_bytes;
        if (p->prec == CS_PREC_SPLIT) CS_CUDA(cs::launch_split_to_fp64_inplace(cnt, src, sc));
        CS_CUDA(cudaEventRecord(out_ev[k], sc));
        CS_CUDA(cudaStreamWaitEvent(sd, out_ev[k], 0));
        CS_CUDA(cudaMemcpyAsync(host_out + c[k] * ld0, src, (size_t)cnt * sizeof(double), cudaMemcpyDeviceToHost, sd));
        return CS_OK;
    };
    if (batch) {
        // One batch launch per set c = 2s + k (band_set).
        const long long nsets = 2 * (sweeps - 1) + bands;
        for (long long set = 0; set < nsets; ++set) {
            if (set < bands) {
                const cs_status st = arrive((int)std::min<long long>(set + 1, bands - 1));
                if (st != CS_OK) return st;
            }
            const cs_plan::BandSet &bs = p->band.sets[set];
            CS_CUDA(cs::launch_tc_batch(fp64, (const char *)p->band.tab + bs.rec * rb, bs.count, bs.tiles, p->wait,
                                        sc));
            for (const auto &x : band_set(bands, sweeps, set))
                if (x.s == sweeps - 1) {
                    const cs_status st = band_done(x.k);
                    if (st != CS_OK) return st;
                }
        }
    } else {
        // One launch per band-sweep, diagonal by diagonal (d = k + s): a
        // topological order too, with (k, s) launched before (k - 1, s + 1),
        // which overwrites the rows it reads; (k, 0) waits for bands k, k + 1.
        for (long long diag = 0; diag < bands + sweeps - 1; ++diag) {
            for (long long sw = std::max(0LL, diag - (bands - 1)); sw <= std::min(sweeps - 1, diag); ++sw) {
                const int k = (int)(diag - sw);
                if (sw == 0) {
                    const cs_status st = arrive(std::min(k + 1, bands - 1));
                    if (st != CS_OK) return st;
                }
                CS_CUDA(launch_sweep_rows(p, algo, d[sw & 1], d[(sw + 1) & 1], b[k], b[k + 1] - b[k], sc));
                if (sw == sweeps - 1) {
                    const cs_status st = band_done(k);
                    if (st != CS_OK) return st;
                }
            }
        }
    }
    CS_CUDA(cudaEventRecord(e1, sc));
    CS_CUDA(cudaStreamSynchronize(sd));
    CS_CUDA(cudaStreamSynchronize(sc));
    float ms = 0.f;
    CS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (loop_seconds) *loop_seconds = ms * 1e-3;
    t_loop_seconds = ms * 1e-3;
    return CS_OK;
}

cs_status host_run(cs_plan *p, const double *host_in, size_t in_elems, double *host_out,
                   size_t out_offset, size_t out_elems, long long steps, double *loop_seconds)
{
    long long sweeps = 0;
    cs_status s = cs_plan_sweeps(p, steps, &sweeps);
    if (s != CS_OK) return s;
    const size_t bytes = p->layout.bytes;
    const size_t elem_bytes = sizeof(double);
    const long long n = p->layout.elements;
    // Two device grids: the plan's kept pair when no other thread holds it.
    std::unique_lock<std::mutex> kept(p->host_mu, std::try_to_lock);
    DevBuf own[2];
    void *d[2];
    if (kept.owns_lock()) {
        if (p->host_bytes < bytes) {
            for (void *&b : p->host_bufs)
                if (b) cudaFree(b), b = nullptr;
            p->host_bytes = 0;
            CS_CUDA(cudaMalloc(&p->host_bufs[0], bytes));
            CS_CUDA(cudaMalloc(&p->host_bufs[1], bytes));
            p->host_bytes = bytes;
        }
        d[0] = p->host_bufs[0];
        d[1] = p->host_bufs[1];
    } else {
        CS_CUDA(cudaMalloc(&own[0].p, bytes));
        CS_CUDA(cudaMalloc(&own[1].p, bytes));
        d[0] = own[0].p;
        d[1] = own[1].p;
    }
    const bool whole = in_elems * elem_bytes == bytes;
    int balgo = 0, bands = 0;
    if (whole && out_offset == 0 && out_elems == (size_t)n && banded_ok(p, sweeps, kept.owns_lock(), &balgo, &bands)) {
        unsigned w0 = 0, w1 = 0;
        s = cs_device_wait_timeouts(&w0, 0);
        if (s != CS_OK) return s;
        s = host_run_banded(p, balgo, bands, host_in, host_out, sweeps, d, kept.owns_lock(), loop_seconds);
        if (s != CS_OK) return s;
        p->last_algo = balgo;
        p->last_time_block = 1;
        s = cs_device_wait_timeouts(&w1, 0);
        if (s != CS_OK) return s;
        if (w1 != w0)
            return fail(CS_ERR_TIMEOUT, "%u bounded device-side wait(s) expired during the run; the result is incomplete",
                        w1 - w0);
        return CS_OK;
    }
    // The copy fills the first grid completely unless the caller passes a
    // part of it; the second grid's halo must read as zero. A split plan's
    // grid is converted from FP64 in place (same 8 bytes per point).
    if (!whole) CS_CUDA(cudaMemset(d[0], 0, bytes));
    CS_CUDA(cudaMemset(d[1], 0, bytes));
    CS_CUDA(cudaMemcpy(d[0], host_in, in_elems * elem_bytes, cudaMemcpyHostToDevice));
    if (p->prec == CS_PREC_SPLIT) CS_CUDA(cs::launch_fp64_to_split_inplace(n, d[0], nullptr));
    // Bounded device-side waits that expire during this call leave outputs
    // unwritten; the counters before and after tell (any expiry in the
    // process during the call counts).
    unsigned waits_before = 0, waits_after = 0;
    s = cs_device_wait_timeouts(&waits_before, 0);
    if (s != CS_OK) return s;
    cudaEvent_t e0, e1;
    CS_CUDA(cudaEventCreate(&e0));
    CS_CUDA(cudaEventCreate(&e1));
    CS_CUDA(cudaEventRecord(e0, nullptr));
    int in_b = 0;
    s = cs_run(p, d[0], d[1], steps, nullptr, &in_b);
    if (s != CS_OK) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return s;
    }
    CS_CUDA(cudaEventRecord(e1, nullptr));
    CS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    CS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (loop_seconds) *loop_seconds = ms * 1e-3;
    t_loop_seconds = ms * 1e-3;
    s = cs_device_wait_timeouts(&waits_after, 0);
    if (s != CS_OK) return s;
    if (waits_after != waits_before)
        return fail(CS_ERR_TIMEOUT, "%u bounded device-side wait(s) expired during the run; the result is incomplete",
                    waits_after - waits_before);
    void *res = d[in_b];
    if (p->prec == CS_PREC_SPLIT) CS_CUDA(cs::launch_split_to_fp64_inplace(n, res, nullptr));
    CS_CUDA(cudaMemcpy(host_out, (const double *)res + out_offset, out_elems * elem_bytes,
                       cudaMemcpyDeviceToHost));
    return CS_OK;
}

cs_status make_ref_plan(cs_plan **p, cs_shape shape, const long long *ext, const double *params,
                        const cs_layout &L)
{
    const ShapeInfo &si = kShapes[shape];
    return cs_plan_create(p, shape, CS_SEM_FUSED, CS_PREC_FP64, ext, params, si.n_fused, &L);
}

void print_timing(const char *banner, bool secs_line, double secs, double points, int steps_mult,
                  int times)
{
    if (!g_verbose.load()) return;
    if (banner) printf("%s\n", banner);
    printf("Time = %lld[ms]\n", (long long)(secs * 1e3));
    if (secs_line) printf("%g\n", secs);
    printf("GStencil/s = %f\n", points * (double)times * steps_mult / secs / 1e9);
    fflush(stdout);
}

// The reference-shaped wrappers keep the plan of their latest call, with the
// two device grids host_run keeps in it, for the next call with the same
// shape, layout and weights: repeated calls (a solver's time loop) skip the
// plan set-up and the grid allocation. A call with other arguments replaces
// it, cs_release_cached_plan() frees it. The cache is never destroyed by a
// static destructor (the CUDA runtime may be gone by then); the process exit
// returns its memory.
struct RefPlanCache {
    std::mutex mu;
    std::shared_ptr<cs_plan> plan;
    std::vector<long long> key;
};
RefPlanCache &ref_cache()
{
    static RefPlanCache *c = new RefPlanCache;
    return *c;
}

cs_status ref_plan(std::shared_ptr<cs_plan> *out, cs_shape shape, const long long *ext, const double *params,
                   const cs_layout &L)
{
    const int nw = kShapes[shape].n_fused;
    std::vector<long long> key = {(long long)shape, L.dims, L.halo, L.origin, L.elements};
    for (int d = 0; d < L.dims; ++d) key.insert(key.end(), {L.extent[d], L.pitch[d]});
    for (int i = 0; i < nw; ++i) {
        long long bits;
        std::memcpy(&bits, &params[i], sizeof bits);
        key.push_back(bits);
    }
    RefPlanCache &c = ref_cache();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        if (c.plan && c.key == key) {
            *out = c.plan;
            return CS_OK;
        }
    }
    cs_plan *p = nullptr;
    const cs_status s = make_ref_plan(&p, shape, ext, params, L);
    if (s != CS_OK) return s;
    std::shared_ptr<cs_plan> sp(p, cs_plan_destroy);
    {
        std::lock_guard<std::mutex> lk(c.mu);
        c.plan = sp;
        c.key = std::move(key);
    }
    *out = std::move(sp);
    return CS_OK;
}

cs_status check_ref_args(const void *in, const void *out, const void *params, int times,
                         std::initializer_list<int> dims)
{
    if (!in || !out || !params) return fail(CS_ERR_INVALID_ARGUMENT, "NULL buffer or params");
    if (times < 0) return fail(CS_ERR_INVALID_ARGUMENT, "negative times");
    for (int d : dims)
        if (d < 1) return fail(CS_ERR_INVALID_ARGUMENT, "grid extent %d < 1", d);
    return CS_OK;
}

}  // namespace

extern "C" {

CS_API void cs_release_cached_plan(void)
{
    std::shared_ptr<cs_plan> old;
    RefPlanCache &c = ref_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    old.swap(c.plan);
    c.key.clear();
}

CS_API cs_status cs_run_host(cs_plan *p, const double *host_in, double *host_out, long long steps)
{
    if (!p || !host_in || !host_out) return fail(CS_ERR_INVALID_ARGUMENT, "NULL argument");
    const size_t n = (size_t)p->layout.elements;
    return host_run(p, host_in, n, host_out, 0, n, steps, nullptr);
}

// src/1d/gpu_1r.cu:227-302. Device grid n+7 (index 0 pad, halo 3); the
// result is read back from device index 1 (src/1d/gpu_1r.cu:299).
CS_API cs_status cs_gpu_1d1r(const double *in, double *out, const double *params, int times, int n)
{
    cs_status s = check_ref_args(in, out, params, times, {n});
    if (s != CS_OK) return s;
    cs_layout L{};
    L.dims = 1;
    L.halo = 3;
    L.extent[0] = n;
    L.pitch[0] = 1;
    L.origin = 4;
    L.elements = (long long)n + 7;
    const long long ext[1] = {n};
    std::shared_ptr<cs_plan> g;
    s = ref_plan(&g, CS_SHAPE_1D1R, ext, params, L);
    if (s != CS_OK) return s;
    double secs = 0;
    s = host_run(g.get(), in, (size_t)n + 7, out, 1, (size_t)n + 6, 3LL * times, &secs);
    if (s == CS_OK) print_timing("ConvStencil(1D): ", false, secs, (double)n, 3, times);
    return s;
}

// src/1d/gpu_2r.cu:85-159. Device grid n+8 (halo 4); n+7 values come back
// (src/1d/gpu_2r.cu:156).
CS_API cs_status cs_gpu_star_1d2r_step2(const double *in, double *out, const double *params,
                                        int times, int n)
{
    cs_status s = check_ref_args(in, out, params, times, {n});
    if (s != CS_OK) return s;
    cs_layout L{};
    L.dims = 1;
    L.halo = 4;
    L.extent[0] = n;
    L.pitch[0] = 1;
    L.origin = 4;
    L.elements = (long long)n + 8;
    const long long ext[1] = {n};
    std::shared_ptr<cs_plan> g;
    s = ref_plan(&g, CS_SHAPE_1D2R, ext, params, L);
    if (s != CS_OK) return s;
    double secs = 0;
    s = host_run(g.get(), in, (size_t)n + 8, out, 0, (size_t)n + 7, 2LL * times, &secs);
    if (s == CS_OK) print_timing(nullptr, false, secs, (double)n, 2, times);
    return s;
}

static cs_status gpu_2d(cs_shape shape, const double *in, double *out, const double *params,
                        int times, int m, int n, int steps_mult)
{
    cs_status s = check_ref_args(in, out, params, times, {m, n});
    if (s != CS_OK) return s;
    // (m+6) x (n+8), interior rows [3, m+3), cols [4, n+4) (src/2d/gpu.cu:359-360).
    cs_layout L{};
    L.dims = 2;
    L.halo = 3;
    L.extent[0] = m;
    L.extent[1] = n;
    L.pitch[0] = (long long)n + 8;
    L.pitch[1] = 1;
    L.origin = 3 * L.pitch[0] + 4;
    L.elements = ((long long)m + 6) * L.pitch[0];
    const long long ext[2] = {m, n};
    std::shared_ptr<cs_plan> g;
    s = ref_plan(&g, shape, ext, params, L);
    if (s != CS_OK) return s;
    double secs = 0;
    const size_t all = (size_t)L.elements;
    s = host_run(g.get(), in, all, out, 0, all, (long long)steps_mult * times, &secs);
    if (s == CS_OK) print_timing("ConvStencil(2D): ", false, secs, (double)m * n, steps_mult, times);
    return s;
}

// src/2d/gpu.cu:245-334 (3 steps per sweep).
CS_API cs_status cs_gpu_box_2d1r(const double *in, double *out, const double *params, int times,
                                 int m, int n)
{
    return gpu_2d(CS_SHAPE_BOX2D1R, in, out, params, times, m, n, 3);
}

// src/2d/gpu.cu:336-425 (1 step per sweep).
CS_API cs_status cs_gpu_box_2d3r(const double *in, double *out, const double *params, int times,
                                 int m, int n)
{
    return gpu_2d(CS_SHAPE_BOX2D3R, in, out, params, times, m, n, 1);
}

static cs_status gpu_3d(cs_shape shape, const double *in, double *out, const double *params,
                        int times, int h, int m, int n, const char *banner)
{
    cs_status s = check_ref_args(in, out, params, times, {h, m, n});
    if (s != CS_OK) return s;
    // (h+6) x (m+6) x (n+6), halo 3 on every axis (src/3d/gpu_box.cu:475-478).
    cs_layout L{};
    L.dims = 3;
    L.halo = 3;
    L.extent[0] = h;
    L.extent[1] = m;
    L.extent[2] = n;
    L.pitch[2] = 1;
    L.pitch[1] = (long long)n + 6;
    L.pitch[0] = L.pitch[1] * ((long long)m + 6);
    L.origin = 3 * L.pitch[0] + 3 * L.pitch[1] + 3;
    L.elements = ((long long)h + 6) * L.pitch[0];
    const long long ext[3] = {h, m, n};
    std::shared_ptr<cs_plan> g;
    s = ref_plan(&g, shape, ext, params, L);
    if (s != CS_OK) return s;
    double secs = 0;
    const size_t all = (size_t)L.elements;
    s = host_run(g.get(), in, all, out, 0, all, 3LL * times, &secs);
    if (s == CS_OK) print_timing(banner, true, secs, (double)h * m * n, 3, times);
    return s;
}

// src/3d/gpu_box.cu:446-536.
CS_API cs_status cs_gpu_box_3d1r(const double *in, double *out, const double *params, int times,
                                 int h, int m, int n)
{
    return gpu_3d(CS_SHAPE_BOX3D1R, in, out, params, times, h, m, n, "ConvStencil(3D): ");
}

// src/3d/gpu_star.cu:238-332.
CS_API cs_status cs_gpu_star_3d1r(const double *in, double *out, const double *params, int times,
                                  int h, int m, int n)
{
    return gpu_3d(CS_SHAPE_STAR3D1R, in, out, params, times, h, m, n, nullptr);
}

}  // extern "C"

// ------------------------------------------------------------------------
// Sweeps from a read-only input into an output through a caller-supplied
// intermediate grid, with no allocation and no tuning run: the algorithm is
// the one the tuner already chose for this plan's class, else the default.
// Used by the no-allocation entry point (cs_noalloc.cu).
namespace cs {

size_t plan_bytes(const cs_plan *p) { return p->layout.bytes; }

cs_status run_into(cs_plan *p, const void *in, void *out, void *scratch, long long steps,
                   cudaStream_t st)
{
    if (reinterpret_cast<uintptr_t>(in) % 8 || reinterpret_cast<uintptr_t>(out) % 8)
        return fail(CS_ERR_INVALID_ARGUMENT, "grid buffers must be 8-byte aligned (double / float2 elements)");
    long long sweeps = 0;
    cs_status s = cs_plan_sweeps(p, steps, &sweeps);
    if (s != CS_OK) return s;
    if (sweeps == 0) {
        CS_CUDA(cudaMemcpyAsync(out, in, p->layout.bytes, cudaMemcpyDeviceToDevice, st));
        return CS_OK;
    }
    int algo;
    if (p->prec == CS_PREC_SPLIT)
        algo = p->algo != CS_ALGO_AUTO ? p->algo : (split_mma_ok(p) ? CS_ALGO_SPLIT_MMA : CS_ALGO_SPLIT_FMA);
    else
        algo = p->algo != CS_ALGO_AUTO ? p->algo : CS_ALGO_FP64_FMA;
    if (p->algo == CS_ALGO_AUTO) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(std::make_tuple(p->dims, p->radius, p->pattern, (int)p->prec, size_class(p)));
        if (it != g_tune.end()) algo = it->second;
    }
    // The last sweep lands in `out`; earlier ones alternate so that sweep i
    // writes `out` when (sweeps - i) is even and `scratch` otherwise.
    const void *src = in;
    for (long long i = 1; i <= sweeps; ++i) {
        void *dst = ((sweeps - i) % 2 == 0) ? out : scratch;
        cudaError_t e;
        if (p->prec == CS_PREC_SPLIT && p->reanchor > 0 && (i % p->reanchor) == 0) {
            if (src == in) {
                // `in` stays untouched: its FP64 form goes to dst, the FP64
                // sweep into the third buffer, and back to (hi, lo) in dst.
                void *third = dst == out ? scratch : out;
                e = launch_split_to_fp64(p->layout.elements, (const float2 *)in, (double *)dst, st);
                if (e == cudaSuccess) {
                    e = fp64_anchor_sweep_fp64_in(p, dst, third, st);
                    if (e == cudaSuccess)
                        e = launch_split_from_fp64(p->layout.elements, (const double *)third, (float2 *)dst, st);
                }
            } else {
                e = fp64_anchor_sweep(p, const_cast<void *>(src), dst, st);
            }
        } else {
            e = launch_sweep(p, algo, src, dst, st);
        }
        if (e != cudaSuccess) return cuda_fail(e, "sweep launch");
        src = dst;
    }
    return CS_OK;
}

cs_status set_error(cs_status s, const char *msg) { return fail(s, "%s", msg); }

bool plan_facts(const cs_plan *p, PlanFacts *f)
{
    if (!p || !f) return false;
    f->dims = p->dims;
    f->radius = p->radius;
    f->pattern = p->pattern;
    f->steps_per_sweep = p->steps_per_sweep;
    f->prec = p->prec;
    f->view = p->view;
    f->origin = p->layout.origin;
    f->elements = p->layout.elements;
    f->reanchor = p->reanchor;
    f->algo = p->algo;
    f->w = &p->w;
    return true;
}

}  // namespace cs
