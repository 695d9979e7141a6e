// cs_serve.cu — a continuous-batching stencil server (C ABI in convstencil.h).
//
// Clients submit stencil solves (shape, grid, weights, steps, precision) from
// any thread; a worker thread owns the GPU work:
//   * admission: a request is admitted when its device buffers fit in the HBM
//     budget (a share of the memory free at creation) and a slot is free; it
//     then stays device-resident until its last step;
//   * execution: every scheduling turn issues one chunk of sweeps per active
//     request on that request's stream (a pool of streams), so the work of
//     different requests overlaps on the device; a chunk is captured once as a
//     CUDA graph and replayed. Small requests (a few ms of work or less) are
//     issued whole, chunk after chunk, on high-priority streams, so the
//     hardware runs their kernels ahead of the large requests' chunks;
//   * packing: small FP64 requests of one family (dims, radius, tap pattern,
//     steps per sweep; 2D radius 1-2 and 3D) admitted in the same turn run together as
//     one batch (cs_batch_*), one launch per sweep for all of them, each
//     grid leaving the batch after its own sweep count; the batch kernels do
//     each point's arithmetic as the request's own kernel would, and FP64
//     re-anchor sweeps fall at the same sweep counts, so a packed result is
//     the one the request gets alone;
//   * completion: the result goes to a pinned host buffer, the device memory is
//     released (making room for queued requests), the latency is recorded. A
//     request during whose life a bounded device-side wait expired (the
//     library's wait-timeout counters moved between its admission and its
//     completion) is reported as CS_ERR_TIMEOUT instead: its result may be
//     incomplete. The attribution is conservative: a request that overlapped
//     another's expiry is reported too.
// Kernel choice and FP64 re-anchoring points depend only on the request, never
// on what else is running, so a request's result is bitwise identical alone
// and in any mix.
#include "../../include/convstencil.h"
#include "cs_internal.h"
#include "cs_plan_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

namespace {

// Requests below this many tap-updates (about 4 ms of FP64 FMA work) are
// issued whole on a high-priority stream: their latency is then their own
// GPU time, not a scheduling turn per chunk behind the large requests.
constexpr double kSmallWork = 2e9;

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Pinned host buffers, reused by size class (powers of two).
class PinnedPool {
  public:
    ~PinnedPool()
    {
        for (auto &kv : free_)
            for (void *p : kv.second) cudaFreeHost(p);
    }
    void *get(size_t bytes, size_t *cls)
    {
        size_t c = 4096;
        while (c < bytes) c <<= 1;
        *cls = c;
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto &v = free_[c];
            if (!v.empty()) {
                void *p = v.back();
                v.pop_back();
                return p;
            }
        }
        void *p = nullptr;
        if (cudaHostAlloc(&p, c, cudaHostAllocDefault) != cudaSuccess) return nullptr;
        return p;
    }
    void put(void *p, size_t cls)
    {
        std::lock_guard<std::mutex> lk(mu_);
        free_[cls].push_back(p);
    }

  private:
    std::mutex mu_;
    std::map<size_t, std::vector<void *>> free_;
};

enum class State { Queued, Active, Draining, Done, Failed };
// `retired` is set (under the server lock) once the worker holds no more
// references to a request; only then may a waiter consume and delete it.

struct Request {
    long long id = 0;
    cs_plan *plan = nullptr;
    cs_precision prec = CS_PREC_FP64;
    cs_layout layout{};
    long long steps = 0, issued = 0, sweeps_per_step = 1;
    void *host = nullptr;  // pinned: packed input, later the packed FP64 result
    size_t host_cls = 0;
    void *d[2] = {nullptr, nullptr};
    void *stage = nullptr;  // FP64 staging for split conversions
    int cur = 0;            // buffer holding the current state
    size_t bytes = 0;       // device bytes reserved
    cudaStream_t stream = nullptr;
    cudaEvent_t chunk_ev = nullptr, done_ev = nullptr;
    bool chunk_pending = false;
    bool small = false;     // little work: issued whole, on a high-priority stream
    bool packable = false;  // small, on a kernel the batcher runs with the same arithmetic
    bool packed = false;    // ran in a batch with other requests of its family
    cudaGraphExec_t graph = nullptr;
    long long graph_steps = 0;
    int full_chunks = 0;
    double t_submit = 0, t_done = 0;
    unsigned waits_at_start = 0;  // wait-timeout count when admitted
    std::atomic<State> state{State::Queued};
    bool retired = false;
    cs_status status = CS_OK;
    std::string error;
};

}  // namespace

struct cs_server {
    cs_server_config cfg{};
    int device = 0;
    std::vector<cudaStream_t> streams;        // large requests (lowest priority)
    std::vector<cudaStream_t> fast_streams;   // small requests (highest priority)
    PinnedPool pinned;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::vector<Request *> active;
    std::map<long long, std::unique_ptr<Request>> all;
    long long next_id = 1;
    size_t budget = 0, reserved = 0;
    bool stop = false;
    std::thread worker;
    // statistics
    std::vector<double> latencies;
    long long completed = 0, failed = 0;
    double point_steps = 0, t_first = 0, t_last = 0;
    int rr = 0, rr_fast = 0;
    int sm_count = 1;
    long long packed = 0;  // requests that ran in shared batch launches
};

namespace {

void fail_request(cs_server *s, Request *r, cs_status st, const std::string &msg)
{
    r->status = st;
    r->error = msg;
    r->state = State::Failed;
    r->t_done = now_s();
    s->failed++;
}

// Device buffers come from the stream-ordered pool (cudaMallocAsync), so
// admitting and retiring requests never synchronises the device.
void release_device(Request *r)
{
    for (void *&p : r->d)
        if (p) cudaFreeAsync(p, r->stream), p = nullptr;
    if (r->stage) cudaFreeAsync(r->stage, r->stream), r->stage = nullptr;
    if (r->graph) cudaGraphExecDestroy(r->graph), r->graph = nullptr;
    if (r->chunk_ev) cudaEventDestroy(r->chunk_ev), r->chunk_ev = nullptr;
}

// Allocates and uploads an admitted request (worker thread).
bool start_request(cs_server *s, Request *r)
{
    const size_t b = r->layout.bytes;
    cs_device_wait_timeouts(&r->waits_at_start, 0);
    r->stream = r->small ? s->fast_streams[s->rr_fast++ % s->fast_streams.size()]
                         : s->streams[s->rr++ % s->streams.size()];
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaMallocAsync(&r->d[i], b, r->stream);
    if (e == cudaSuccess && r->prec == CS_PREC_SPLIT) e = cudaMallocAsync(&r->stage, b, r->stream);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->chunk_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->done_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        fail_request(s, r, e == cudaErrorMemoryAllocation ? CS_ERR_OUT_OF_MEMORY : CS_ERR_CUDA,
                     cudaGetErrorString(e));
        return false;
    }
    cudaMemsetAsync(r->d[1], 0, b, r->stream);
    if (r->prec == CS_PREC_FP64) {
        e = cudaMemcpyAsync(r->d[0], r->host, b, cudaMemcpyHostToDevice, r->stream);
    } else {
        e = cudaMemcpyAsync(r->stage, r->host, b, cudaMemcpyHostToDevice, r->stream);
        if (e == cudaSuccess && cs_split_from_fp64(r->plan, (const double *)r->stage, r->d[0], r->stream) != CS_OK)
            e = cudaErrorUnknown;
    }
    if (e != cudaSuccess) {
        fail_request(s, r, CS_ERR_CUDA, cudaGetErrorString(e));
        return false;
    }
    r->cur = 0;
    r->state = State::Active;
    return true;
}

// Issues `steps` steps of r on its stream. The sweeps are numbered from the
// request's start, so split grids take their FP64 re-anchor sweeps at the
// same global sweep counts however the run is chunked.
cs_status issue_steps(Request *r, long long steps)
{
    int in_b = 0;
    cs_status st = cs::run_from(r->plan, r->d[r->cur], r->d[r->cur ^ 1], r->issued / r->sweeps_per_step, steps,
                                r->stream, &in_b);
    if (st != CS_OK) return st;
    r->cur ^= in_b;
    return CS_OK;
}

// Result to the pinned host buffer; completion is seen through done_ev.
void finish_request(Request *r)
{
    const void *res = r->d[r->cur];
    if (r->prec == CS_PREC_SPLIT) {
        cs_split_to_fp64(r->plan, res, (double *)r->stage, r->stream);
        res = r->stage;
    }
    cudaMemcpyAsync(r->host, res, r->layout.bytes, cudaMemcpyDeviceToHost, r->stream);
    cudaEventRecord(r->done_ev, r->stream);
    r->state = State::Draining;
}

// One scheduling turn for an active request: the next chunk of steps (all of
// them for a small request).
void advance(cs_server *s, Request *r)
{
    if (r->chunk_pending) {
        if (cudaEventQuery(r->chunk_ev) == cudaErrorNotReady) return;  // at most one chunk in flight
        r->chunk_pending = false;
    }
    // Chunks are whole fused sweeps: a multiple of the plan's steps per sweep.
    const long long full = std::max(1LL, s->cfg.chunk_steps / r->sweeps_per_step) * r->sweeps_per_step;
    if (r->small) {
        // All chunks now, back to back on the request's high-priority stream:
        // the same kernels and re-anchoring points as chunk-by-chunk issue,
        // without a scheduling turn between chunks.
        while (r->issued < r->steps) {
            const long long chunk = std::min(full, r->steps - r->issued);
            const cs_status st = issue_steps(r, chunk);
            if (st != CS_OK) {
                fail_request(s, r, st, cs_last_error());
                return;
            }
            r->issued += chunk;
        }
        finish_request(r);
        return;
    }
    const long long chunk = std::min(full, r->steps - r->issued);
    cs_status st = CS_OK;
    const bool graphable = s->cfg.use_graphs && chunk == full &&
                           (chunk / r->sweeps_per_step) % 2 == 0 && r->prec == CS_PREC_FP64;
    if (graphable && r->graph && r->graph_steps == chunk) {
        st = cudaGraphLaunch(r->graph, r->stream) == cudaSuccess ? CS_OK : CS_ERR_CUDA;
    } else if (graphable && r->full_chunks >= 1) {
        // Capture one chunk (an even number of sweeps returns to the same
        // buffer, so the graph can be replayed as is).
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const int cur = r->cur;
            st = issue_steps(r, chunk);
            r->cur = cur;
            e = cudaStreamEndCapture(r->stream, &g);
        }
        if (e == cudaSuccess && st == CS_OK && cudaGraphInstantiate(&r->graph, g, 0) == cudaSuccess) {
            r->graph_steps = chunk;
            st = cudaGraphLaunch(r->graph, r->stream) == cudaSuccess ? CS_OK : CS_ERR_CUDA;
        } else if (st == CS_OK) {
            st = issue_steps(r, chunk);  // capture unavailable: plain launches
        }
        if (g) cudaGraphDestroy(g);
    } else {
        st = issue_steps(r, chunk);
    }
    if (st != CS_OK) {
        fail_request(s, r, st, cs_last_error());
        return;
    }
    if (chunk == full) r->full_chunks++;
    r->issued += chunk;
    if (r->issued >= r->steps) {
        finish_request(r);
    } else {
        cudaEventRecord(r->chunk_ev, r->stream);
        r->chunk_pending = true;
    }
}

// Runs a family of admitted small requests (two or more) as one batch on a
// high-priority stream: after their uploads, one launch per sweep for every
// member still running (members with fewer sweeps leave the batch), an FP64
// re-anchor sweep per split member wherever it would take one alone, and each
// member's result copied out right after its last sweep. Returns false (and
// leaves the members to the normal path) if the batch cannot be set up.
bool run_pack(cs_server *s, std::vector<Request *> &grp)
{
    const int n = (int)grp.size();
    cudaStream_t st = s->fast_streams[s->rr_fast++ % s->fast_streams.size()];
    std::vector<cs_plan *> plans(n);
    std::vector<void *> a(n), b(n);
    std::vector<long long> sweeps(n);
    long long most = 0;
    for (int i = 0; i < n; ++i) {
        Request *r = grp[i];
        // the member's upload (on its own stream) comes first
        if (cudaEventRecord(r->chunk_ev, r->stream) != cudaSuccess ||
            cudaStreamWaitEvent(st, r->chunk_ev, 0) != cudaSuccess)
            return false;
        plans[i] = r->plan;
        a[i] = r->d[0];
        b[i] = r->d[1];
        sweeps[i] = r->steps / r->sweeps_per_step;
        most = std::max(most, sweeps[i]);
    }
    cs_batch *bt = nullptr;
    if (cs::batch_create_ex(&bt, plans.data(), a.data(), b.data(), n, sweeps.data(), false, st) != CS_OK)
        return false;
    cs::PlanFacts f;
    cs::plan_facts(grp[0]->plan, &f);
    for (Request *r : grp) {
        r->stream = st;  // every later operation of the member is ordered on the batch's stream
        r->packed = true;
    }
    cs_status err = CS_OK;
    for (long long j = 0; j < most && err == CS_OK; ++j) {
        const bool anchor = f.prec == CS_PREC_SPLIT && f.reanchor > 0 && (j + 1) % f.reanchor == 0;
        if (anchor) {
            for (int i = 0; i < n && err == CS_OK; ++i)
                if (sweeps[i] > j && cs::fp64_anchor_sweep(grp[i]->plan, grp[i]->d[j & 1], grp[i]->d[(j & 1) ^ 1],
                                                          st) != cudaSuccess)
                    err = CS_ERR_CUDA;
        } else {
            err = cs::batch_sweep(bt, j, st);
        }
        for (int i = 0; i < n && err == CS_OK; ++i)
            if (sweeps[i] == j + 1) {
                grp[i]->cur = (int)((j + 1) & 1);
                grp[i]->issued = grp[i]->steps;
                finish_request(grp[i]);
            }
    }
    cs_batch_destroy(bt);  // tables freed in order on st
    for (Request *r : grp)
        if (r->state == State::Active) {
            std::lock_guard<std::mutex> lk(s->mu);
            fail_request(s, r, err == CS_OK ? CS_ERR_CUDA : err, "batched sweep launch failed");
        }
    std::lock_guard<std::mutex> lk(s->mu);
    s->packed += n;
    return true;
}

void worker_main(cs_server *s)
{
    cudaSetDevice(s->device);
    for (;;) {
        std::vector<Request *> admitted;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop && s->queue.empty() && s->active.empty()) return;
            if (s->queue.empty() && s->active.empty())
                s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
            while (!s->queue.empty() && (int)s->active.size() < s->cfg.max_active) {
                Request *r = s->queue.front();
                if (s->reserved + r->bytes > s->budget) {
                    if (s->active.empty()) {  // can never fit
                        s->queue.pop_front();
                        fail_request(s, r, CS_ERR_OUT_OF_MEMORY, "request exceeds the server's HBM budget");
                        r->retired = true;
                        s->cv_done.notify_all();
                        continue;
                    }
                    break;  // wait for memory
                }
                s->queue.pop_front();
                s->reserved += r->bytes;
                s->active.push_back(r);
                admitted.push_back(r);
            }
        }
        std::map<std::tuple<int, int, int, int, int>, std::vector<Request *>> families;
        for (Request *r : admitted) {
            if (!start_request(s, r)) {
                std::lock_guard<std::mutex> lk(s->mu);
                release_device(r);
                s->reserved -= r->bytes;
                s->active.erase(std::find(s->active.begin(), s->active.end(), r));
                r->retired = true;
                s->cv_done.notify_all();
            } else if (r->packable) {
                cs::PlanFacts f;
                cs::plan_facts(r->plan, &f);
                families[std::make_tuple(f.dims, f.radius, f.pattern, (int)f.prec, f.steps_per_sweep)].push_back(r);
            }
        }
        for (auto &kv : families)
            if (kv.second.size() >= 2) run_pack(s, kv.second);
        std::vector<Request *> act;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            act = s->active;
        }
        bool progressed = false;
        for (Request *r : act) {
            if (r->state == State::Active) {
                const long long before = r->issued;
                advance(s, r);
                progressed |= r->issued != before;
            }
            bool finished = r->state == State::Draining && cudaEventQuery(r->done_ev) == cudaSuccess;
            if (finished) {
                unsigned waits = 0;
                if (cs_device_wait_timeouts(&waits, 0) == CS_OK && waits != r->waits_at_start) {
                    std::lock_guard<std::mutex> lk(s->mu);
                    fail_request(s, r, CS_ERR_TIMEOUT,
                                 "a bounded device-side wait expired while this request ran; result incomplete");
                    finished = false;
                }
            }
            if (finished || r->state == State::Failed) {
                std::lock_guard<std::mutex> lk(s->mu);
                if (finished) {
                    r->t_done = now_s();
                    r->state = State::Done;
                    s->latencies.push_back(r->t_done - r->t_submit);
                    s->completed++;
                    double pts = 1;
                    for (int d = 0; d < r->layout.dims; ++d) pts *= (double)r->layout.extent[d];
                    s->point_steps += pts * (double)r->steps;
                    s->t_last = r->t_done;
                }
                release_device(r);
                s->reserved -= r->bytes;
                s->active.erase(std::find(s->active.begin(), s->active.end(), r));
                r->retired = true;
                s->cv_done.notify_all();
                progressed = true;
            }
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

// Packs a dense interior (row-major) into the plan's layout, zero halo.
void pack(const cs_layout &L, const double *interior, double *buf)
{
    memset(buf, 0, L.bytes);
    const long long nx = L.extent[L.dims - 1];
    const long long rows = L.dims == 1 ? 1 : L.dims == 2 ? L.extent[0] : L.extent[0] * L.extent[1];
    for (long long r = 0; r < rows; ++r) {
        long long off = L.origin;
        if (L.dims == 2) off += r * L.pitch[0];
        if (L.dims == 3) off += (r / L.extent[1]) * L.pitch[0] + (r % L.extent[1]) * L.pitch[1];
        memcpy(buf + off, interior + r * nx, nx * sizeof(double));
    }
}

void unpack(const cs_layout &L, const double *buf, double *interior)
{
    const long long nx = L.extent[L.dims - 1];
    const long long rows = L.dims == 1 ? 1 : L.dims == 2 ? L.extent[0] : L.extent[0] * L.extent[1];
    for (long long r = 0; r < rows; ++r) {
        long long off = L.origin;
        if (L.dims == 2) off += r * L.pitch[0];
        if (L.dims == 3) off += (r / L.extent[1]) * L.pitch[0] + (r % L.extent[1]) * L.pitch[1];
        memcpy(interior + r * nx, buf + off, nx * sizeof(double));
    }
}

}  // namespace

extern "C" {

CS_API cs_status cs_server_create(cs_server **out, const cs_server_config *cfg)
{
    if (!out) return CS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cs_server_config c{8, 64, 0.8, 32, 1};
    if (cfg) c = *cfg;
    if (c.streams < 1 || c.streams > 128 || c.max_active < 1 || c.hbm_fraction <= 0 || c.hbm_fraction > 1 ||
        c.chunk_steps < 1)
        return CS_ERR_INVALID_ARGUMENT;
    auto s = std::make_unique<cs_server>();
    s->cfg = c;
    if (cudaGetDevice(&s->device) != cudaSuccess) return CS_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
    if (s->sm_count < 1) s->sm_count = 1;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return CS_ERR_CUDA;
    s->budget = (size_t)(c.hbm_fraction * (double)free_b);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
        unsigned long long keep = s->budget;  // keep freed blocks for the next admissions
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = greatest = 0;
    for (int i = 0; i < c.streams; ++i) {
        cudaStream_t st, fast;
        if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, least) != cudaSuccess) return CS_ERR_CUDA;
        s->streams.push_back(st);
        if (cudaStreamCreateWithPriority(&fast, cudaStreamNonBlocking, greatest) != cudaSuccess)
            return CS_ERR_CUDA;
        s->fast_streams.push_back(fast);
    }
    s->worker = std::thread(worker_main, s.get());
    *out = s.release();
    return CS_OK;
}

}  // extern "C"

namespace {

// Everything a request needs before it is queued: plan, kernel choice,
// packed host copy of its input (no server lock held).
cs_status prepare_request(cs_server *s, const cs_request_desc *d, std::unique_ptr<Request> &out)
{
    if (!d || !d->interior_in || !d->weights || d->steps < 0) return CS_ERR_INVALID_ARGUMENT;
    auto r = std::make_unique<Request>();
    cs_status st = cs_plan_create(&r->plan, d->shape, d->semantics, d->precision, d->extent, d->weights,
                                  d->n_weights, nullptr);
    if (st != CS_OK) return st;
    // A fixed kernel choice keeps results identical in any mix and keeps the
    // plan tuner (which times candidates synchronously) off the worker
    // thread: the FP64 FMA kernels; for split precision the tcgen05 slice
    // kernel where it applies (it falls back by itself on buffers it cannot
    // use), else the double-float kernels with a fixed temporal block (their
    // results do not depend on it).
    if (d->precision == CS_PREC_SPLIT) {
        int algo;
        if (d->shape == CS_SHAPE_STAR3D1R || d->shape == CS_SHAPE_BOX3D1R) {
            // 3D: the 27-point box on tcgen05 from about 128^3 points up
            // (measured crossover), else the double-float kernels (the
            // 7-point star always: its own kernel is faster).
            const double pts = (double)d->extent[0] * (double)d->extent[1] * (double)d->extent[2];
            algo = d->shape == CS_SHAPE_BOX3D1R && d->semantics == CS_SEM_STEP && pts >= 2.0e6
                       ? CS_ALGO_SPLIT_TC
                       : CS_ALGO_SPLIT_FMA;
        } else {
            // tcgen05 pays a fixed ~16 us per sweep (one 64 x 64 tile per CTA
            // and SM, set-up of its weight matrices and TMEM); below about four
            // tiles per SM the mma.sync slice kernel (~8 us floor) finishes sooner.
            const long long tiles = ((d->extent[0] + 63) / 64) * ((d->extent[1] + 63) / 64);
            algo = tiles >= 4LL * s->sm_count ? CS_ALGO_SPLIT_TC : CS_ALGO_SPLIT_MMA;
        }
        if (cs_plan_set_option(r->plan, CS_OPT_ALGO, algo) != CS_OK)
            cs_plan_set_option(r->plan, CS_OPT_ALGO, CS_ALGO_SPLIT_FMA);
        const int tb = (d->shape == CS_SHAPE_1D1R || d->shape == CS_SHAPE_1D2R) ? 4
                       : d->shape == CS_SHAPE_STAR2D1R                           ? 3
                                                                                 : 2;
        cs_plan_set_option(r->plan, CS_OPT_TIME_BLOCK, tb);
    } else {
        // FP64: 7x7 kernels of at least four 64 x 64 tiles per SM on the
        // tcgen05 digit pipeline (same cost model as the split slices), the
        // FP64 FMA kernels otherwise.
        const long long tiles = ((d->extent[0] + 63) / 64) * ((d->extent[1] + 63) / 64);
        const bool r3_2d = (d->shape == CS_SHAPE_BOX2D3R || d->shape == CS_SHAPE_STAR2D3R ||
                            (d->semantics == CS_SEM_FUSED &&
                             (d->shape == CS_SHAPE_BOX2D1R || d->shape == CS_SHAPE_STAR2D1R)));
        if (!(r3_2d && tiles >= 4LL * s->sm_count &&
              cs_plan_set_option(r->plan, CS_OPT_ALGO, CS_ALGO_FP64_TC) == CS_OK))
            cs_plan_set_option(r->plan, CS_OPT_ALGO, CS_ALGO_FP64_FMA);
    }
    // The FP64 FMA 2D kernel's tile rows: fixed here (the plan tuner would
    // time both on the worker thread); results do not depend on them.
    if (d->precision == CS_PREC_FP64 && (d->shape >= CS_SHAPE_STAR2D1R && d->shape <= CS_SHAPE_BOX2D3R)) {
        const long long t32 = ((d->extent[1] + 63) / 64) * ((d->extent[0] + 31) / 32);
        cs_plan_set_option(r->plan, CS_OPT_TILE_ROWS, t32 < 6LL * s->sm_count ? 16 : 32);
    }
    long long sweeps1 = 0;
    if (d->semantics == CS_SEM_FUSED) {
        for (long long k = 1; k <= 3; ++k)
            if (cs_plan_sweeps(r->plan, k, &sweeps1) == CS_OK && sweeps1 == 1) {
                r->sweeps_per_step = k;
                break;
            }
    }
    if (cs_plan_sweeps(r->plan, d->steps, &sweeps1) != CS_OK) {
        cs_plan_destroy(r->plan);
        return CS_ERR_INVALID_ARGUMENT;
    }
    cs_plan_get_layout(r->plan, &r->layout);
    r->prec = d->precision;
    r->steps = d->steps;
    {
        // Work estimate: point-sweeps times the stencil window, split precision
        // counted at an eighth (its kernels run ~10x the FP64 rate).
        double pts = 1, taps = 1;
        for (int k = 0; k < r->layout.dims; ++k) {
            pts *= (double)r->layout.extent[k];
            taps *= 2.0 * r->layout.halo + 1.0;
        }
        const double work = pts * (double)sweeps1 * taps / (d->precision == CS_PREC_SPLIT ? 8.0 : 1.0);
        r->small = work < kSmallWork;
    }
    {
        // Packable: small FP64 requests, 2D (not radius 3: those run tcgen05
        // alone from four tiles per SM) or 3D, on the FP64 FMA kernels whose
        // per-point arithmetic and form the batch kernels repeat. Split
        // requests stay alone: their own kernels (temporal blocking in 2D, the
        // z-queue star and packed-pair box in 3D) beat the batch's generic
        // double-float form (measured, 48 saturated split requests: 104
        // GStencil/s alone, 85 with all small split requests packed, 90 with
        // the 3D ones packed; FP64 31.3 alone, 31.0 packed).
        cs::PlanFacts f;
        cs::plan_facts(r->plan, &f);
        r->packable = r->small && d->precision == CS_PREC_FP64 && f.algo == CS_ALGO_FP64_FMA &&
                      ((f.dims == 2 && f.radius != 3) || (f.dims == 3 && (f.radius == 1 || f.radius == 3)));
    }
    r->bytes = r->layout.bytes * (d->precision == CS_PREC_SPLIT ? 3 : 2);
    r->host = s->pinned.get(r->layout.bytes, &r->host_cls);
    if (!r->host) {
        cs_plan_destroy(r->plan);
        return CS_ERR_OUT_OF_MEMORY;
    }
    pack(r->layout, d->interior_in, (double *)r->host);
    out = std::move(r);
    return CS_OK;
}

// Queues a prepared request (server lock held).
long long enqueue(cs_server *s, std::unique_ptr<Request> r)
{
    r->id = s->next_id++;
    r->t_submit = now_s();
    if (s->t_first == 0) s->t_first = r->t_submit;
    const long long id = r->id;
    Request *raw = r.get();
    s->all[id] = std::move(r);
    if (raw->steps == 0) {  // nothing to run: the result is the input
        raw->state = State::Done;
        raw->retired = true;
        raw->t_done = raw->t_submit;
        s->completed++;
        s->latencies.push_back(0.0);
        s->cv_done.notify_all();
    } else {
        s->queue.push_back(raw);
    }
    return id;
}

void discard(cs_server *s, std::unique_ptr<Request> &r)
{
    if (!r) return;
    if (r->host) s->pinned.put(r->host, r->host_cls);
    cs_plan_destroy(r->plan);
    r.reset();
}

}  // namespace

extern "C" {

CS_API cs_status cs_server_submit(cs_server *s, const cs_request_desc *d, long long *id)
{
    if (!s || !id) return CS_ERR_INVALID_ARGUMENT;
    std::unique_ptr<Request> r;
    const cs_status st = prepare_request(s, d, r);
    if (st != CS_OK) return st;
    std::lock_guard<std::mutex> lk(s->mu);
    *id = enqueue(s, std::move(r));
    s->cv_work.notify_one();
    return CS_OK;
}

CS_API cs_status cs_server_submit_many(cs_server *s, const cs_request_desc *reqs, int count, long long *ids)
{
    if (!s || !reqs || !ids || count < 1) return CS_ERR_INVALID_ARGUMENT;
    std::vector<std::unique_ptr<Request>> rs(count);
    for (int i = 0; i < count; ++i) {
        const cs_status st = prepare_request(s, &reqs[i], rs[i]);
        if (st != CS_OK) {
            for (auto &r : rs) discard(s, r);
            return st;
        }
    }
    std::lock_guard<std::mutex> lk(s->mu);  // one lock: the worker sees all of them at once
    for (int i = 0; i < count; ++i) ids[i] = enqueue(s, std::move(rs[i]));
    s->cv_work.notify_one();
    return CS_OK;
}

CS_API cs_status cs_server_wait(cs_server *s, long long id, double *interior_out, double timeout_seconds,
                                double *latency_seconds)
{
    if (!s) return CS_ERR_INVALID_ARGUMENT;
    Request *r = nullptr;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return CS_ERR_INVALID_ARGUMENT;
    r = it->second.get();
    const auto deadline = std::chrono::steady_clock::now() +
                          std::chrono::duration<double>(timeout_seconds > 0 ? timeout_seconds : 1e9);
    while (!r->retired) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !r->retired)
            return CS_ERR_TIMEOUT;
    }
    cs_status st = r->status;
    if (r->state == State::Done && interior_out) unpack(r->layout, (const double *)r->host, interior_out);
    if (latency_seconds) *latency_seconds = r->t_done - r->t_submit;
    if (r->done_ev) cudaEventDestroy(r->done_ev);
    s->pinned.put(r->host, r->host_cls);
    cs_plan_destroy(r->plan);
    s->all.erase(it);
    return st;
}

CS_API cs_status cs_server_get_stats(cs_server *s, cs_server_stats *out)
{
    if (!s || !out) return CS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof *out);
    out->completed = s->completed;
    out->failed = s->failed;
    out->queued = (long long)s->queue.size();
    out->active = (long long)s->active.size();
    out->hbm_budget_bytes = (long long)s->budget;
    out->hbm_reserved_bytes = (long long)s->reserved;
    std::vector<double> v = s->latencies;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) { return v[std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5))]; };
        out->p50_s = pct(0.50);
        out->p99_s = pct(0.99);
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_s = sum / (double)v.size();
    }
    out->point_steps = s->point_steps;
    out->wall_s = s->t_last > s->t_first ? s->t_last - s->t_first : 0.0;
    out->gstencil_s = out->wall_s > 0 ? s->point_steps / out->wall_s / 1e9 : 0.0;
    out->packed = s->packed;
    return CS_OK;
}

CS_API cs_status cs_server_destroy(cs_server *s)
{
    if (!s) return CS_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    for (auto &kv : s->all) {
        Request *r = kv.second.get();
        release_device(r);
        if (r->done_ev) cudaEventDestroy(r->done_ev);
        if (r->host) s->pinned.put(r->host, r->host_cls);
        cs_plan_destroy(r->plan);
    }
    for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
    for (cudaStream_t st : s->fast_streams) cudaStreamDestroy(st);
    delete s;
    return CS_OK;
}

}  // extern "C"
