/*
 * convstencil.h — C ABI of the GB300-native ConvStencil library
 * (libconvstencil_gb300.so).
 *
 * Two surfaces:
 *
 * 1. Reference-shaped wrappers, one per host wrapper of microsoft/ConvStencil.
 *    Same arguments, layouts and meaning; a status code instead of exit()/abort().
 *    Host buffers in and out, device memory allocated and released inside the
 *    call (the reference leaks it), timing lines printed to stdout only when
 *    `cs_set_verbose(1)` (the C++-linkage drop-in symbols in
 *    convstencil_ref.h always print, as the reference does).
 *
 * 2. Plans over caller-owned DEVICE buffers: reentrant (no global state, no
 *    __constant__ symbols; weights travel in kernel parameters), explicit
 *    CUDA stream, any layout with a zero halo, FP64 or split precision.
 *
 * All functions return CS_OK or an error code; cs_last_error() gives a
 * per-thread message for the last failure. Nothing here exits or aborts.
 */
#ifndef CONVSTENCIL_H
#define CONVSTENCIL_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CS_API __attribute__((visibility("default")))

typedef enum cs_status {
    CS_OK = 0,
    CS_ERR_INVALID_ARGUMENT = 1, /* bad shape, size, pointer, weight count */
    CS_ERR_UNSUPPORTED = 2,      /* valid request this build does not serve */
    CS_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    CS_ERR_OUT_OF_MEMORY = 4,    /* device or host allocation failed */
    CS_ERR_TIMEOUT = 5,          /* a bounded device-side wait expired */
    CS_ERR_NO_DEVICE = 6         /* no usable CUDA device */
} cs_status;

/* The eight stencil shapes of the reference CLIs (src/1d/main.cu:69-79,
 * src/2d/main.cu:138-160, src/3d/main.cu:489-500). */
typedef enum cs_shape {
    CS_SHAPE_1D1R = 0,     /* 3-point, radius 1 */
    CS_SHAPE_1D2R = 1,     /* 5-point, radius 2 */
    CS_SHAPE_STAR2D1R = 2, /* 5-point cross, radius 1 */
    CS_SHAPE_BOX2D1R = 3,  /* 3x3 box */
    CS_SHAPE_STAR2D3R = 4, /* 13-point cross, radius 3 */
    CS_SHAPE_BOX2D3R = 5,  /* 7x7 box */
    CS_SHAPE_STAR3D1R = 6, /* 7-point cross, radius 1 */
    CS_SHAPE_BOX3D1R = 7   /* 3x3x3 box */
} cs_shape;

/* What one "sweep" means.
 * CS_SEM_STEP : weights are the base stencil's (3, 5, 5, 9, 13, 49, 7, 27
 *               values, row-major over the cells of the shape); a step is
 *               one sweep of that stencil with a zero halo of its radius.
 * CS_SEM_FUSED: weights are the reference wrappers' fused parameters
 *               (7, 9, 49, 49, 49, 49, 44, 196 values); a sweep applies the
 *               fused kernel once with a zero halo of the fused radius, and
 *               counts as 3 steps (1d1r, 2d1r shapes, 3D shapes), 2 (1d2r)
 *               or 1 (2d3r shapes), as the reference counts it
 *               (src/2d/gpu.cu:329, src/1d/gpu_2r.cu:154, src/3d/gpu_box.cu:531). */
typedef enum cs_semantics { CS_SEM_STEP = 0, CS_SEM_FUSED = 1 } cs_semantics;

/* Arithmetic of the sweep.
 * CS_PREC_FP64 : FP64 grids. FP64 FMA or FP64 MMA arithmetic, or, for 2D
 *                kernels up to 7x7 and 3D radius-1 kernels, the FP64-accurate
 *                tensor-core form (CS_ALGO_FP64_TC) when the tuner measures
 *                it faster: every
 *                product and level sum is exact, inputs keep 52 bits below
 *                their 64x70 tile's largest value and weights 53 below the
 *                largest weight (relative error per sweep ~1e-16 of the
 *                tile's scale). Pin CS_ALGO_FP64_FMA for IEEE FP64 sums.
 * CS_PREC_SPLIT: grids stored as FP32 (hi, lo) pairs (8 bytes per point,
 *                about 48 significant bits); no FP64 arithmetic in the sweep.
 *                Dense 7x7 kernels contract exact 9-bit fixed-point slices
 *                on FP16 tensor cores (FP32 accumulation is exact for them);
 *                other kernels use double-float FP32 arithmetic. Relative
 *                error per sweep ~1e-13. Inputs must be finite. */
typedef enum cs_precision { CS_PREC_FP64 = 0, CS_PREC_SPLIT = 1 } cs_precision;

/* Kernel family; CS_ALGO_AUTO lets the plan's tuner choose. */
typedef enum cs_algo {
    CS_ALGO_AUTO = 0,
    CS_ALGO_FP64_FMA = 1,  /* FP64 FMA, one FMA per non-zero tap (fewest FP64 ops) */
    CS_ALGO_FP64_MMA = 2,  /* FP64 tensor-core MMA (mma.sync m8n8k4.f64), 2x4 output blocks;
                              2D dense radius-3 kernels */
    CS_ALGO_SPLIT_MMA = 3, /* split precision: five exact 9-bit fixed-point slices per operand on
                              FP16 tensor cores (mma.sync m16n8k16), one exact FP32
                              accumulator per slice level; 2D dense radius-3 kernels */
    CS_ALGO_SPLIT_FMA = 4, /* split precision: double-float arithmetic on FP32 cores */
    CS_ALGO_SPLIT_MMA_TMA = 5, /* as CS_ALGO_SPLIT_MMA, tiles fetched by TMA (cp.async.bulk.tensor)
                                  one tile ahead */
    CS_ALGO_SPLIT_TC = 6, /* the same slices on fifth-generation tensor cores (tcgen05.mma,
                             accumulators in tensor memory), TMA-fed; 2D dense radius-3 kernels
                             on buffers with an even pitch, >= 4 halo columns, 16-byte aligned;
                             also 3D dense radius-1 split plans */
    CS_ALGO_FP64_TC = 7   /* FP64 plans on the same tcgen05 pipeline: six exact 9-bit digits per
                             operand cut from the FP64 bits by integer operations, exact FP32
                             level sums, integer recombination to FP64 (no FP64 instruction in
                             the sweep); 2D FP64 plans of radius up to 3 (the weights at the
                             centre of the 7x7) of at least 8x8, even pitch and interior column,
                             16-byte aligned buffers; also 3D radius-1 FP64
                             plans, box and star (an output's three plane parts are added as exact
                             integers when their plane exponents agree, in FP64 otherwise), and 1D
                             FP64 plans of radius up to 3 whose length is a multiple of 64 (at
                             least 512) with 4 halo points either side (as rows of 64 outputs) */
} cs_algo;

typedef enum cs_option {
    CS_OPT_ALGO = 0,              /* cs_algo */
    CS_OPT_REANCHOR_INTERVAL = 2, /* split: every N-th sweep is an FP64 re-anchor sweep,
                                     computed in FP64 arithmetic from the (hi, lo) state
                                     (converted in place, no allocation; the tcgen05 FP64
                                     pipeline for 2D radius-3 plans, FP64 FMA otherwise);
                                     sweeps are counted from the start of the run
                                     (default 100, 0 = never) */
    CS_OPT_TIME_BLOCK = 3,        /* split double-float kernels, 2D radius 1 and 1D:
                                     steps fused per launch by temporal blocking
                                     (0 = tuner picks 1..4, default; 1 = off) */
    CS_OPT_TILE_ROWS = 6,         /* FP64 FMA 2D kernel: rows per CTA tile, 16 or 32 (0 = tuner,
                                     default: the first run times both; results do not depend on it) */
    CS_OPT_WAIT_LIMIT_US = 4,     /* bound of each device-side wait of the tcgen05 kernels, in
                                     microseconds (default 2,000,000; 1 .. 60,000,000) */
    CS_OPT_WAIT_TEST_SKIP_LOADS = 5 /* test hook (0/1): the tcgen05 kernels issue no TMA loads,
                                     so their first wait runs out after CS_OPT_WAIT_LIMIT_US and
                                     the synchronous runs return CS_ERR_TIMEOUT; exercises the
                                     timeout path without faulting the GPU. Outputs of such runs
                                     are incomplete. */
} cs_option;

/* Where a grid lives in a buffer. extent/pitch are slowest axis first; the
 * last axis is contiguous (pitch 1). `origin` is the element offset of
 * interior point (0,...,0). Every interior point must have `halo` cells of
 * zeros (or of the caller's fixed boundary values) around it in memory. */
typedef struct cs_layout {
    int dims;
    int halo;
    long long extent[3];
    long long pitch[3];
    long long origin;
    long long elements; /* elements per buffer */
    size_t bytes;       /* bytes per buffer */
} cs_layout;

typedef struct cs_plan cs_plan;

/* ---- plans over device buffers --------------------------------------- */

/* extent: `dims` interior sizes, slowest first. weights: see cs_semantics.
 * layout: NULL for the library's native layout (rows padded to 16 bytes,
 * halo = the sweep's radius; 1D: at least 4 points before the interior and
 * 60 after it), or the caller's own layout. */
CS_API cs_status cs_plan_create(cs_plan **plan, cs_shape shape, cs_semantics sem,
                                cs_precision prec, const long long *extent,
                                const double *weights, int n_weights,
                                const cs_layout *layout);
CS_API cs_status cs_plan_set_option(cs_plan *plan, cs_option opt, long long value);
CS_API cs_status cs_plan_get_layout(const cs_plan *plan, cs_layout *out);
/* Sweep count and steps per sweep for `steps` steps (FUSED: steps must be a
 * multiple of the fused step count). */
CS_API cs_status cs_plan_sweeps(const cs_plan *plan, long long steps, long long *sweeps);
/* The cs_algo the plan's last cs_run used (its tuner's choice under
 * CS_ALGO_AUTO); CS_ALGO_AUTO before the first run. */
CS_API cs_status cs_plan_get_algo(const cs_plan *plan, int *algo);
/* Steps per launch the plan's last cs_run used (temporal blocking; 1 = off). */
CS_API cs_status cs_plan_get_time_block(const cs_plan *plan, int *steps_per_launch);
/* Rows per CTA tile of the FP64 FMA 2D kernel in the plan's last cs_run
 * (the tuner's choice under 0; 0 when another kernel ran). */
CS_API cs_status cs_plan_get_tile_rows(const cs_plan *plan, int *rows);
CS_API cs_status cs_plan_destroy(cs_plan *plan);

/* Runs `steps` steps from buffer a, ping-ponging with b (both per the plan's
 * layout, halos zero, both device pointers). *result_in_b is set to 1 when
 * the final grid is in b. Asynchronous on `stream` (a cudaStream_t; NULL =
 * legacy default stream). */
CS_API cs_status cs_run(cs_plan *plan, void *a, void *b, long long steps, void *stream,
                        int *result_in_b);

/* Runs `steps` steps from device buffer `in` into device buffer `out` (plan
 * layout, zero halos) and allocates nothing: the intermediate grid of the
 * ping-pong is a fixed 16 MiB array that this library reserves on every GPU
 * that loads it, for the life of the process. `in` is left unchanged.
 * No counterpart in the reference, whose wrappers always cudaMalloc.
 * For callers that must not allocate device memory at this point: a host
 * process whose framework allocator already holds the GPU's memory (a fresh
 * cudaMalloc would fail or fragment it), or a latency-critical loop that
 * cannot afford cudaMalloc's implicit device synchronisation.
 * Limits: one buffer of the plan's layout must fit in 16 MiB (2,097,152
 * points of 8 bytes); larger grids get CS_ERR_INVALID_ARGUMENT. The first
 * call on each device looks up the array's device address (with that device
 * current; again after the device's context changes, e.g. after
 * cudaDeviceReset); make that first call before any stream capture. Every
 * call shares the one array per device: calls whose work overlaps on the GPU
 * (different streams, or threads) race on it and must be serialised by the
 * caller. With CS_ALGO_AUTO it uses the kernel the tuner already chose for
 * this kind of plan (else the default), and runs no tuning sweeps of its own.
 * It launches one kernel per sweep, without cs_run's temporal blocking or
 * CUDA-graph replay, so small grids run slower than through cs_run. */
CS_API cs_status cs_run_noalloc(cs_plan *plan, const void *in, void *out, long long steps,
                                void *stream);

/* Split precision: FP64 grid <-> (hi, lo) FP32 pairs, same layout. */
CS_API cs_status cs_split_from_fp64(const cs_plan *plan, const double *src, void *dst, void *stream);
CS_API cs_status cs_split_to_fp64(const cs_plan *plan, const void *src, double *dst, void *stream);

/* Host-buffer form of cs_run: copies host_in (FP64, plan layout) into a
 * device grid (converted to (hi, lo) in place for split plans), runs, copies
 * the result (FP64) to host_out. Synchronous. When the kernel is known
 * without a timing run (pinned, or tuned earlier for this kind of plan), the
 * grid has at least two bands (256 rows for split 7x7 plans on the tensor
 * cores, else 1024 rows in 2D or 64 planes in 3D), and no temporal blocking
 * or re-anchor sweep is involved, the copies overlap the sweeps: the grid
 * moves in bands, the sweeps run as a wavefront over the bands already there,
 * and each band returns after its last sweep (results bitwise those of
 * whole-grid sweeps). The two device grids are
 * allocated by the plan's first call and kept for its later calls until
 * cs_plan_destroy (a call that finds them in use by another thread allocates
 * and frees its own). Returns CS_ERR_TIMEOUT (result incomplete) if a
 * bounded device-side wait expired during the call. */
CS_API cs_status cs_run_host(cs_plan *plan, const double *host_in, double *host_out,
                             long long steps);

/* ---- reference-shaped wrappers (FUSED semantics, reference layouts) ---- */
/* Each returns CS_ERR_TIMEOUT (result incomplete) if a bounded device-side
 * wait expired during the call; the reference exits on any CUDA error
 * (src/2d/2d_utils.h:35-65). Unlike the reference, which allocates and frees
 * its device arrays on every call, the wrappers keep the plan of their latest
 * call and its two device grids for the next call with the same shape, sizes
 * and params (a time loop then skips the set-up and the allocation); a call
 * with other arguments replaces it and cs_release_cached_plan() frees it. */
/* Replaces gpu_1d1r (src/1d/1d_utils.h:75, src/1d/gpu_1r.cu:227-302).
 * in: n+7 doubles (index 0 alignment pad, halo 3); out: n+6 doubles, the
 * device array from index 1 (src/1d/gpu_1r.cu:299). params: 7. */
CS_API cs_status cs_gpu_1d1r(const double *in, double *out, const double *params,
                             int times, int input_n);
/* Replaces gpu_star_1d2r_step2 (src/1d/1d_utils.h:85, src/1d/gpu_2r.cu:85-159).
 * in: n+8 doubles (halo 4); out: n+7 doubles (src/1d/gpu_2r.cu:156). params: 9. */
CS_API cs_status cs_gpu_star_1d2r_step2(const double *in, double *out, const double *params,
                                        int times, int input_n);
/* Replaces gpu_box_2d1r (src/2d/2d_utils.h:77, src/2d/gpu.cu:245-334).
 * in/out: (m+6) x (n+8) doubles; params: 49; counts 3 steps per sweep. */
CS_API cs_status cs_gpu_box_2d1r(const double *in, double *out, const double *params,
                                 int times, int input_m, int input_n);
/* Replaces gpu_box_2d3r (src/2d/2d_utils.h:79, src/2d/gpu.cu:336-425). */
CS_API cs_status cs_gpu_box_2d3r(const double *in, double *out, const double *params,
                                 int times, int input_m, int input_n);
/* Replaces gpu_box_3d1r (src/3d/3d_utils.h:75, src/3d/gpu_box.cu:446-536).
 * in/out: (h+6) x (m+6) x (n+6); params: 196 (4 planes, plane p <-> |dz|=3-p). */
CS_API cs_status cs_gpu_box_3d1r(const double *in, double *out, const double *params,
                                 int times, int input_h, int input_m, int input_n);
/* Replaces gpu_star_3d1r (src/3d/3d_utils.h:85, src/3d/gpu_star.cu:238-332).
 * params: 44 (octahedron cells by plane, src/3d/gpu_star.cu:30-56). */
CS_API cs_status cs_gpu_star_3d1r(const double *in, double *out, const double *params,
                                  int times, int input_h, int input_m, int input_n);

/* ---- batches: uneven 2D grids in one persistent launch per sweep ------- */
/* Plans of one batch share dims (2), radius, tap pattern, precision and
 * steps per sweep; sizes, weights and layouts may differ. Every grid of the
 * batch advances by the same number of steps; one launch per sweep covers
 * the tiles of all grids. Per grid the arithmetic is that of the FP64 FMA or
 * the split double-float kernel, so results equal a cs_run with that kernel
 * bitwise. On a non-default stream, an even number of sweeps is captured
 * into a CUDA graph on first use and replayed afterwards. Not in the
 * reference. */
typedef struct cs_batch cs_batch;
CS_API cs_status cs_batch_create(cs_batch **batch, cs_plan *const *plans, void *const *a,
                                 void *const *b, int count);
/* *result_in_b: 1 when every grid's state is now in its b buffer. */
CS_API cs_status cs_batch_run(cs_batch *batch, long long steps, void *stream, int *result_in_b);
CS_API cs_status cs_batch_destroy(cs_batch *batch);

/* ---- serving: continuous batching of stencil solves --------------------- */
/* A worker thread admits requests while their device buffers fit in the HBM
 * budget and a slot is free, keeps their grids device-resident, and issues
 * one chunk of sweeps per active request per turn on a pool of streams (the
 * work of different requests overlaps on the GPU; full chunks are replayed as
 * captured CUDA graphs). Small FP64 requests of one family (2D radius 1-2
 * or 3D, same radius and tap pattern) admitted in the same turn share batch
 * launches. Kernel choice and re-anchoring depend only on the
 * request, so a result is bitwise the same alone and in any mix. Not in the
 * reference (its CLIs run one solve per process). */
typedef struct cs_server cs_server;
typedef struct cs_server_config {
    int streams;           /* CUDA streams shared by the active requests (default 8) */
    int max_active;        /* requests resident on the GPU at once (default 64) */
    double hbm_fraction;   /* share of the device memory free at creation the server may use (0.8) */
    long long chunk_steps; /* steps issued per request per scheduling turn (default 32) */
    int use_graphs;        /* replay full FP64 chunks as captured CUDA graphs (default 1) */
} cs_server_config;
typedef struct cs_request_desc {
    cs_shape shape;
    cs_semantics semantics;
    cs_precision precision;
    long long extent[3];       /* interior sizes, slowest first */
    const double *weights;
    int n_weights;
    const double *interior_in; /* dense row-major interior, FP64 (halo is zero) */
    long long steps;
} cs_request_desc;
typedef struct cs_server_stats {
    long long completed, failed, queued, active;
    long long hbm_budget_bytes, hbm_reserved_bytes;
    double p50_s, p99_s, mean_s; /* submit -> result on the host */
    double point_steps;          /* interior points x steps of completed requests */
    double wall_s;               /* first submit -> last completion */
    double gstencil_s;           /* point_steps / wall_s / 1e9 */
    long long packed;            /* requests that ran in shared batch launches */
} cs_server_stats;

/* cfg NULL = defaults. Uses the calling thread's current device. */
CS_API cs_status cs_server_create(cs_server **server, const cs_server_config *cfg);
/* Copies the input; returns at once with the request id. */
CS_API cs_status cs_server_submit(cs_server *server, const cs_request_desc *req, long long *id);
/* Submits `count` requests at once (ids[i] for reqs[i]); the worker sees them
 * together, so small requests of one family among them are admitted in the
 * same turn and run as one batch (one launch per sweep for all of them).
 * On an invalid request nothing is submitted. */
CS_API cs_status cs_server_submit_many(cs_server *server, const cs_request_desc *reqs, int count,
                                       long long *ids);
/* Waits (timeout_seconds <= 0: no limit) and copies the dense interior result
 * to interior_out (may be NULL). Returns the request's status (e.g.
 * CS_ERR_OUT_OF_MEMORY if it can never fit the budget), CS_ERR_TIMEOUT if not
 * finished in time. Each id is waited for once. */
CS_API cs_status cs_server_wait(cs_server *server, long long id, double *interior_out,
                                double timeout_seconds, double *latency_seconds);
CS_API cs_status cs_server_get_stats(cs_server *server, cs_server_stats *out);
/* Finishes the admitted and queued work, then releases everything. */
CS_API cs_status cs_server_destroy(cs_server *server);

/* ---- utilities --------------------------------------------------------- */
CS_API const char *cs_status_string(cs_status s);
CS_API const char *cs_last_error(void);
CS_API void cs_set_verbose(int on);
/* Seconds of GPU time of the last timed loop run by a reference-shaped
 * wrapper on this thread (CUDA events around the launch loop). */
CS_API double cs_last_loop_seconds(void);
/* Frees the plan and device grids the reference-shaped wrappers keep from
 * their latest call (no counterpart in the reference, whose wrappers keep
 * nothing). Safe to call at any time; the next wrapper call builds anew. */
CS_API void cs_release_cached_plan(void);
/* Number of kernel launches issued by this process so far. */
CS_API long long cs_kernel_launch_count(void);
/* Library version string. */
CS_API const char *cs_version(void);
/* Device-side waits (mbarrier waits in the pipelined kernels) are bounded;
 * each one that expires is counted here instead of hanging the GPU. Reads
 * the count (synchronous) and, if reset, clears it. A non-zero count means
 * the affected sweeps' outputs are incomplete. */
CS_API cs_status cs_device_wait_timeouts(unsigned *count, int reset);

#ifdef __cplusplus
}
#endif
#endif /* CONVSTENCIL_H */
