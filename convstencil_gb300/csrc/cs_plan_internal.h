// cs_plan_internal.h — library-internal access to plans and batches, shared
// by the plan code (cs_api.cu), the batcher (cs_batch.cu) and the server
// (cs_serve.cu). Not part of the C ABI.
#pragma once

#include "../../include/convstencil.h"
#include "cs_internal.h"

namespace cs {

// Read-only view of a plan.
struct PlanFacts {
    int dims, radius, pattern, steps_per_sweep;
    cs_precision prec;
    GridView view;
    long long origin, elements;
    long long reanchor;  // split: FP64 re-anchor interval in sweeps (0 = never)
    int algo;            // the pinned cs_algo (CS_ALGO_AUTO: the tuner's)
    const Weights *w;
};
bool plan_facts(const cs_plan *p, PlanFacts *f);
cs_status set_error(cs_status s, const char *msg);

// cs_run with the sweeps numbered from first_sweep (so chunked runs take
// their FP64 re-anchor sweeps at the same global sweep counts).
cs_status run_from(cs_plan *p, void *a, void *b, long long first_sweep, long long steps, cudaStream_t st,
                   int *result_in_b);
// One FP64 re-anchor sweep of a split plan: (hi, lo) state in src -> dst.
cudaError_t fp64_anchor_sweep(const cs_plan *p, void *src, void *dst, cudaStream_t st);

// cs_batch_create with per-grid sweep counts (NULL: unbounded), the tcgen05
// path optional, and tables allocated in order on mem_stream when not NULL.
cs_status batch_create_ex(cs_batch **out, cs_plan *const *plans, void *const *a, void *const *b, int count,
                          const long long *sweeps, bool allow_tc, cudaStream_t mem_stream);
// One launch of sweep `sweep` for every grid of the batch with more sweeps.
cs_status batch_sweep(cs_batch *bt, long long sweep, cudaStream_t st);

}  // namespace cs
