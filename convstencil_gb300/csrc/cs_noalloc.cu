// cs_noalloc.cu — cs_run_noalloc: sweeps between caller-owned device buffers
// without allocating any device memory.
//
// The ping-pong partner grid that cs_run asks the caller to provide (and that
// the host-buffer wrappers cudaMalloc) lives here in a file-scope __device__
// array of fixed size, reserved on every GPU that loads this module for the
// life of the process. See cs_run_noalloc in include/convstencil.h for who
// needs this and what it costs.
#include "../../include/convstencil.h"
#include "cs_internal.h"

#include <cuda.h>

#include <cstdio>
#include <mutex>

struct cs_plan;

namespace cs {
size_t plan_bytes(const cs_plan *p);
cs_status run_into(cs_plan *p, const void *in, void *out, void *scratch, long long steps,
                   cudaStream_t st);
cs_status set_error(cs_status s, const char *msg);
}  // namespace cs

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;  // 16 MiB: 2,097,152 grid points
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Device address of the scratch, per device, with the driver context it was
// looked up in: after cudaDeviceReset (or under another context) the module
// is loaded again, possibly at another address, so a changed context repeats
// the look-up.
void *g_addr[kMaxDevices];
CUcontext g_ctx[kMaxDevices];

// The current driver context (null if none or unknown), through the runtime's
// driver entry point so that the library needs no link-time libcuda symbol.
CUcontext current_context()
{
    typedef CUresult (*CtxGetCurrent)(CUcontext *);
    static CtxGetCurrent fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrent>(p);
    });
    CUcontext ctx = nullptr;
    if (!fn || fn(&ctx) != CUDA_SUCCESS) return nullptr;
    return ctx;
}

}  // namespace

extern "C" CS_API cs_status cs_run_noalloc(cs_plan *plan, const void *in, void *out,
                                           long long steps, void *stream)
{
    if (!plan || !in || !out) return cs::set_error(CS_ERR_INVALID_ARGUMENT, "NULL plan or buffer");
    if (in == out) return cs::set_error(CS_ERR_INVALID_ARGUMENT, "input and output buffers must differ");
    const size_t bytes = cs::plan_bytes(plan);
    if (bytes > kScratchBytes) {
        char msg[200];
        snprintf(msg, sizeof msg,
                 "grid needs %zu bytes per buffer; cs_run_noalloc's fixed scratch holds %zu bytes "
                 "(use cs_run with a caller-allocated second buffer)",
                 bytes, kScratchBytes);
        return cs::set_error(CS_ERR_INVALID_ARGUMENT, msg);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cs::set_error(CS_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return cs::set_error(CS_ERR_UNSUPPORTED, "device index out of range");
    // Rejected calls leave the shared scratch untouched: the step count is
    // checked before anything is queued.
    long long sweeps = 0;
    const cs_status ss = cs_plan_sweeps(plan, steps, &sweeps);
    if (ss != CS_OK) return ss;
    void *scratch = nullptr;
    {
        // Once per device (and driver context), with that device current: the
        // host-side name of a __device__ array is not a device address, so
        // ask the runtime for it.
        std::lock_guard<std::mutex> lk(g_mu);
        CUcontext ctx = current_context();
        if (!g_addr[dev] || g_ctx[dev] != ctx) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cs::set_error(CS_ERR_CUDA, cudaGetErrorString(e));
            ctx = current_context();  // the look-up may have made the primary context current
            g_addr[dev] = p;
            g_ctx[dev] = ctx;
        }
        scratch = g_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    // The scratch keeps whatever the previous call left; its halo must read
    // as zero. A zero-sweep call only copies `in` to `out` and never reads it.
    if (sweeps > 0) {
        e = cudaMemsetAsync(scratch, 0, bytes, st);
        if (e != cudaSuccess) return cs::set_error(CS_ERR_CUDA, cudaGetErrorString(e));
    }
    return cs::run_into(plan, in, out, scratch, steps, st);
}
