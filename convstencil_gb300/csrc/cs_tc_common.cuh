// cs_tc_common.cuh — building blocks shared by the tcgen05 split kernels
// (cs_kernels_split_tc.cu for 2D, cs_kernels_split_tc3d.cu for 3D): bounded
// mbarrier waits, shared-memory matrix and instruction descriptors for
// kind::f16 MMAs with TMEM accumulators, TMEM loads and TMA tile loads.
//
// Every wait is bounded by WaitCfg::limit_ns of %globaltimer (2 s unless the
// plan sets another limit). An expired wait adds one to the caller's device
// counter and raises the CTA's abort flag, so every role of the CTA stops at
// its next wait; mbar_drain is the bounded wait used at exit for copies and
// MMAs still in flight. The host reads the counter after synchronous runs and
// reports CS_ERR_TIMEOUT.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <utility>

namespace cs {
namespace tc {

constexpr unsigned long long kWaitNs = 2000000000ull;  // default bound of one wait

// Per-launch wait settings (kernel parameter).
struct WaitCfg {
    unsigned long long limit_ns;  // bound of every mbarrier wait
    int skip_loads;               // test hook: the producer issues no TMA loads, so the
                                  // consumers' first wait runs out and the CTA leaves
};

// Programmatic dependent launch. A sweep launched with the programmatic
// stream serialization attribute may be scheduled while the previous kernel
// of its stream is still finishing: it sets up (barriers, TMEM, B matrices)
// at once and calls pdl_wait(), which returns once the previous grid has
// completed and its writes are visible, before its first global-memory
// access (the first window load; every store comes after loads). Launched
// without the attribute, pdl_wait() returns at once. pdl_allow_dependents()
// lets the next such kernel be scheduled as this one's CTAs leave.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_allow_dependents()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches a sweep kernel with the programmatic stream serialization
// attribute (see pdl_wait).
template <typename... Exp, typename... Act>
cudaError_t launch_programmatic(void (*kernel)(Exp...), int grid, int block, size_t smem, cudaStream_t st,
                                Act &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Act>(args)...);
}

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

// The polling loop of mbar_wait, out of line: it is entered only when the
// phase is not complete at the first test.
static __device__ __noinline__ bool mbar_wait_slow(unsigned bar, unsigned parity, volatile int *abort,
                                                   unsigned *timeouts, unsigned long long limit_ns)
{
    const unsigned long long t0 = globaltimer();
    for (;;) {
        for (int i = 0; i < 16; ++i)
            if (mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
        if (globaltimer() - t0 > limit_ns) {
            atomicAdd(timeouts, 1u);
            *abort = 1;
            return false;
        }
    }
}

// Waits for the phase with the given parity. Gives up after limit_ns
// (counted in *timeouts, and *abort raised so every other role stops too) or
// as soon as another role has raised *abort. The first test is inline: a call
// costs the issuing role several hundred cycles under load (measured on the
// 3D kernel's MMA thread), and most waits find their phase complete.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, volatile int *abort, unsigned *timeouts,
                                          unsigned long long limit_ns = kWaitNs)
{
    return mbar_try_wait(bar, parity) || mbar_wait_slow(bar, parity, abort, timeouts, limit_ns);
}

// Bounded wait used only at exit for copies / MMAs still in flight.
static __device__ __noinline__ bool mbar_drain(unsigned bar, unsigned parity, unsigned *timeouts,
                                               unsigned long long limit_ns = kWaitNs)
{
    const unsigned long long t0 = globaltimer();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer() - t0 > limit_ns) {
            atomicAdd(timeouts, 1u);
            return false;
        }
    return true;
}

__device__ __forceinline__ void mbar_arrive(unsigned bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, no swizzle; lbo = byte stride of
// the 16-byte K chunks, sbo = byte stride of the 8-row groups.
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo)
{
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) | ((unsigned long long)(lbo >> 4) << 16) |
           ((unsigned long long)(sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP16 A and B, FP32 D, both K-major, M = 128.
__host__ __device__ constexpr unsigned instr_desc(int n)
{
    return (1u << 4) | ((unsigned)(n >> 3) << 17) | ((unsigned)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(unsigned d_tmem, unsigned long long a, unsigned long long b,
                                        unsigned idesc, unsigned accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(unsigned bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld8(unsigned taddr, float (&v)[8])
{
    unsigned r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap *map, int x, int y, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

}  // namespace tc
}  // namespace cs
