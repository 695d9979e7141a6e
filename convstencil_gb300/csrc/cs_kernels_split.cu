// cs_kernels_split.cu — split-precision grids: FP32 (hi, lo) pairs.
#include "cs_internal.h"

namespace cs {
namespace {

__global__ void k_from_fp64(const double *__restrict__ src, float2 *__restrict__ dst, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = src[i];
        const float hi = __double2float_rn(v);
        const float lo = __double2float_rn(v - (double)hi);
        dst[i] = make_float2(hi, lo);
    }
}

__global__ void k_to_fp64(const float2 *__restrict__ src, double *__restrict__ dst, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 v = src[i];
        dst[i] = (double)v.x + (double)v.y;
    }
}

unsigned grid_for(long long n)
{
    long long b = (n + 255) / 256;
    return (unsigned)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

}  // namespace

cudaError_t launch_split_from_fp64(const GridView &g, int, const double *src, float2 *dst,
                                   cudaStream_t st)
{
    note_launch();
    k_from_fp64<<<grid_for(g.ext[0]), 256, 0, st>>>(src, dst, g.ext[0]);
    return cudaGetLastError();
}

cudaError_t launch_split_to_fp64(const GridView &g, int, const float2 *src, double *dst,
                                 cudaStream_t st)
{
    note_launch();
    k_to_fp64<<<grid_for(g.ext[0]), 256, 0, st>>>(src, dst, g.ext[0]);
    return cudaGetLastError();
}

bool split_supported(int, int, int) { return false; }

cudaError_t launch_split_sweep(const GridView &, int, int, const Weights &, int, const float2 *,
                               float2 *, cudaStream_t)
{
    return cudaErrorNotSupported;
}

cudaError_t launch_split_reanchor(const GridView &, float2 *, cudaStream_t) { return cudaSuccess; }

}  // namespace cs
