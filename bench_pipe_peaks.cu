// bench_pipe_peaks.cu — issue-rate microbenchmark of the arithmetic pipes
// the stencil kernels use on this GPU: FP64 FMA, FP64 MMA (every mma.sync f64
// shape), a mix of both (are they one pipe?), FP32 FMA, FP16/BF16/TF32
// mma.sync, 32-bit integer operations, and the conversions the FP64
// tensor-core sweep leans on (FP32 -> INT32, INT64 -> FP64). Each kernel runs
// independent chains long enough to saturate its pipe; throughput = operations
// / CUDA-event time. Prints one line per pipe, or with --json one JSON object
// (bench.py reads the FP64 FMA rate from it as the FP64 roofline denominator).
// Built by convstencil_gb300/build_lib.py into convstencil_gb300/_lib/pipe_peaks.
#include <cstdio>
#include <cstring>

#include <cuda_runtime.h>

namespace {

constexpr int kIters = 4096;

__device__ __forceinline__ void sink(double r, double *out)
{
    if (r == 12345.0) out[threadIdx.x] = r;
}

__device__ void dfma_work(double *out, int n)
{
    double a[8];
    for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 1e-9 + i;
#pragma unroll 1
    for (int it = 0; it < n; ++it)
#pragma unroll
        for (int i = 0; i < 8; i++) a[i] = fma(a[i], 0.999, 1e-7);
    double r = 0;
    for (int i = 0; i < 8; i++) r += a[i];
    sink(r, out);
}

__device__ void dmma884_work(double *out, int n)
{
    const double a = threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-4;
    double c[8][2] = {};
#pragma unroll 1
    for (int it = 0; it < n; ++it)
#pragma unroll
        for (int i = 0; i < 8; i++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                         : "+d"(c[i][0]), "+d"(c[i][1])
                         : "d"(a), "d"(b));
    double r = 0;
    for (int i = 0; i < 8; i++) r += c[i][0] + c[i][1];
    sink(r, out);
}

__global__ void k_dfma(double *out) { dfma_work(out, kIters); }
__global__ void k_dmma884(double *out) { dmma884_work(out, kIters / 8); }
// Half the warps on each pipe, equal FLOPs per warp.
__global__ void k_mix(double *out)
{
    if ((threadIdx.x / 32) & 1) dmma884_work(out, kIters / 8);
    else dfma_work(out, kIters);
}

__global__ void k_dmma16816(double *out)
{
    double a[8], b[4];
    for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 1e-3 * (i + 1);
    for (int i = 0; i < 4; i++) b[i] = 1.0 - threadIdx.x * 1e-4 * (i + 1);
    double c[4][4] = {};
#pragma unroll 1
    for (int it = 0; it < kIters / 4; ++it)
#pragma unroll
        for (int i = 0; i < 4; i++)
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
                : "+d"(c[i][0]), "+d"(c[i][1]), "+d"(c[i][2]), "+d"(c[i][3])
                : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]),
                  "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
    double r = 0;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r += c[i][j];
    sink(r, out);
}

__global__ void k_ffma(double *out)
{
    float a[16];
    for (int i = 0; i < 16; i++) a[i] = threadIdx.x * 1e-9f + i;
#pragma unroll 1
    for (int it = 0; it < kIters; ++it)
#pragma unroll
        for (int i = 0; i < 16; i++) a[i] = fmaf(a[i], 0.999f, 1e-7f);
    float r = 0;
    for (int i = 0; i < 16; i++) r += a[i];
    sink(r, out);
}

template <int KIND>  // 0 f16, 1 bf16, 2 tf32
__global__ void k_hmma(double *out)
{
    const unsigned one = KIND == 2 ? 0x3f800000u : (KIND == 1 ? 0x3f803f80u : 0x3c003c00u);
    const unsigned a0 = one + threadIdx.x, b0 = one;
    float c[8][4] = {};
#pragma unroll 1
    for (int it = 0; it < kIters; ++it)
#pragma unroll
        for (int i = 0; i < 8; i++) {
            if (KIND == 0)
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, "
                             "{%4,%4,%4,%4}, {%5,%5}, {%0,%1,%2,%3};"
                             : "+f"(c[i][0]), "+f"(c[i][1]), "+f"(c[i][2]), "+f"(c[i][3])
                             : "r"(a0), "r"(b0));
            else if (KIND == 1)
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, "
                             "{%4,%4,%4,%4}, {%5,%5}, {%0,%1,%2,%3};"
                             : "+f"(c[i][0]), "+f"(c[i][1]), "+f"(c[i][2]), "+f"(c[i][3])
                             : "r"(a0), "r"(b0));
            else
                asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, "
                             "{%4,%4,%4,%4}, {%5,%5}, {%0,%1,%2,%3};"
                             : "+f"(c[i][0]), "+f"(c[i][1]), "+f"(c[i][2]), "+f"(c[i][3])
                             : "r"(a0), "r"(b0));
        }
    float r = 0;
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 4; j++) r += c[i][j];
    sink(r, out);
}


// 32-bit integer ALU: independent xor/add/shift chains (LOP3, IADD3, SHF).
__global__ void k_int(double *out)
{
    unsigned a[8];
    for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 2654435761u + i;
    const unsigned k = 0x9E3779B9u + blockIdx.x;
#pragma unroll 1
    for (int it = 0; it < kIters / 2; ++it)
#pragma unroll
        for (int i = 0; i < 8; i++) {
            asm volatile("xor.b32 %0, %0, %1;" : "+r"(a[i]) : "r"(k));
            asm volatile("shf.r.wrap.b32 %0, %0, %0, 7;" : "+r"(a[i]));
        }
    unsigned r = 0;
    for (int i = 0; i < 8; i++) r += a[i];
    sink((double)r, out);
}

// 32x32 -> 64-bit multiply-add (mad.wide.s32), as used to combine levels.
__global__ void k_imad_wide(double *out)
{
    long long a[8];
    for (int i = 0; i < 8; i++) a[i] = threadIdx.x + i;
    const int m = 512 + blockIdx.x;
#pragma unroll 1
    for (int it = 0; it < kIters; ++it)
#pragma unroll
        for (int i = 0; i < 8; i++) asm volatile("mad.wide.s32 %0, %1, %2, %0;" : "+l"(a[i]) : "r"(m), "r"(i + 3));
    long long r = 0;
    for (int i = 0; i < 8; i++) r += a[i];
    sink((double)r, out);
}

// FP32 -> INT32 conversion (cvt.rni.s32.f32).
__global__ void k_f2i(double *out)
{
    float a[8];
    int acc[8] = {};
    for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 1.25f + i;
#pragma unroll 1
    for (int it = 0; it < kIters / 2; ++it)
#pragma unroll
        for (int i = 0; i < 8; i++) {
            int v;
            asm volatile("cvt.rni.s32.f32 %0, %1;" : "=r"(v) : "f"(a[i]));
            acc[i] += v;
        }
    int r = 0;
    for (int i = 0; i < 8; i++) r += acc[i];
    sink((double)r, out);
}

// INT64 -> FP64 conversion (cvt.rn.f64.s64).
__global__ void k_i2d(double *out)
{
    long long a[8];
    double acc[8] = {};
    for (int i = 0; i < 8; i++) a[i] = (long long)threadIdx.x * 1000003 + i;
#pragma unroll 1
    for (int it = 0; it < kIters / 8; ++it)
#pragma unroll
        for (int i = 0; i < 8; i++) {
            double v;
            asm volatile("cvt.rn.f64.s64 %0, %1;" : "=d"(v) : "l"(a[i] + it));
            acc[i] = v;
        }
    double r = 0;
    for (int i = 0; i < 8; i++) r += acc[i];
    sink(r, out);
}

}  // namespace

int main(int argc, char **argv)
{
    const bool json = argc > 1 && !strcmp(argv[1], "--json");
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
        printf("no CUDA device\n");
        return 1;
    }
    double *d = nullptr;
    cudaMalloc(&d, 1 << 20);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const dim3 grid(p.multiProcessorCount * 4), block(256);
    const double warps = grid.x * 8.0, threads = grid.x * 256.0;
    if (json)
        printf("{\"device\": \"%s\", \"sms\": %d", p.name, p.multiProcessorCount);
    else
        printf("device %s, %d SMs, cc %d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
    auto run = [&](const char *name, auto launch, double flops) {
        launch();
        cudaDeviceSynchronize();
        cudaEventRecord(e0);
        for (int r = 0; r < 3; ++r) launch();
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        const cudaError_t err = cudaGetLastError();
        const double rate = flops / (ms / 3 * 1e-3) / 1e12;
        if (json)
            printf(", \"%s\": %.4f", name, err == cudaSuccess ? rate : -1.0);
        else
            printf("%-28s %10.2f T/s  (%s)\n", name, rate, cudaGetErrorString(err));
    };
    run("fp64 fma", [&] { k_dfma<<<grid, block>>>(d); }, threads * 8 * 2.0 * kIters);
    run("fp64 mma m8n8k4", [&] { k_dmma884<<<grid, block>>>(d); }, warps * 8 * 512.0 * (kIters / 8));
    run("fp64 mma m16n8k16", [&] { k_dmma16816<<<grid, block>>>(d); },
        warps * 4 * 4096.0 * (kIters / 4));
    run("fp64 fma+mma (half each)", [&] { k_mix<<<grid, block>>>(d); },
        warps / 2 * 512.0 * kIters + warps / 2 * 8 * 512.0 * (kIters / 8));
    run("fp32 fma", [&] { k_ffma<<<grid, block>>>(d); }, threads * 16 * 2.0 * kIters);
    run("fp16 mma.sync m16n8k16", [&] { k_hmma<0><<<grid, block>>>(d); }, warps * 8 * 4096.0 * kIters);
    run("bf16 mma.sync m16n8k16", [&] { k_hmma<1><<<grid, block>>>(d); }, warps * 8 * 4096.0 * kIters);
    run("tf32 mma.sync m16n8k8", [&] { k_hmma<2><<<grid, block>>>(d); }, warps * 8 * 2048.0 * kIters);
    // Operations (not FLOPs) per second for the rest.
    run("int32 xor+shf ops", [&] { k_int<<<grid, block>>>(d); }, threads * 8 * 2.0 * (kIters / 2));
    run("mad.wide.s32 ops", [&] { k_imad_wide<<<grid, block>>>(d); }, threads * 8.0 * kIters);
    run("cvt f32->s32 ops", [&] { k_f2i<<<grid, block>>>(d); }, threads * 8.0 * (kIters / 2));
    run("cvt s64->f64 ops", [&] { k_i2d<<<grid, block>>>(d); }, threads * 8.0 * (kIters / 8));
    if (json) printf("}\n");
    cudaFree(d);
    return 0;
}
