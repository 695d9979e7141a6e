// cs_kernels_fp64.cu — FP64 stencil sweeps for sm_103a.
//
// On GB300 the FP64 pipe is narrow: FP64 FMA and FP64 MMA (mma.sync f64, any
// shape) issue through the same unit at ~1 TFLOP/s per GPU, far below what HBM
// can feed (a sweep needs 16 B per point). A FP64 sweep is therefore bounded by
// FP64 operations, not bytes, and the kernels here are built to spend the
// fewest FP64 operations per output:
//
//  * k*_fma: one FP64 FMA per non-zero tap. Tap patterns (dense box, axis
//    cross, L1 diamond/octahedron) are compile-time, so zero taps cost
//    nothing. Weights travel in the kernel's parameter space (constant bank),
//    so every FMA takes its weight as a constant operand; inputs are staged
//    once per tile in shared memory with coalesced loads.
//
//  * k2d_mma: the tensor-core form the reference uses (its `kernel2d`,
//    src/2d/gpu.cu:30-70, runs 26 DMMA m8n8k4 per 64 outputs = 104 FMA per
//    point for 49 taps). Here each MMA column is a 2x4 block of outputs, so one
//    K row covers an 8x10 input window: 20 DMMA per 64 outputs = 80 FMA per
//    point. Still more FP64 work than the FMA form (49 per point), so the
//    plan's tuner only picks it if it measures faster.
#include "cs_internal.h"

#include <algorithm>

#include <cstdio>

namespace cs {
namespace {

template <int K>
struct WK {
    double v[K];
};

__host__ __device__ constexpr int iabs(int x) { return x < 0 ? -x : x; }

template <int P, int R>
__host__ __device__ constexpr bool tap2(int i, int j)
{
    return P == PAT_DENSE  ? true
           : P == PAT_STAR ? (i == R || j == R)
                           : (iabs(i - R) + iabs(j - R) <= R);
}

template <int P, int R>
__host__ __device__ constexpr bool tap3(int a, int i, int j)
{
    return P == PAT_DENSE ? true
           : P == PAT_STAR
               ? ((a != R) + (i != R) + (j != R) <= 1)
               : (iabs(a - R) + iabs(i - R) + iabs(j - R) <= R);
}

// ---------------------------------------------------------------- 1D
// 1024 outputs per CTA, 4 per thread. Tile + halo staged in shared memory.
template <int R>
__global__ void __launch_bounds__(256) k1d_fma(const double *__restrict__ in,
                                               double *__restrict__ out, long long n,
                                               WK<2 * R + 1> w)
{
    constexpr int T = 1024;
    __shared__ double s[T + 2 * R];
    const long long x0 = (long long)blockIdx.x * T;
    for (int i = threadIdx.x; i < T + 2 * R; i += blockDim.x) {
        const long long gx = x0 - R + i;
        s[i] = (gx < n + R) ? __ldg(in + gx) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < T / 256; ++p) {
        const int lx = threadIdx.x + p * 256;
        double acc = 0.0;
#pragma unroll
        for (int t = 0; t <= 2 * R; ++t) acc = fma(w.v[t], s[lx + t], acc);
        const long long gx = x0 + lx;
        if (gx < n) out[gx] = acc;
    }
}

// ---------------------------------------------------------------- 2D
// CTA tile (4 RPT) x 64 outputs; thread (c, g) computes column c of rows
// RPT g .. RPT g + RPT-1, sweeping the RPT+2R input rows of its column window
// once. RPT = 8 (32-row tiles) normally; RPT = 4 on grids too small to give
// every SM several 32-row tiles. Each output sums its taps in the same order
// either way.
template <int R, int P, int RPT>
__global__ void __launch_bounds__(256) k2d_fma(const double *__restrict__ in,
                                               double *__restrict__ out, int m, int n,
                                               long long ld, WK<(2 * R + 1) * (2 * R + 1)> w)
{
    constexpr int K = 2 * R + 1, TX = 64, TY = 4 * RPT;
    constexpr int SX = TX + 2 * R, SY = TY + 2 * R;
    __shared__ double s[SY * SX];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    for (int idx = threadIdx.x; idx < SY * SX; idx += blockDim.x) {
        const int sy = idx / SX, sx = idx - sy * SX;
        const int gy = y0 - R + sy, gx = x0 - R + sx;
        s[idx] = (gy < m + R && gx < n + R) ? __ldg(in + (long long)gy * ld + gx) : 0.0;
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
        // Output row o = ir - i receives input row ir through weight row i.
        // For a fixed o the rows arrive with ascending i, so each output sums
        // its taps in the (i, j) order of the reference's naive loop.
#pragma unroll
        for (int i = 0; i < K; ++i) {
            const int o = ir - i;
            if (o >= 0 && o < RPT) {
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if (tap2<P, R>(i, j)) acc[o] = fma(w.v[i * K + j], v[j], acc[o]);
            }
        }
    }
#pragma unroll
    for (int o = 0; o < RPT; ++o) {
        const int y = y0 + g * RPT + o, x = x0 + c;
        if (y < m && x < n) out[(long long)y * ld + x] = acc[o];
    }
}

// ---------------------------------------------------------------- 3D
// CTA column of 16 x 32 outputs marching ZC planes in z; a ring of 2R+1
// input planes (with halo) lives in shared memory.
template <int R>
constexpr int k3d_smem_bytes()
{
    return (2 * R + 1) * (16 + 2 * R) * (32 + 2 * R) * (int)sizeof(double);
}

template <int R, int P>
__global__ void __launch_bounds__(256) k3d_fma(const double *__restrict__ in,
                                               double *__restrict__ out, int h, int m, int n,
                                               long long ldy, long long ldz, int zc,
                                               WK<(2 * R + 1) * (2 * R + 1) * (2 * R + 1)> w)
{
    constexpr int K = 2 * R + 1, TX = 32, TY = 16;
    constexpr int SX = TX + 2 * R, SY = TY + 2 * R, PL = SX * SY;
    extern __shared__ double ring[];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * zc;
    const int zend = min(z0 + zc, h);

    auto load_plane = [&](int gz) {  // gz in [-R, h+R)
        double *dst = ring + ((gz + K) % K) * PL;
        const bool zok = gz < h + R;
        for (int idx = threadIdx.x; idx < PL; idx += blockDim.x) {
            const int sy = idx / SX, sx = idx - sy * SX;
            const int gy = y0 - R + sy, gx = x0 - R + sx;
            dst[idx] = (zok && gy < m + R && gx < n + R)
                           ? __ldg(in + (long long)gz * ldz + (long long)gy * ldy + gx)
                           : 0.0;
        }
    };
    for (int gz = z0 - R; gz < z0 + R; ++gz) load_plane(gz);
    const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
    for (int z = z0; z < zend; ++z) {
        load_plane(z + R);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int ly = ly0 + 8 * q;
            double acc = 0.0;
#pragma unroll
            for (int a = 0; a < K; ++a) {
                const double *pl = ring + ((z - R + a + K) % K) * PL + ly * SX + lx;
#pragma unroll
                for (int i = 0; i < K; ++i)
#pragma unroll
                    for (int j = 0; j < K; ++j)
                        if (tap3<P, R>(a, i, j))
                            acc = fma(w.v[(a * K + i) * K + j], pl[i * SX + j], acc);
            }
            const int y = y0 + ly, x = x0 + lx;
            if (y < m && x < n) out[(long long)z * ldz + (long long)y * ldy + x] = acc;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- 2D FP64 MMA
// mma.sync.m8n8k4.f64: A 8x4 (row), B 4x8 (col), C 8x8. Lane l holds
// A[l/4][l%4], B[l%4][l/4], C[l/4][2(l%4)], C[l/4][2(l%4)+1].
// Rows of A (M) are 8 output blocks side by side; columns of B (N) are the 8
// outputs of a 2x4 block (n = 4a + b); K runs over the block's 8x10 input
// window (k = 10r + j), so B[k][n] = w[r-a][j-b] (zero outside the 7x7).
__device__ __forceinline__ void dmma_884(double &c0, double &c1, double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(c0), "+d"(c1)
                 : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(256) k2d_mma(const double *__restrict__ in,
                                               double *__restrict__ out, int m, int n,
                                               long long ld, WK<49> w)
{
    constexpr int R = 3, TX = 64, TY = 32, SX = TX + 2 * R + 2, SY = TY + 2 * R, KS = 20;
    __shared__ double s[SY * SX];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    for (int idx = threadIdx.x; idx < SY * (TX + 2 * R); idx += blockDim.x) {
        const int sy = idx / (TX + 2 * R), sx = idx - sy * (TX + 2 * R);
        const int gy = y0 - R + sy, gx = x0 - R + sx;
        s[sy * SX + sx] = (gy < m + R && gx < n + R) ? __ldg(in + (long long)gy * ld + gx) : 0.0;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    double bf[KS];
    int off[KS];
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
        const int k = 4 * ks + t, r = k / 10, j = k - 10 * (k / 10);
        const int a = g >> 2, b = g & 3, ri = r - a, ci = j - b;
        bf[ks] = (ri >= 0 && ri < 7 && ci >= 0 && ci < 7) ? w.v[ri * 7 + ci] : 0.0;
        off[ks] = r * SX + j;
    }
    __syncthreads();
#pragma unroll
    for (int chain = 0; chain < 4; ++chain) {
        const int brow = warp * 2 + (chain >> 1);  // 2-row block row, 0..15
        const int bc = (chain & 1) * 8 + g;        // this lane's A row = block column
        const double *base = s + (2 * brow) * SX + 4 * bc;
        double c0 = 0.0, c1 = 0.0;
#pragma unroll
        for (int ks = 0; ks < KS; ++ks) dmma_884(c0, c1, base[off[ks]], bf[ks]);
        // C[g][2t], C[g][2t+1]: block (chain's g-th), outputs n = 2t, 2t+1.
        const int y = y0 + 2 * brow + (t >> 1);
        const int x = x0 + 4 * ((chain & 1) * 8 + g) + 2 * (t & 1);
        if (y < m) {
            if (x < n) out[(long long)y * ld + x] = c0;
            if (x + 1 < n) out[(long long)y * ld + x + 1] = c1;
        }
    }
}

template <int K>
WK<K> pack(const Weights &w)
{
    WK<K> p;
    for (int i = 0; i < K; ++i) p.v[i] = w.v[i];
    return p;
}

unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Planes per CTA of the z-marching 3D kernels: 32 on large grids; fewer on
// small ones, so that the grid still gives every SM several CTAs (a CTA
// marches its planes one after another, so a small grid with 32-plane
// columns would leave most SMs idle and make each sweep a long serial chain).
int z_chunk(const GridView &g)
{
    const long long cols = (long long)ceil_div(g.ext[2], 32) * ceil_div(g.ext[1], 16);
    const long long want = 4LL * device_sm_count();
    long long zc = (g.ext[0] * cols + want - 1) / want;
    return (int)std::max(1LL, std::min(32LL, zc));
}


// Rows per CTA tile: 16 (4 per thread) or 32 (8 per thread); 0 picks 16 on
// grids too small to give every SM several 32-row tiles. Both tile shapes sum
// every point's taps in the same order, so results do not depend on it.
template <int R, int P>
cudaError_t go2d(const GridView &g, const Weights &w, const double *in, double *out, int tile_rows,
                 cudaStream_t st)
{
    constexpr int K = 2 * R + 1;
    const unsigned gx = ceil_div(g.ext[1], 64);
    if (tile_rows == 0) tile_rows = (long long)gx * ceil_div(g.ext[0], 32) < 6LL * device_sm_count() ? 16 : 32;
    if (tile_rows == 16) {
        dim3 grid(gx, ceil_div(g.ext[0], 16));
        k2d_fma<R, P, 4><<<grid, 256, 0, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], g.pitch[0],
                                                pack<K * K>(w));
    } else {
        dim3 grid(gx, ceil_div(g.ext[0], 32));
        k2d_fma<R, P, 8><<<grid, 256, 0, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], g.pitch[0],
                                                pack<K * K>(w));
    }
    return cudaGetLastError();
}

template <int R, int P>
cudaError_t go3d(const GridView &g, const Weights &w, const double *in, double *out,
                 cudaStream_t st)
{
    constexpr int K = 2 * R + 1;
    constexpr int smem = k3d_smem_bytes<R>();  // <= 46,816 B: no opt-in needed
    static_assert(smem <= 48 * 1024, "3D ring exceeds the default shared-memory window");
    const int zc = z_chunk(g);
    dim3 grid(ceil_div(g.ext[2], 32), ceil_div(g.ext[1], 16), ceil_div(g.ext[0], zc));
    k3d_fma<R, P><<<grid, 256, smem, st>>>(in, out, (int)g.ext[0], (int)g.ext[1],
                                            (int)g.ext[2], g.pitch[1], g.pitch[0], zc,
                                            pack<K * K * K>(w));
    return cudaGetLastError();
}

template <int R>
cudaError_t go1d(const GridView &g, const Weights &w, const double *in, double *out,
                 cudaStream_t st)
{
    dim3 grid(ceil_div(g.ext[0], 1024));
    k1d_fma<R><<<grid, 256, 0, st>>>(in, out, g.ext[0], pack<2 * R + 1>(w));
    return cudaGetLastError();
}

}  // namespace

bool fp64_fma_supported(int dims, int radius, int pattern)
{
    if (dims == 1) return radius >= 1 && radius <= 4;
    if (dims == 2) return radius == 1 || radius == 2 || radius == 3;
    if (dims == 3) return radius == 1 || radius == 3;
    return false;
}

cudaError_t launch_fp64_fma(const GridView &g, int R, int P, const Weights &w, const double *in,
                            double *out, cudaStream_t st, int tile_rows)
{
    note_launch();
    if (g.dims == 1) {
        switch (R) {
        case 1: return go1d<1>(g, w, in, out, st);
        case 2: return go1d<2>(g, w, in, out, st);
        case 3: return go1d<3>(g, w, in, out, st);
        case 4: return go1d<4>(g, w, in, out, st);
        }
    } else if (g.dims == 2) {
        if (R == 1) {
            if (P == PAT_STAR) return go2d<1, PAT_STAR>(g, w, in, out, tile_rows, st);
            return go2d<1, PAT_DENSE>(g, w, in, out, tile_rows, st);
        }
        if (R == 2) {
            if (P == PAT_STAR) return go2d<2, PAT_STAR>(g, w, in, out, tile_rows, st);
            if (P == PAT_DIAMOND) return go2d<2, PAT_DIAMOND>(g, w, in, out, tile_rows, st);
            return go2d<2, PAT_DENSE>(g, w, in, out, tile_rows, st);
        }
        if (R == 3) {
            if (P == PAT_STAR) return go2d<3, PAT_STAR>(g, w, in, out, tile_rows, st);
            if (P == PAT_DIAMOND) return go2d<3, PAT_DIAMOND>(g, w, in, out, tile_rows, st);
            return go2d<3, PAT_DENSE>(g, w, in, out, tile_rows, st);
        }
    } else if (g.dims == 3) {
        if (R == 1) {
            if (P == PAT_STAR) return go3d<1, PAT_STAR>(g, w, in, out, st);
            return go3d<1, PAT_DENSE>(g, w, in, out, st);
        }
        if (R == 3) {
            if (P == PAT_STAR) return go3d<3, PAT_STAR>(g, w, in, out, st);
            if (P == PAT_DIAMOND) return go3d<3, PAT_DIAMOND>(g, w, in, out, st);
            return go3d<3, PAT_DENSE>(g, w, in, out, st);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_fp64_mma_2d(const GridView &g, const Weights &w, const double *in,
                               double *out, cudaStream_t st)
{
    note_launch();
    dim3 grid(ceil_div(g.ext[1], 64), ceil_div(g.ext[0], 32));
    k2d_mma<<<grid, 256, 0, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], g.pitch[0],
                                  pack<49>(w));
    return cudaGetLastError();
}

}  // namespace cs
