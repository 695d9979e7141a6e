// cs_kernels_split3d.cu — the 3D double-float split sweeps (kept apart from
// cs_kernels_split.cu so the two compile in parallel: the fused 7x7x7 forms
// unroll 343 taps).
#include "cs_internal.h"
#include "cs_split_common.cuh"
#include "cs_split_ff.cuh"

#include <algorithm>
#include <mutex>

namespace cs {
namespace {

using namespace ff;

unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Rows per thread of the 7-point star kernel (tile 32 x 8 kStarRows).
constexpr int kStarRows = 2;

// Planes per CTA of the z-marching 3D kernels: 32 on large grids; fewer on
// small ones, so that the grid still gives every SM several CTAs (a CTA
// marches its planes one after another, so a small grid with 32-plane
// columns would leave most SMs idle and make each sweep a long serial chain).
int z_chunk(const GridView &g, int tile_rows = 16)
{
    const long long cols = (long long)ceil_div(g.ext[2], 32) * ceil_div(g.ext[1], tile_rows);
    const long long want = 4LL * device_sm_count();
    long long zc = (g.ext[0] * cols + want - 1) / want;
    return (int)std::max(1LL, std::min(32LL, zc));
}


// Dense 3D kernels (27 or 343 taps). CTA column of 16 x 32 outputs marching
// zc planes in z. Thread (lx, ly) computes rows ly and ly + 8 of column lx
// together, one output per lane of
// packed FP32 pairs. Each input plane of the ring is stored as row pairs:
// slot s holds rows s and s + 8 of the window side by side (hi parts in one
// array, lo parts in another), so a tap reads both outputs' inputs with one
// 64-bit load.
template <int R, int P>
__global__ void __launch_bounds__(256) k3d_ff2(const float2 *__restrict__ in, float2 *__restrict__ out,
                                               int h, int m, int n, long long ldy, long long ldz, int zc,
                                               FW2<(2 * R + 1) * (2 * R + 1) * (2 * R + 1)> w)
{
    using split::f2x;
    constexpr int K = 2 * R + 1, TX = 32, TY = 16;
    constexpr int SX = TX + 2 * R, NS = TY / 2 + 2 * R;  // columns, row-pair slots
    constexpr int HALF = NS * SX;                         // pairs per hi (or lo) array
    extern __shared__ f2x ring3[];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * zc;
    const int zend = min(z0 + zc, h);
    auto load_plane = [&](int gz) {
        float *hi = reinterpret_cast<float *>(ring3 + ((gz + K) % K) * 2 * HALF);
        float *lo = hi + 2 * HALF;
        const bool zok = gz < h + R;
        for (int idx = threadIdx.x; idx < 2 * HALF; idx += blockDim.x) {
            const int half = idx & 1, rest = idx >> 1;
            const int sy = rest / SX, sx = rest - sy * SX;
            const int gy = y0 - R + sy + (TY / 2) * half, gx = x0 - R + sx;
            const float2 v = (zok && gy < m + R && gx < n + R)
                                 ? in[(long long)gz * ldz + (long long)gy * ldy + gx]
                                 : make_float2(0.f, 0.f);
            hi[idx] = v.x;
            lo[idx] = v.y;
        }
    };
    for (int gz = z0 - R; gz < z0 + R; ++gz) load_plane(gz);
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    for (int z = z0; z < zend; ++z) {
        load_plane(z + R);
        __syncthreads();
        f2x sh = 0ull, sl = 0ull;
        // Planes of the radius-3 (fused 7x7x7) kernels stay a loop: 49 taps
        // unrolled per plane keep the code size and compile time in bounds.
#pragma unroll(R == 1 ? K : 1)
        for (int a = 0; a < K; ++a) {
            const f2x *ph = ring3 + ((z - R + a + K) % K) * 2 * HALF + ly * SX + lx;
            const f2x *pl = ph + HALF;
#pragma unroll
            for (int i = 0; i < K; ++i)
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if (tap3s<P, R>(a, i, j)) {
                        const int t = (a * K + i) * K + j;
                        ff_tap2(sh, sl, w.w[t], w.nw[t], w.wl[t], ph[i * SX + j], pl[i * SX + j]);
                    }
        }
        float2 r0, r1;
        ff_finish2(sh, sl, r0, r1);
        const int x = x0 + lx, ya = y0 + ly, yb = ya + TY / 2;
        if (x < n) {
            if (ya < m) out[(long long)z * ldz + (long long)ya * ldy + x] = r0;
            if (yb < m) out[(long long)z * ldz + (long long)yb * ldy + x] = r1;
        }
        __syncthreads();
    }
}

// Scalar form (one output at a time per thread, float2 ring): used for the
// sparse star and diamond patterns, where loading the planes outweighs the
// arithmetic that the packed form halves.
template <int R, int P>
__global__ void __launch_bounds__(256) k3d_ff1(const float2 *__restrict__ in, float2 *__restrict__ out,
                                              int h, int m, int n, long long ldy, long long ldz, int zc,
                                              FW<(2 * R + 1) * (2 * R + 1) * (2 * R + 1)> w)
{
    constexpr int K = 2 * R + 1, TX = 32, TY = 16;
    constexpr int SX = TX + 2 * R, SY = TY + 2 * R, PL = SX * SY;
    extern __shared__ float2 ring2[];
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * zc;
    const int zend = min(z0 + zc, h);
    auto load_plane = [&](int gz) {
        float2 *dst = ring2 + ((gz + K) % K) * PL;
        const bool zok = gz < h + R;
        for (int idx = threadIdx.x; idx < PL; idx += blockDim.x) {
            const int sy = idx / SX, sx = idx - sy * SX;
            const int gy = y0 - R + sy, gx = x0 - R + sx;
            dst[idx] = (zok && gy < m + R && gx < n + R)
                           ? in[(long long)gz * ldz + (long long)gy * ldy + gx]
                           : make_float2(0.f, 0.f);
        }
    };
    for (int gz = z0 - R; gz < z0 + R; ++gz) load_plane(gz);
    const int lx = threadIdx.x & 31, ly0 = threadIdx.x >> 5;
    for (int z = z0; z < zend; ++z) {
        load_plane(z + R);
        __syncthreads();
#pragma unroll 1
        for (int q = 0; q < 2; ++q) {
            const int ly = ly0 + 8 * q;
            float sh = 0.f, sl = 0.f;
            // Planes of the radius-3 (fused 7x7x7) kernels stay a loop (see k3d_ff2).
#pragma unroll(R == 1 ? K : 1)
            for (int a = 0; a < K; ++a) {
                const float2 *pl = ring2 + ((z - R + a + K) % K) * PL + ly * SX + lx;
#pragma unroll
                for (int i = 0; i < K; ++i)
#pragma unroll
                    for (int j = 0; j < K; ++j)
                        if (tap3s<P, R>(a, i, j)) {
                            const float2 v = pl[i * SX + j];
                            const int t = (a * K + i) * K + j;
                            ff_tap(sh, sl, w.hi[t], w.lo[t], v.x, v.y);
                        }
            }
            const int y = y0 + ly, x = x0 + lx;
            if (y < m && x < n) out[(long long)z * ldz + (long long)y * ldy + x] = ff_finish(sh, sl);
        }
        __syncthreads();
    }
}

// The 7-point star (radius 1). A CTA owns a 32 x (8 RPT) column of outputs
// and marches zc planes; thread (lx, ly) computes rows ly, ly + 8, ... of
// column lx. The z neighbours of its outputs stay in registers (planes z-1,
// z, z+1), plane z+2 is loaded one iteration ahead, and only plane z with its
// x/y halo goes through shared memory, double buffered so that one barrier
// per plane suffices: in iteration z the CTA reads buffer z and fills buffer
// z+1 (its interior from the registers holding plane z+1, its halo ring from
// loads issued one iteration earlier by the first 2 + RPT/2 warps). Taps in
// the order of k3d_ff1 (z-1, y-1, x-1, centre, x+1, y+1, z+1), so the sums
// are the same.
template <int RPT>
__global__ void __launch_bounds__(256) k3d_star1(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                int h, int m, int n, long long ldy, long long ldz, int zc,
                                                FW<27> w)
{
    constexpr int TX = 32, TY = 8 * RPT, SX = TX + 2, SY = TY + 2;
    constexpr int kHaloWarps = 2 + RPT / 2;  // rows above and below, then the side columns
    __shared__ float2 pl[2][SY][SX];
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * zc;
    const int zend = min(z0 + zc, h);
    // Loads stay inside the buffer: coordinates -1 .. m (rows), -1 .. n
    // (columns), -1 .. h (planes) relative to the interior origin.
    const int x = x0 + lx;
    const float2 *p0 = in + (long long)(y0 + ly) * ldy + x;
    bool rok[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) rok[q] = x <= n && y0 + ly + 8 * q <= m;
    // Halo ring (edges only; a star reads no corner).
    int hy = 0, hx = 0;
    if (ly == 0) {
        hy = 0, hx = 1 + lx;
    } else if (ly == 1) {
        hy = SY - 1, hx = 1 + lx;
    } else if (ly < kHaloWarps) {
        const int k = (ly - 2) * 32 + lx;  // 0 .. 2 TY - 1
        hy = 1 + (k < TY ? k : k - TY), hx = k < TY ? 0 : SX - 1;
    }
    const bool hown = ly < kHaloWarps;
    const int hgy = y0 - 1 + hy, hgx = x0 - 1 + hx;
    const bool hok = hown && hgy <= m && hgx <= n;
    const float2 *ph = in + (long long)hgy * ldy + hgx;
    const float2 zero = make_float2(0.f, 0.f);
    auto ld = [&](bool ok, const float2 *p, int gz) { return (ok && gz <= h) ? p[(long long)gz * ldz] : zero; };
    auto row = [&](int q) { return p0 + (long long)(8 * q) * ldy; };

    float2 zm[RPT], zk[RPT], zp[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
        zm[q] = ld(rok[q], row(q), z0 - 1);
        zk[q] = ld(rok[q], row(q), z0);
        zp[q] = ld(rok[q], row(q), z0 + 1);
        pl[0][ly + 1 + 8 * q][lx + 1] = zk[q];
    }
    if (hown) pl[0][hy][hx] = ld(hok, ph, z0);
    float2 hv = ld(hok, ph, z0 + 1);
    __syncthreads();
    int buf = 0;
    for (int z = z0; z < zend; ++z) {
        float2 zn[RPT];
#pragma unroll
        for (int q = 0; q < RPT; ++q) zn[q] = ld(rok[q], row(q), z + 2);
        const float2(*s)[SX] = pl[buf];
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            const int r = ly + 8 * q;
            float sh, sl;
            ff_first(sh, sl, w.hi[4], w.lo[4], zm[q].x, zm[q].y);
            ff_tap(sh, sl, w.hi[10], w.lo[10], s[r][lx + 1].x, s[r][lx + 1].y);
            ff_tap(sh, sl, w.hi[12], w.lo[12], s[r + 1][lx].x, s[r + 1][lx].y);
            ff_tap(sh, sl, w.hi[13], w.lo[13], zk[q].x, zk[q].y);
            ff_tap(sh, sl, w.hi[14], w.lo[14], s[r + 1][lx + 2].x, s[r + 1][lx + 2].y);
            ff_tap(sh, sl, w.hi[16], w.lo[16], s[r + 2][lx + 1].x, s[r + 2][lx + 1].y);
            ff_tap(sh, sl, w.hi[22], w.lo[22], zp[q].x, zp[q].y);
            const int y = y0 + r;
            if (x < n && y < m) out[(long long)z * ldz + (long long)y * ldy + x] = ff_finish(sh, sl);
        }
        buf ^= 1;
#pragma unroll
        for (int q = 0; q < RPT; ++q) pl[buf][ly + 1 + 8 * q][lx + 1] = zp[q];
        if (hown) pl[buf][hy][hx] = hv;
        hv = ld(hok, ph, z + 2);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            zm[q] = zk[q];
            zk[q] = zp[q];
            zp[q] = zn[q];
        }
    }
}

template <int R, int P>
cudaError_t go3d(const GridView &g, const Weights &w, const float2 *in, float2 *out, cudaStream_t st)
{
    constexpr int K = 2 * R + 1;
    const int zc = z_chunk(g);
    dim3 grid(ceil_div(g.ext[2], 32), ceil_div(g.ext[1], 16), ceil_div(g.ext[0], zc));
    if constexpr (R == 1 && P == PAT_STAR) {
        constexpr int RPT = kStarRows;
        const int zs = z_chunk(g, 8 * RPT);
        dim3 sgrid(ceil_div(g.ext[2], 32), ceil_div(g.ext[1], 8 * RPT), ceil_div(g.ext[0], zs));
        k3d_star1<RPT><<<sgrid, 256, 0, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], (int)g.ext[2], g.pitch[1],
                                              g.pitch[0], zs, pack_ff<27>(w));
    } else if constexpr (P == PAT_DENSE) {
        constexpr int smem = K * 2 * (8 + 2 * R) * (32 + 2 * R) * (int)sizeof(split::f2x);
        static std::once_flag once;
        static cudaError_t attr = cudaSuccess;
        std::call_once(once, [] {
            if (smem > 48 * 1024)
                attr = cudaFuncSetAttribute(k3d_ff2<R, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        });
        if (attr != cudaSuccess) return attr;
        k3d_ff2<R, P><<<grid, 256, smem, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], (int)g.ext[2],
                                                g.pitch[1], g.pitch[0], zc, pack_ff2<K * K * K>(w));
    } else {
        constexpr int smem = K * (16 + 2 * R) * (32 + 2 * R) * (int)sizeof(float2);
        static_assert(smem <= 48 * 1024, "3D ring exceeds the default shared-memory window");
        k3d_ff1<R, P><<<grid, 256, smem, st>>>(in, out, (int)g.ext[0], (int)g.ext[1], (int)g.ext[2],
                                                g.pitch[1], g.pitch[0], zc, pack_ff<K * K * K>(w));
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_split_sweep_3d(const GridView &g, int R, int P, const Weights &w, const float2 *in,
                                  float2 *out, cudaStream_t st)
{
    if (R == 1) {
        if (P == PAT_STAR) return go3d<1, PAT_STAR>(g, w, in, out, st);
        return go3d<1, PAT_DENSE>(g, w, in, out, st);
    }
    if (R == 3) {
        if (P == PAT_STAR) return go3d<3, PAT_STAR>(g, w, in, out, st);
        if (P == PAT_DIAMOND) return go3d<3, PAT_DIAMOND>(g, w, in, out, st);
        return go3d<3, PAT_DENSE>(g, w, in, out, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace cs
