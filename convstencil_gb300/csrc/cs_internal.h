// cs_internal.h — shared declarations between the host library and the kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace cs {

// Tap patterns a kernel can be specialised for. A dense (2r+1)^d weight array
// is classified on the host into the smallest pattern that covers its
// non-zero taps, so zero taps cost no FP64 instructions.
enum Pattern : int {
    PAT_DENSE = 0,   // every tap of the (2r+1)^d box
    PAT_STAR = 1,    // axis-aligned cross: taps with at most one non-zero offset
    PAT_DIAMOND = 2  // L1 ball: |d0| + |d1| (+ |d2|) <= r  (2D diamond, 3D octahedron)
};

constexpr int kMaxTaps = 343;  // 7^3

struct Weights {
    double v[kMaxTaps];
};

// A grid as the kernels see it: pointer to interior point (0,..,0), extents and
// pitches slowest axis first (pitch of the last axis is 1).
struct GridView {
    int dims;
    long long ext[3];
    long long pitch[3];
};

// Kernel entry points (cs_kernels_fp64.cu). Each launches one sweep
// in -> out on `stream`; `in`/`out` address interior point 0. Returns
// cudaSuccess or the launch error.
// tile_rows (2D only): 16 or 32 rows per CTA tile, 0 = by grid size.
cudaError_t launch_fp64_fma(const GridView &g, int radius, int pattern, const Weights &w,
                            const double *in, double *out, cudaStream_t stream, int tile_rows = 0);
// FP64 tensor-core path (mma.sync m8n8k4.f64), 2D radius-3 dense kernels only.
cudaError_t launch_fp64_mma_2d(const GridView &g, const Weights &w, const double *in, double *out,
                               cudaStream_t stream);
bool fp64_fma_supported(int dims, int radius, int pattern);

// Split precision (cs_kernels_split.cu). Grids hold float2 (hi, lo) pairs.
// use_mma selects the FP16 tensor-core slice kernel (2D, radius 3, layouts
// accepted by split_mma_layout_ok), otherwise double-float FP32 kernels run.
cudaError_t launch_split_sweep(const GridView &g, int radius, int pattern, const Weights &w,
                               int use_mma, const float2 *in, float2 *out, cudaStream_t stream);
bool split_supported(int dims, int radius, int pattern);
// The 3D double-float sweeps (cs_kernels_split3d.cu); called by launch_split_sweep.
cudaError_t launch_split_sweep_3d(const GridView &g, int radius, int pattern, const Weights &w,
                                  const float2 *in, float2 *out, cudaStream_t stream);
// Temporal blocking: T (2..4) steps per launch of the double-float kernels,
// 2D radius 1 and 1D radius 1-2; bitwise identical to T single sweeps.
bool split_tb_supported(int dims, int radius, int pattern);
cudaError_t launch_split_sweep_tb(const GridView &g, int radius, int pattern, int T, const Weights &w,
                                  const float2 *in, float2 *out, cudaStream_t stream);
bool split_mma_layout_ok(const GridView &g, long long origin);
// TMA-fed variant of the mma.sync slice kernel (cs_kernels_split_tma.cu);
// needs an even row pitch, >= 4 halo columns left of the interior (the TMA box
// starts 16-byte aligned at x0-4), >= 3 halo rows, and a 16-byte aligned base.
bool split_tma_layout_ok(const GridView &g, long long origin, const void *base);
cudaError_t launch_split_sweep_tma(const GridView &g, const Weights &w, long long origin,
                                   long long elements, const float2 *in_base, float2 *out_base,
                                   cudaStream_t stream);
// Bounded device-side waits of the tcgen05 kernels, per launch.
struct TcWait {
    unsigned long long limit_ns = 2000000000ull;  // bound of one mbarrier wait
    int skip_loads = 0;  // test hook: issue no TMA loads, so the first wait runs out
};
// tcgen05 slice kernel with TMEM accumulators (cs_kernels_split_tc.cu); same
// layout conditions as the TMA variant.
cudaError_t launch_split_sweep_tc(const GridView &g, const Weights &w, long long origin,
                                  long long elements, const float2 *in_base, float2 *out_base,
                                  const TcWait &wait, cudaStream_t stream);
// The same pipeline on FP64 grids (2D dense 7x7): six exact 9-bit digits per
// operand cut from the FP64 bits by integer operations, exact FP32 level sums
// on tcgen05, integer recombination to FP64. Layout conditions as above.
cudaError_t launch_fp64_sweep_tc(const GridView &g, const Weights &w, long long origin, long long elements,
                                 const double *in_base, double *out_base, const TcWait &wait,
                                 cudaStream_t stream);
// Batches of 2D radius-3 grids on the tcgen05 kernels (split or FP64): one
// device record per grid (tc_batch_record_bytes each, 128-byte aligned)
// holding its tensor map over `in_base`, output, sizes, first tile and
// weight digits; tiles of a grid are numbered from tile_begin and *tiles
// returns their count. Records with the same digits_id must hold the same
// weights (a CTA crossing between them keeps its B matrices). One launch
// advances every grid by one sweep; each CTA takes a contiguous run of tiles.
size_t tc_batch_record_bytes(bool fp64);
cudaError_t tc_batch_fill_record(bool fp64, void *rec, const GridView &g, const Weights &w, long long origin,
                                 long long elements, const void *in_base, void *out_base, int tile_begin,
                                 int digits_id, int *tiles);
cudaError_t launch_tc_batch(bool fp64, const void *records, int ngrids, int total_tiles, const TcWait &wait,
                            cudaStream_t stream);
// 2D tensor map over a whole (hi, lo) buffer of `rows` x `ld` pairs, box_x x box_y tiles.
cudaError_t encode_split_window_map(CUtensorMap *map, const float2 *base, long long ld, long long rows,
                                    unsigned box_x, unsigned box_y);
// 1D FP64 sweep of radius <= 3 on the 2D tcgen05 digit kernel: the n
// interior points at `origin` (n a multiple of 64 and >= 512, origin even and
// >= 4, at least 60 points of the array after them, 16-byte aligned bases) as
// rows of 64 outputs, each read as the 72 points around them; w7 holds the
// taps in row 3 of a 7x7.
cudaError_t launch_fp64_sweep_tc_rows1d(long long n, const Weights &w7, long long origin, long long elements,
                                        const double *in_base, double *out_base, const TcWait &wait,
                                        cudaStream_t stream);
// 3D tensor map: `planes` planes of pitch ldz, rows of pitch ld; box
// box_x x box_y x 1.
cudaError_t encode_split_window_map_3d(CUtensorMap *map, const float2 *base, long long ld, long long ldz,
                                       long long planes, unsigned box_x, unsigned box_y);
// tcgen05 slice kernel for dense 3x3x3 (27-point) split plans
// (cs_kernels_split_tc3d.cu). Needs even row and plane pitches, a plane pitch
// that is a whole number of rows, an even interior column offset and 16-byte
// aligned buffers.
bool split_tc3d_layout_ok(const GridView &g, long long origin, const void *in_base, const void *out_base);
cudaError_t launch_split_sweep_tc3d(const GridView &g, const Weights &w, long long origin,
                                    long long elements, const float2 *in_base, float2 *out_base,
                                    const TcWait &wait, cudaStream_t stream);
// The same pipeline on FP64 grids of dense 3x3x3 plans: six digits cut from
// the FP64 bits with integer operations, exact level sums, one rounding to
// FP64 per output (an output whose parts had different plane exponents is
// summed in FP64). Same layout conditions.
cudaError_t launch_fp64_sweep_tc3d(const GridView &g, const Weights &w, long long origin, long long elements,
                                   const double *in_base, double *out_base, const TcWait &wait,
                                   cudaStream_t stream);
int device_sm_count();
// Bounded device-side waits that expired since the last reset (TMA/mma.sync
// kernel, 2D and 3D tcgen05 kernels).
cudaError_t split_wait_timeouts(unsigned *count, bool reset);
cudaError_t split_tc_wait_timeouts(unsigned *count, bool reset);
cudaError_t split_tc3d_wait_timeouts(unsigned *count, bool reset);
// Whole-buffer conversions over n elements, and the in-place forms used by
// the FP64 re-anchor sweeps ((hi, lo) pairs and FP64 values share a buffer
// layout: 8 bytes per point).
cudaError_t launch_split_from_fp64(long long n, const double *src, float2 *dst, cudaStream_t stream);
cudaError_t launch_split_to_fp64(long long n, const float2 *src, double *dst, cudaStream_t stream);
cudaError_t launch_split_to_fp64_inplace(long long n, void *grid, cudaStream_t stream);
cudaError_t launch_fp64_to_split_inplace(long long n, void *grid, cudaStream_t stream);

// Process-wide launch counter (host side), for the bench's launch accounting.
void note_launch(long long n = 1);

}  // namespace cs
