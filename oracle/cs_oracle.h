/*
 * cs_oracle.h — CPU oracle for the ConvStencil stencil sweeps.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: only tests/, the
 * smoke check in __graft_entry__.py and bench.py's CPU-baseline leg may load
 * it. The product (convstencil_gb300) never links or calls it.
 *
 * It restates, in plain C with OpenMP, the CPU reference functions of
 * microsoft/ConvStencil:
 *   naive_1d              src/1d/main.cu:38-47
 *   naive_box2d1r         src/2d/main.cu:57-115
 *   naive_star3d1r_step3  src/3d/main.cu:42-113
 *   naive_box3d1r_step3   src/3d/main.cu:115-467
 * generalised to any radius and any dense (2r+1)^d weight array, plus the
 * weight algebra the reference does on the host (the k-fold self-convolution
 * of a radius-1 kernel: src/1d/main.cu:133-150, src/2d/main.cu:233-281) and
 * the parameter layouts of the 3D wrappers (src/3d/gpu_box.cu:450-468,
 * src/3d/gpu_star.cu:30-56).
 *
 * Parity pinning: tests/golden/ holds vectors produced by the reference's own
 * naive functions (compiled from the reference sources by oracle/build_ref.sh);
 * tests/test_oracle.py checks this oracle against them.
 */
#ifndef CS_ORACLE_H
#define CS_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- seeded synthetic inputs (SplitMix64, top 53 bits -> [0,1)) ---- */
uint64_t cso_splitmix64_next(uint64_t *state);
void cso_fill_uniform(double *dst, size_t count, uint64_t seed);
/* count weights uniform in [0,1), normalised so that they sum to 1 */
void cso_fill_weights(double *w, int count, uint64_t seed);

/* ---- one sweep of a dense correlation stencil of radius r ----
 * out[p] = sum_{taps t} w[t] * in[p + t - r]  (row-major tap order, last axis
 * fastest). Only interior points are written; the halo of `out` is untouched.
 * Pointers address the whole padded array; (i0 | r0,c0 | z0,y0,x0) locate the
 * first interior point; ld* are row / plane pitches in elements.          */
void cso_apply_1d(const double *in, double *out, const double *w, int r,
                  long n, long i0);
void cso_apply_2d(const double *in, double *out, const double *w, int r,
                  long m, long n, long ld, long r0, long c0);
void cso_apply_3d(const double *in, double *out, const double *w, int r,
                  long h, long m, long n, long ldy, long ldz,
                  long z0, long y0, long x0);

/* `sweeps` applications, ping-ponging between a (input) and b. Returns 0 if
 * the result is in a, 1 if it is in b. The halo of b must be zero (as the
 * reference's second buffer is: src/2d/gpu.cu:366-368).                   */
int cso_run_1d(double *a, double *b, const double *w, int r, long n, long i0,
               int sweeps);
int cso_run_2d(double *a, double *b, const double *w, int r, long m, long n,
               long ld, long r0, long c0, int sweeps);
int cso_run_3d(double *a, double *b, const double *w, int r, long h, long m,
               long n, long ldy, long ldz, long z0, long y0, long x0,
               int sweeps);

/* ---- weight algebra ----
 * k-fold self-convolution of a dense radius-r kernel (composition of k
 * correlation sweeps on an unbounded grid). Output radius k*r, dense.      */
void cso_selfconv(const double *w, int dims, int r, int k, double *out);

/* Expand the reference's shape parameter layouts to dense kernels.         */
/* star2d1r: 5 weights (N, W, C, E, S) -> dense 3x3 (src/2d/main.cu:211-217) */
void cso_star2d1r_to_dense(const double *p5, double *w9);
/* star2d3r: 13 weights, row-major cells of the radius-3 cross -> dense 7x7 */
void cso_star2d3r_to_dense(const double *p13, double *w49);
/* star3d1r: 7 weights (z-1, y-1, x-1, C, x+1, y+1, z+1) -> dense 3x3x3
 * (src/3d/main.cu:557-565)                                                  */
void cso_star3d1r_to_dense(const double *p7, double *w27);
/* box3d1r fused: 196 = 4 planes x 49, plane p <-> |dz| = 3-p
 * (src/3d/gpu_box.cu:450-468, src/3d/main.cu:115-467) -> dense 7x7x7       */
void cso_box3d_planes_to_dense(const double *p196, double *w343);
/* star3d1r fused: 44 params of the radius-3 octahedron
 * (src/3d/main.cu:42-113, src/3d/gpu_star.cu:30-56) -> dense 7x7x7         */
void cso_star3d_params_to_dense(const double *p44, double *w343);

#ifdef __cplusplus
}
#endif
#endif
