/*
 * cs_oracle.c — CPU oracle (test infrastructure only; see cs_oracle.h).
 *
 * Every loop here restates the reference's naive CPU stencils; the product
 * never calls this file.
 */
#include "cs_oracle.h"

#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------------- */
/* Seeded inputs. SplitMix64 (Steele, Lea, Flood 2014), doubles from the   */
/* top 53 bits. The same generator is restated in numpy in tests/ and in   */
/* the product's bench harness so that all three see identical grids.      */
/* ---------------------------------------------------------------------- */
uint64_t cso_splitmix64_next(uint64_t *state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void cso_fill_uniform(double *dst, size_t count, uint64_t seed)
{
    uint64_t s = seed;
    for (size_t i = 0; i < count; ++i)
        dst[i] = (double)(cso_splitmix64_next(&s) >> 11) * 0x1.0p-53;
}

void cso_fill_weights(double *w, int count, uint64_t seed)
{
    double sum = 0.0;
    cso_fill_uniform(w, (size_t)count, seed);
    for (int i = 0; i < count; ++i) sum += w[i];
    for (int i = 0; i < count; ++i) w[i] /= sum;
}

/* ---------------------------------------------------------------------- */
/* One sweep. naive_1d (src/1d/main.cu:38-47): out[j] = sum_k p[k+r] in[j+k] */
/* for j in [halo, N+halo). Here i0 plays the role of `halo` so that the   */
/* reference's padded layouts (1d1r has one extra leading pad element,     */
/* src/1d/gpu_1r.cu:263) can be addressed directly.                        */
/* ---------------------------------------------------------------------- */
void cso_apply_1d(const double *in, double *out, const double *w, int r,
                  long n, long i0)
{
    const int k = 2 * r + 1;
#pragma omp parallel for schedule(static)
    for (long j = i0; j < i0 + n; ++j) {
        double acc = 0.0;
        for (int t = 0; t < k; ++t) acc += w[t] * in[j + t - r];
        out[j] = acc;
    }
}

/* naive_box2d1r (src/2d/main.cu:57-115): rows [3, rows-3), cols [4, cols-4), */
/* out = sum_{i,j<7} p[7i+j] in[row-3+i][col-3+j]. Generalised to radius r */
/* and an arbitrary interior origin (r0, c0).                               */
void cso_apply_2d(const double *in, double *out, const double *w, int r,
                  long m, long n, long ld, long r0, long c0)
{
    const int k = 2 * r + 1;
#pragma omp parallel for schedule(static)
    for (long y = r0; y < r0 + m; ++y) {
        for (long x = c0; x < c0 + n; ++x) {
            double acc = 0.0;
            for (int i = 0; i < k; ++i) {
                const double *row = in + (y - r + i) * ld + (x - r);
                for (int j = 0; j < k; ++j) acc += w[i * k + j] * row[j];
            }
            out[y * ld + x] = acc;
        }
    }
}

/* naive_box3d1r_step3 / naive_star3d1r_step3 (src/3d/main.cu:42-467):     */
/* planes/rows/cols [3, dim-3), a sum over the dz = -3..3 planes.          */
void cso_apply_3d(const double *in, double *out, const double *w, int r,
                  long h, long m, long n, long ldy, long ldz,
                  long z0, long y0, long x0)
{
    const int k = 2 * r + 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (long z = z0; z < z0 + h; ++z) {
        for (long y = y0; y < y0 + m; ++y) {
            for (long x = x0; x < x0 + n; ++x) {
                double acc = 0.0;
                for (int a = 0; a < k; ++a) {
                    for (int b = 0; b < k; ++b) {
                        const double *row = in + (z - r + a) * ldz + (y - r + b) * ldy + (x - r);
                        const double *wr = w + (a * k + b) * k;
                        for (int c = 0; c < k; ++c) acc += wr[c] * row[c];
                    }
                }
                out[z * ldz + y * ldy + x] = acc;
            }
        }
    }
}

/* Ping-pong time loop: the reference wrappers launch `times` sweeps from   */
/* buffer i%2 into buffer (i+1)%2 (src/2d/gpu.cu:409-411).                  */
int cso_run_1d(double *a, double *b, const double *w, int r, long n, long i0,
               int sweeps)
{
    double *buf[2] = {a, b};
    for (int t = 0; t < sweeps; ++t) cso_apply_1d(buf[t & 1], buf[(t + 1) & 1], w, r, n, i0);
    return sweeps & 1;
}

int cso_run_2d(double *a, double *b, const double *w, int r, long m, long n,
               long ld, long r0, long c0, int sweeps)
{
    double *buf[2] = {a, b};
    for (int t = 0; t < sweeps; ++t)
        cso_apply_2d(buf[t & 1], buf[(t + 1) & 1], w, r, m, n, ld, r0, c0);
    return sweeps & 1;
}

int cso_run_3d(double *a, double *b, const double *w, int r, long h, long m,
               long n, long ldy, long ldz, long z0, long y0, long x0,
               int sweeps)
{
    double *buf[2] = {a, b};
    for (int t = 0; t < sweeps; ++t)
        cso_apply_3d(buf[t & 1], buf[(t + 1) & 1], w, r, h, m, n, ldy, ldz, z0, y0, x0);
    return sweeps & 1;
}

/* ---------------------------------------------------------------------- */
/* Weight algebra.                                                         */
/* Composition of correlation sweeps: two sweeps with kernels u (radius a) */
/* and v (radius b) on an unbounded grid equal one sweep with the full     */
/* convolution u*v (radius a+b). The reference hand-expands this for k=3   */
/* (src/1d/main.cu:133-140, src/2d/main.cu:233-281) and k=2                */
/* (src/1d/main.cu:142-150).                                               */
/* ---------------------------------------------------------------------- */
static void conv_full(const double *u, int ru, const double *v, int rv,
                      int dims, double *out)
{
    const int ku = 2 * ru + 1, kv = 2 * rv + 1, ko = ku + kv - 1;
    long no = 1;
    for (int d = 0; d < dims; ++d) no *= ko;
    memset(out, 0, sizeof(double) * (size_t)no);
    if (dims == 1) {
        for (int i = 0; i < ku; ++i)
            for (int j = 0; j < kv; ++j) out[i + j] += u[i] * v[j];
    } else if (dims == 2) {
        for (int i0 = 0; i0 < ku; ++i0)
            for (int i1 = 0; i1 < ku; ++i1)
                for (int j0 = 0; j0 < kv; ++j0)
                    for (int j1 = 0; j1 < kv; ++j1)
                        out[(i0 + j0) * ko + (i1 + j1)] += u[i0 * ku + i1] * v[j0 * kv + j1];
    } else {
        for (int i0 = 0; i0 < ku; ++i0)
            for (int i1 = 0; i1 < ku; ++i1)
                for (int i2 = 0; i2 < ku; ++i2)
                    for (int j0 = 0; j0 < kv; ++j0)
                        for (int j1 = 0; j1 < kv; ++j1)
                            for (int j2 = 0; j2 < kv; ++j2)
                                out[((i0 + j0) * ko + (i1 + j1)) * ko + (i2 + j2)] +=
                                    u[(i0 * ku + i1) * ku + i2] * v[(j0 * kv + j1) * kv + j2];
    }
}

void cso_selfconv(const double *w, int dims, int r, int k, double *out)
{
    long n1 = 1;
    for (int d = 0; d < dims; ++d) n1 *= (2 * r * k + 1);
    double *acc = (double *)malloc(sizeof(double) * (size_t)n1);
    double *tmp = (double *)malloc(sizeof(double) * (size_t)n1);
    long nw = 1;
    for (int d = 0; d < dims; ++d) nw *= (2 * r + 1);
    memcpy(acc, w, sizeof(double) * (size_t)nw);
    for (int s = 1; s < k; ++s) {
        conv_full(acc, r * s, w, r, dims, tmp);
        long nt = 1;
        for (int d = 0; d < dims; ++d) nt *= (2 * r * (s + 1) + 1);
        memcpy(acc, tmp, sizeof(double) * (size_t)nt);
    }
    memcpy(out, acc, sizeof(double) * (size_t)n1);
    free(acc);
    free(tmp);
}

/* --custom for star2d1r places its 5 values at cells 1,3,4,5,7 of the 3x3 */
/* (src/2d/main.cu:211-217).                                                */
void cso_star2d1r_to_dense(const double *p5, double *w9)
{
    memset(w9, 0, 9 * sizeof(double));
    w9[1] = p5[0];
    w9[3] = p5[1];
    w9[4] = p5[2];
    w9[5] = p5[3];
    w9[7] = p5[4];
}

void cso_star2d3r_to_dense(const double *p13, double *w49)
{
    int t = 0;
    memset(w49, 0, 49 * sizeof(double));
    for (int i = 0; i < 7; ++i)
        for (int j = 0; j < 7; ++j)
            if (i == 3 || j == 3) w49[i * 7 + j] = p13[t++];
}

/* --custom for star3d1r places its 7 values at cells 4,10,12,13,14,16,22  */
/* of the 3x3x3 (src/3d/main.cu:557-565).                                   */
void cso_star3d1r_to_dense(const double *p7, double *w27)
{
    static const int cell[7] = {4, 10, 12, 13, 14, 16, 22};
    memset(w27, 0, 27 * sizeof(double));
    for (int i = 0; i < 7; ++i) w27[cell[i]] = p7[i];
}

/* Box 3D: plane p of 49 weights serves dz = -(3-p) and dz = +(3-p); within */
/* a plane weight i*7+j multiplies in[y-3+i][x-3+j] (src/3d/main.cu:115-467). */
void cso_box3d_planes_to_dense(const double *p196, double *w343)
{
    for (int a = 0; a < 7; ++a) {
        const int dz = a - 3;
        const int plane = 3 - (dz < 0 ? -dz : dz);
        memcpy(w343 + a * 49, p196 + plane * 49, 49 * sizeof(double));
    }
}

/* Star 3D fused: the plane at |dz| holds the row-major cells of the diamond */
/* |dy|+|dx| <= 3-|dz|; parameter blocks start at 0 (|dz|=3), 1 (|dz|=2),    */
/* 6 (|dz|=1) and 19 (dz=0) (src/3d/main.cu:42-113, gpu_star.cu:30-56).      */
void cso_star3d_params_to_dense(const double *p44, double *w343)
{
    static const int base[4] = {0, 1, 6, 19}; /* indexed by 3-|dz| */
    memset(w343, 0, 343 * sizeof(double));
    for (int a = 0; a < 7; ++a) {
        const int dz = a - 3, adz = dz < 0 ? -dz : dz, rho = 3 - adz;
        int t = base[rho];
        for (int i = 0; i < 7; ++i) {
            for (int j = 0; j < 7; ++j) {
                const int dy = i - 3, dx = j - 3;
                const int l1 = (dy < 0 ? -dy : dy) + (dx < 0 ? -dx : dx);
                if (l1 <= rho) w343[(a * 7 + i) * 7 + j] = p44[t++];
            }
        }
    }
}
