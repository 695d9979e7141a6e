// Exposes the reference's CPU stencils naive_star3d1r_step3 and
// naive_box3d1r_step3 (src/3d/main.cu:42-467) with C linkage.
// Test infrastructure only; built by oracle/build_ref.sh.
#include "main.cu"
extern "C" void ref_naive_star3d1r_step3(double *in, double *out, double *param, int h, int r, int c)
{
    naive_star3d1r_step3(in, out, param, h, r, c);
}
extern "C" void ref_naive_box3d1r_step3(double *in, double *out, double *param, int h, int r, int c)
{
    naive_box3d1r_step3(in, out, param, h, r, c);
}
