// Exposes the reference's CPU stencil naive_box2d1r (src/2d/main.cu:57-115)
// with C linkage. Test infrastructure only; built by oracle/build_ref.sh.
#include "main.cu"
extern "C" void ref_naive_box2d1r(double *in, double *out, double *param, int rows, int cols)
{
    naive_box2d1r(in, out, param, rows, cols);
}
