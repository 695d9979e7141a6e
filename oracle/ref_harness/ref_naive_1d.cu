// Exposes the reference's CPU stencil naive_1d (src/1d/main.cu:38-47) with C
// linkage. The reference file is compiled where it lies; `main` is renamed by
// the build recipe (oracle/build_ref.sh). Test infrastructure only.
#include "main.cu"
extern "C" void ref_naive_1d(double *in, double *out, double *param, int n, int halo)
{
    naive_1d(in, out, param, n, halo);
}
