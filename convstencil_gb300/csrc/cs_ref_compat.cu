// cs_ref_compat.cu — the reference's wrapper symbols with C++ linkage
// (include/convstencil_ref.h), forwarding to the C ABI. On failure they
// report and exit(1), as the reference's CUDA_CHECK does (src/2d/2d_utils.h:51-65).
#include "../../include/convstencil.h"
#include "../../include/convstencil_ref.h"

#include <cstdio>
#include <cstdlib>

namespace {

void check(cs_status s, const char *fn)
{
    if (s == CS_OK) return;
    printf("CUDA Error:\n");
    printf("    File:       %s\n", __FILE__);
    printf("    Function:   %s\n", fn);
    printf("    Error code: %d\n", (int)s);
    printf("    Error text: %s (%s)\n", cs_status_string(s), cs_last_error());
    exit(1);
}

struct Verbose {  // the reference always prints its timing lines
    Verbose() { cs_set_verbose(1); }
    ~Verbose() { cs_set_verbose(0); }
};

}  // namespace

#define CS_FWD_1D(name, target)                                                              \
    __attribute__((visibility("default"))) void name(                                        \
        const double *__restrict__ in, double *__restrict__ out,                             \
        const double *__restrict__ params, const int times, const int n)                     \
    {                                                                                        \
        Verbose v;                                                                           \
        check(target(in, out, params, times, n), #name);                                     \
    }
#define CS_FWD_2D(name, target)                                                              \
    __attribute__((visibility("default"))) void name(                                        \
        const double *__restrict__ in, double *__restrict__ out,                             \
        const double *__restrict__ params, const int times, const int m, const int n)        \
    {                                                                                        \
        Verbose v;                                                                           \
        check(target(in, out, params, times, m, n), #name);                                  \
    }
#define CS_FWD_3D(name, target)                                                              \
    __attribute__((visibility("default"))) void name(                                        \
        const double *__restrict__ in, double *__restrict__ out,                             \
        const double *__restrict__ params, const int times, const int h, const int m,        \
        const int n)                                                                         \
    {                                                                                        \
        Verbose v;                                                                           \
        check(target(in, out, params, times, h, m, n), #name);                               \
    }

CS_FWD_1D(gpu_1d1r, cs_gpu_1d1r)
CS_FWD_1D(gpu_1d1r_breakdown1, cs_gpu_1d1r)
CS_FWD_1D(gpu_1d1r_breakdown2, cs_gpu_1d1r)
CS_FWD_1D(gpu_1d1r_breakdown3, cs_gpu_1d1r)
CS_FWD_1D(gpu_1d1r_breakdown4, cs_gpu_1d1r)
CS_FWD_1D(gpu_star_1d2r_step2, cs_gpu_star_1d2r_step2)
CS_FWD_2D(gpu_box_2d1r, cs_gpu_box_2d1r)
CS_FWD_2D(gpu_box_2d3r, cs_gpu_box_2d3r)
CS_FWD_2D(gpu_box_2d1r_breakdown1, cs_gpu_box_2d1r)
CS_FWD_2D(gpu_box_2d1r_breakdown2, cs_gpu_box_2d1r)
CS_FWD_2D(gpu_box_2d1r_breakdown3, cs_gpu_box_2d1r)
CS_FWD_2D(gpu_box_2d1r_breakdown4, cs_gpu_box_2d1r)
CS_FWD_3D(gpu_box_3d1r, cs_gpu_box_3d1r)
CS_FWD_3D(gpu_box_3d1r_breakdown1, cs_gpu_box_3d1r)
CS_FWD_3D(gpu_box_3d1r_breakdown2, cs_gpu_box_3d1r)
CS_FWD_3D(gpu_box_3d1r_breakdown3, cs_gpu_box_3d1r)
CS_FWD_3D(gpu_box_3d1r_breakdown4, cs_gpu_box_3d1r)
CS_FWD_3D(gpu_star_3d1r, cs_gpu_star_3d1r)
