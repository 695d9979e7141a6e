// convstencil_3d — drop-in for the reference's 3D program (src/3d/main.cu:469-693):
//   convstencil_3d {box3d1r|star3d1r} H M N T [--custom|--breakdown|--help]
// Same command line, prompts, defaults (196 params i/100, 44 ones) and output
// lines. Difference, by intent: --custom values are used (the reference reads
// and ignores them, src/3d/main.cu:536-567): the 27 (box) or 7 (star) base
// weights run 3*T steps of the base stencil with a zero halo. The grid is
// seeded uniform [0,1) with a zero halo.
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "cli_common.h"

static void help()
{
    printf("Program name: convstencil_2d\n"
           "Usage: convstencil_3d shape input_size_of_first_dimension input_size_of_second_dimension "
           "input_size_of_third_dimension time_iteration_size [Options]\n"
           "Shape: box3d1r or star3d1r\n"
           "Options:\n"
           "  --help    Display this help message and exit\n"
           "  --custom  If you want to use costum parameters, please use this option and input your "
           "parameters like 0.2 0.2 0.2 0.2 0.2 if the shape is star2d1r\n\n");
}

int main(int argc, char **argv)
{
    if (argc < 6 || std::string(argv[argc - 1]) == "--help") {
        help();
        return argc < 6 ? 1 : 0;
    }
    const std::string shape = argv[1];
    if (shape != "box3d1r" && shape != "star3d1r") {
        help();
        return 1;
    }
    const bool box = shape == "box3d1r";
    int v[4];
    if (!cli::parse_ints(argv, 2, 4, v)) return 1;
    const int h = v[0], m = v[1], n = v[2], times = v[3];
    const bool custom = argc == 7 && std::string(argv[6]) == "--custom";
    const bool breakdown = argc == 7 && std::string(argv[6]) == "--breakdown";
    std::vector<double> base;
    if (custom && !cli::read_params(box ? 27 : 7, base)) return 1;
    printf("INFO: shape = %s, h = %d, m = %d, n = %d, times = %d\n", box ? "box_3d1r" : "star_3d1r", h,
           m, n, times);
    const size_t H = (size_t)h + 6, R = (size_t)m + 6, C = (size_t)n + 6;
    std::vector<double> grid(H * R * C, 0.0), out(H * R * C, 0.0), row(n);
    for (int z = 0; z < h; ++z)
        for (int y = 0; y < m; ++y) {
            cli::fill_uniform(row.data(), n, 1 + ((uint64_t)z * m + y) * 0x9E3779B97F4A7C15ull);
            memcpy(&grid[((z + 3) * R + y + 3) * C + 3], row.data(), n * sizeof(double));
        }
    cs_set_verbose(1);
    if (!custom) {
        std::vector<double> p(box ? 196 : 44);
        for (size_t i = 0; i < p.size(); ++i) p[i] = box ? (double)i / 100 : 1.0;
        const int runs = breakdown && box ? 5 : 1;
        for (int r = 0; r < runs; ++r) {
            cs_status s = box ? cs_gpu_box_3d1r(grid.data(), out.data(), p.data(), times, h, m, n)
                              : cs_gpu_star_3d1r(grid.data(), out.data(), p.data(), times, h, m, n);
            if (s != CS_OK) return cli::fail(s);
        }
        return 0;
    }
    // Custom base weights: 3*T steps of the radius-1 stencil, reference layout.
    cs_layout L{};
    L.dims = 3;
    L.halo = 3;
    L.extent[0] = h;
    L.extent[1] = m;
    L.extent[2] = n;
    L.pitch[2] = 1;
    L.pitch[1] = (long long)C;
    L.pitch[0] = (long long)(R * C);
    L.origin = 3 * L.pitch[0] + 3 * L.pitch[1] + 3;
    L.elements = (long long)(H * R * C);
    const long long ext[3] = {h, m, n};
    cs_plan *p = nullptr;
    cs_status s = cs_plan_create(&p, box ? CS_SHAPE_BOX3D1R : CS_SHAPE_STAR3D1R, CS_SEM_STEP, CS_PREC_FP64,
                                 ext, base.data(), (int)base.size(), &L);
    if (s != CS_OK) return cli::fail(s);
    s = cs_run_host(p, grid.data(), out.data(), 3LL * times);
    if (s != CS_OK) return cli::fail(s);
    const double secs = cs_last_loop_seconds();
    if (box) printf("ConvStencil(3D): \n");
    printf("Time = %lld[ms]\n%g\n", (long long)(secs * 1e3), secs);
    printf("GStencil/s = %f\n", (double)h * m * n * times * 3 / secs / 1e9);
    cs_plan_destroy(p);
    return 0;
}
