// convstencil_1d — drop-in for the reference's 1D program (src/1d/main.cu:49-286):
//   convstencil_1d {1d1r|1d2r} N T [--custom|--breakdown|--help]
// Same command line, prompts, defaults (weights 1..7 and 1..9) and output
// lines; --custom cubes 3 values (1d1r) or squares 5 values (1d2r) exactly as
// the reference does (src/1d/main.cu:133-150). The grid is seeded uniform
// [0,1) with a zero halo.
#include <string>
#include <vector>

#include "cli_common.h"

static void help()
{
    printf("Program name: convstencil_1d\n"
           "Usage: convstencil_2 shape input_size time_iteration_size [Options]\n"
           "Shape: 1d1r or 1d2r\n"
           "Options:\n"
           "  --help    Display this help message and exit\n"
           "  --custom  If you want to use costum parameters, please use this option and input your "
           "parameters like 0.2 0.2 0.2 0.2 0.2 if the shape is star2d1r\n\n");
}

int main(int argc, char **argv)
{
    if (argc < 4 || std::string(argv[argc - 1]) == "--help") {
        help();
        return argc < 4 ? 1 : 0;
    }
    const std::string shape = argv[1];
    if (shape != "1d1r" && shape != "1d2r") {
        help();
        return 1;
    }
    int v[2];
    if (!cli::parse_ints(argv, 2, 2, v)) return 1;
    const int n = v[0], times = v[1];
    const bool r1 = shape == "1d1r";
    std::vector<double> p(r1 ? 7 : 9);
    for (size_t i = 0; i < p.size(); ++i) p[i] = (double)(i + 1);
    const bool custom = argc == 5 && std::string(argv[4]) == "--custom";
    const bool breakdown = argc == 5 && std::string(argv[4]) == "--breakdown";
    if (custom) {
        std::vector<double> in;
        if (!cli::read_params(r1 ? 3 : 5, in)) return 1;
        if (r1) {
            p = cli::selfconv(in, 1, 3);
        } else {  // square of a radius-2 kernel
            std::vector<double> sq(9, 0.0);
            for (int i = 0; i < 5; ++i)
                for (int j = 0; j < 5; ++j) sq[i + j] += in[i] * in[j];
            p = sq;
        }
    }
    printf("INFO: shape = %s,  n = %d, times = %d\n", shape.c_str(), n, times);
    const int halo = r1 ? 3 : 4;
    std::vector<double> in((size_t)n + 2 * halo + 1, 0.0), out((size_t)n + 2 * halo + 1, 0.0);
    // 1d1r's device layout has one leading pad element (src/1d/gpu_1r.cu:263).
    cli::fill_uniform(in.data() + (r1 ? 4 : 4), n, 1);
    cs_set_verbose(1);
    const int runs = breakdown && r1 ? 5 : 1;
    for (int r = 0; r < runs; ++r) {
        cs_status s = r1 ? cs_gpu_1d1r(in.data(), out.data(), p.data(), times, n)
                         : cs_gpu_star_1d2r_step2(in.data(), out.data(), p.data(), times, n);
        if (s != CS_OK) return cli::fail(s);
    }
    return 0;
}
