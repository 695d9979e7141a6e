// cli_common.h — helpers shared by the convstencil_{1d,2d,3d} programs.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "convstencil.h"

namespace cli {

// Seeded grid values: SplitMix64, top 53 bits -> [0, 1).
inline void fill_uniform(double *dst, size_t n, uint64_t seed)
{
    uint64_t s = seed;
    for (size_t i = 0; i < n; ++i) {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        dst[i] = (double)(z >> 11) * 0x1.0p-53;
    }
}

// std::stoi with the reference's two error messages (src/2d/main.cu:168-181).
inline bool parse_ints(char **argv, int first, int count, int *out)
{
    try {
        for (int i = 0; i < count; ++i) out[i] = std::stoi(argv[first + i]);
    } catch (const std::invalid_argument &) {
        fprintf(stderr, "Invalid argument: cannot convert the parameter(s) to integer.\n");
        return false;
    } catch (const std::out_of_range &) {
        fprintf(stderr, "Argument out of range: the parameter(s) is(are) too large.\n");
        return false;
    }
    return true;
}

// "Please enter K parameters:" then K doubles from stdin (src/2d/main.cu:204-210).
inline bool read_params(int k, std::vector<double> &v)
{
    printf("Please enter %d parameters:\n", k);
    fflush(stdout);
    v.resize(k);
    for (int i = 0; i < k; ++i)
        if (scanf("%lf", &v[i]) != 1) return false;
    return true;
}

// k-fold self-convolution of a dense radius-1 kernel in `dims` dimensions:
// the fused kernel of k sweeps on an unbounded grid (what the reference's
// CLIs hand-expand for k = 3 and k = 2).
inline std::vector<double> selfconv(const std::vector<double> &w, int dims, int k)
{
    std::vector<double> acc = w;
    int r = 1;
    for (int s = 1; s < k; ++s) {
        const int ka = 2 * r + 1, kb = 3, ko = ka + 2;
        int n = 1;
        for (int d = 0; d < dims; ++d) n *= ko;
        std::vector<double> out(n, 0.0);
        int na = 1;
        for (int d = 0; d < dims; ++d) na *= ka;
        int nb = 1;
        for (int d = 0; d < dims; ++d) nb *= kb;
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
                int ra = ia, rb = ib, io = 0, mul = 1;
                for (int d = 0; d < dims; ++d) {
                    io += ((ra % ka) + (rb % kb)) * mul;
                    ra /= ka;
                    rb /= kb;
                    mul *= ko;
                }
                out[io] += acc[ia] * w[ib];
            }
        acc.swap(out);
        ++r;
    }
    return acc;
}

inline int fail(cs_status s)
{
    printf("CUDA Error:\n    Error code: %d\n    Error text: %s (%s)\n", (int)s, cs_status_string(s),
           cs_last_error());
    return 1;
}

}  // namespace cli
