// Host driver for exact_sum.cuh (compiled by tests/test_host_exact_sum.py): seeded sets of
// double-double values in several magnitude patterns, summed as the warp sums them -- 32
// lane accumulators, then the xor-shuffle tree -- and printed with the inputs in hex.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "exact_sum.cuh"

using namespace lmm;

int main(int argc, char** argv)
{
    const int cases = argc > 1 ? std::atoi(argv[1]) : 100;
    std::mt19937_64 g(20240917);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (int c = 0; c < cases; c++) {
        const int count = 1 + (int)(g() % 700);
        const int mode = c % 6;
        std::vector<double> v(2 * count);
        for (int k = 0; k < count; k++) {
            double hi;
            switch (mode) {
            case 0: hi = nd(g); break;                                                         // one scale
            case 1: hi = nd(g) * std::ldexp(1.0, (int)(g() % 200) - 100); break;               // wide range
            case 2: hi = (g() % 3 == 0) ? 0.0 : nd(g) * 1e-310; break;                         // zeros, subnormals
            case 3: hi = (k % 2 ? 1.0 : -1.0) * (1.0 + nd(g) * 1e-12); break;                  // cancellation
            case 4: hi = nd(g) * std::ldexp(1.0, (int)(g() % 2000) - 1000); break;             // beyond 2^170
            default: hi = (g() % 5 == 0) ? -0.0 : std::ldexp(nd(g), 900); break;               // large, signed zeros
            }
            double lo = hi * std::ldexp(nd(g), -54);
            const double s = hi + lo;
            lo = lo - (s - hi);
            v[2 * k] = s;
            v[2 * k + 1] = lo;
        }
        unsigned emax = 0;
        for (double x : v) emax = std::max(emax, f64_exponent_field(x));
        if (emax == 0) emax = 1;
        Fixed192 lane[32] = {};
        for (int k = 0; k < count; k++) {
            fixed_add_double(lane[k % 32], v[2 * k], emax);
            fixed_add_double(lane[k % 32], v[2 * k + 1], emax);
        }
        for (int off = 16; off > 0; off >>= 1) {
            Fixed192 next[32];
            for (int l = 0; l < 32; l++) {
                next[l] = lane[l];
                uint32_t x[6];
                for (int i = 0; i < 6; i++) x[i] = lane[l ^ off].w[i];
                fixed_add(next[l], x, 0u);
            }
            for (int l = 0; l < 32; l++) lane[l] = next[l];
        }
        for (int l = 1; l < 32; l++)
            for (int i = 0; i < 6; i++)
                if (lane[l].w[i] != lane[0].w[i]) {
                    std::printf("lanes differ\n");
                    return 1;
                }
        const dd r = fixed_to_dd(lane[0], emax);
        std::printf("%d", count);
        for (double x : v) std::printf(" %a", x);
        std::printf(" | %a %a\n", r.hi, r.lo);
    }
    return 0;
}
