// Input generator for the golden fixtures (compiled and run by make_golden.py).
//
//   gen_inputs harness   <seed> <fi> <count> <out.bin>
//       std::mt19937(seed); each value u * exp(fi * n) with u ~ uniform_real(-0.5, 0.5)
//       and n ~ normal(0, 1), the formula of the Oz-AIE test harness
//       (src/programming_examples/basic/matrix_multiplication/test.cpp:219-237).
//       Callers draw A then B from one stream, as that harness does.
//   gen_inputs uniform64 <seed> <lo> <hi> <count> <out.bin>
//       std::mt19937_64(seed); uniform_real_distribution(lo, hi).
// Values are written as little-endian doubles.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    std::vector<double> v;
    const char *out = nullptr;
    if (!std::strcmp(argv[1], "harness") && argc == 6) {
        const int seed = std::atoi(argv[2]);
        const double fi = std::atof(argv[3]);
        const long n = std::atol(argv[4]);
        out = argv[5];
        std::mt19937 rng(seed);
        std::uniform_real_distribution<double> u(-0.5, 0.5);
        std::normal_distribution<double> g(0.0, 1.0);
        v.resize(n);
        for (long i = 0; i < n; ++i) v[i] = u(rng) * std::exp(fi * g(rng));
    } else if (!std::strcmp(argv[1], "uniform64") && argc == 7) {
        const unsigned long long seed = std::strtoull(argv[2], nullptr, 10);
        const double lo = std::atof(argv[3]), hi = std::atof(argv[4]);
        const long n = std::atol(argv[5]);
        out = argv[6];
        std::mt19937_64 rng(seed);
        std::uniform_real_distribution<double> u(lo, hi);
        v.resize(n);
        for (long i = 0; i < n; ++i) v[i] = u(rng);
    } else {
        return 2;
    }
    FILE *f = std::fopen(out, "wb");
    if (!f) return 1;
    const size_t w = std::fwrite(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
    return w == v.size() ? 0 : 1;
}
