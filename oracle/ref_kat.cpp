// ref_kat.cpp - golden-vector generator built against the reference's own
// vendored headers (external/pcg-cpp-0.98, external/eigen) and this
// machine's libstdc++ <random>.  oracle/build_ref.py compiles it into
// oracle/_ref/ and writes its output to tests/golden/ref_kat.json.
//
// It pins the leaves of the replay contract used by oracle/rta_oracle.cpp
// and the GPU replay mode:
//   - pcg64(seed, stream) raw outputs (pcg_random.hpp:1675)
//   - std::uniform_real_distribution<double>(0,1) over pcg64, as called by
//     random_dt and Grid_distribution::sample (include/sampling.hpp:40-114)
//   - std::uniform_int_distribution<> over pcg64, as called by alma::choose
//     (include/utilities.hpp:45-49) and the void-border choice
//     (src/RTA_MC2D.cpp:1234-1235)
//   - Eigen::VectorXd::LinSpaced time grids (src/RTA_MC2D.cpp:2118-2124)
//   - glibc std::log of uniforms (random_dt's -log(u))
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#include <Eigen/Dense>
#include <pcg_random.hpp>

static void u128out(const char* key, unsigned long long seed, unsigned long long stream, int n) {
    pcg64 g(seed, stream);
    std::printf("  \"%s\": {\"seed\": %llu, \"stream\": %llu, \"raw\": [", key, seed, stream);
    for (int i = 0; i < n; ++i) std::printf("%s\"%llu\"", i ? ", " : "", (unsigned long long)g());
    std::printf("]},\n");
}

int main() {
    std::printf("{\n");
    u128out("pcg64_s0_t0", 0ULL, 0ULL, 16);
    u128out("pcg64_s42_t54", 42ULL, 54ULL, 16);
    u128out("pcg64_s20261203_t7", 20261203ULL, 7ULL, 16);
    u128out("pcg64_big", 0xfedcba9876543210ULL, 0x0123456789abcdefULL, 16);
    // canonical doubles and -log
    {
        pcg64 g(20261203ULL, 3ULL);
        std::printf("  \"canonical\": {\"seed\": 20261203, \"stream\": 3, \"u\": [");
        std::vector<double> us;
        for (int i = 0; i < 64; ++i) {
            double u = std::uniform_real_distribution(0., 1.)(g);
            us.push_back(u);
            std::printf("%s%.17g", i ? ", " : "", u);
        }
        std::printf("], \"neglog\": [");
        for (std::size_t i = 0; i < us.size(); ++i) std::printf("%s%.17g", i ? ", " : "", -std::log(us[i]));
        std::printf("]},\n");
    }
    // uniform ints for several ranges, sharing one stream in sequence
    {
        pcg64 g(99ULL, 5ULL);
        int his[] = {0, 1, 2, 3, 6, 1000, 2147483646};
        std::printf("  \"uniform_int\": {\"seed\": 99, \"stream\": 5, \"cases\": [");
        bool first = true;
        for (int hi : his)
            for (int r = 0; r < 8; ++r) {
                int v = std::uniform_int_distribution<>(0, hi)(g);
                std::printf("%s[%d, %d]", first ? "" : ", ", hi, v);
                first = false;
            }
        std::printf("]},\n");
    }
    // time grids
    {
        double cases[][2] = {{10., 1000.}, {0.25, 1000.}, {50., 10000.}, {0.3, 7.}, {1.0 / 3.0, 10.}};
        std::printf("  \"linspaced\": [");
        for (int c = 0; c < 5; ++c) {
            double dt = cases[c][0], maxtime = cases[c][1];
            std::size_t ntime = std::floor(maxtime / dt + 1.0e-6) + 1;
            maxtime = (ntime - 1) * dt;
            Eigen::VectorXd tg = Eigen::VectorXd::LinSpaced(ntime, 0.0, maxtime);
            std::printf("%s{\"dt\": %.17g, \"maxtime\": %.17g, \"grid\": [", c ? ", " : "", cases[c][0], cases[c][1]);
            for (Eigen::Index i = 0; i < tg.size(); ++i) std::printf("%s%.17g", i ? ", " : "", tg(i));
            std::printf("]}");
        }
        std::printf("]\n");
    }
    std::printf("}\n");
    return 0;
}
