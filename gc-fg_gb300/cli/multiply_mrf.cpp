// multiply_mrf -- larger MRF test problems from smaller ones, in the two
// modes of the reference's tiler (multiplyMRF.cpp), written to stdout:
//
//   multiply_mrf MRF_file mult
//       the MRF `mult` times as wide (multiplyMRF.cpp:64-92): ground truth
//       all 1, t-links repeated with period W, horizontal cues with period
//       W - 1 (their last row 0, as the reference's loader leaves it),
//       vertical cues with period W;
//   multiply_mrf --square t-links.dat [side [penalty]]
//       a side x side MRF (default 3600, penalty 600; multiplyMRF.cpp:94-122)
//       whose t-links repeat the .dat arrays along each row; every cue is the
//       penalty.  Row i reads row i of the arrays, so they need >= side rows.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mrf_io.hpp"

using gcfg_cli::IntWriter;

static int tile(const char *path, int mult) {
    gcfg_cli::Mrf m = gcfg_cli::read_mrf(path);
    if (mult < 1 || m.W < 2) throw std::runtime_error("need mult >= 1 and an MRF at least 2 wide");
    const long long Wm = (long long)m.W * mult;
    IntWriter w(stdout);
    w.put(Wm);
    w.put(m.H);
    w.put(2);
    for (long long i = 0; i < Wm * m.H; ++i) w.put(1);
    for (const std::vector<int> *a : {&m.dp, &m.dn})
        for (int y = 0; y < m.H; ++y)
            for (long long x = 0; x < Wm; ++x) w.put((*a)[(size_t)y * m.W + (size_t)(x % m.W)]);
    for (int y = 0; y < m.H; ++y)
        for (long long x = 0; x + 1 < Wm; ++x) w.put(m.hcue[(size_t)y * m.W + (size_t)(x % (m.W - 1))]);
    for (int y = 0; y + 1 < m.H; ++y)
        for (long long x = 0; x < Wm; ++x) w.put(m.vcue[(size_t)y * m.W + (size_t)(x % m.W)]);
    return 0;
}

static int square(const char *dat, int side, int penalty) {
    int W = 0, H = 0;
    std::vector<int> dp, dn;
    gcfg_cli::read_dat(dat, W, H, dp, dn);
    if (side < 2 || H < side) throw std::runtime_error("the .dat arrays need at least `side` rows");
    IntWriter w(stdout);
    w.put(side);
    w.put(side);
    w.put(2);
    for (long long i = 0; i < (long long)side * side; ++i) w.put(1);
    for (const std::vector<int> *a : {&dp, &dn})
        for (int y = 0; y < side; ++y)
            for (int x = 0; x < side; ++x) w.put((*a)[(size_t)y * W + (size_t)(x % W)]);
    for (long long i = 0; i < 2LL * side * (side - 1); ++i) w.put(penalty);
    return 0;
}

int main(int argc, char **argv) {
    try {
        if (argc >= 3 && std::strcmp(argv[1], "--square") == 0)
            return square(argv[2], argc > 3 ? std::atoi(argv[3]) : 3600, argc > 4 ? std::atoi(argv[4]) : 600);
        if (argc == 3) return tile(argv[1], std::atoi(argv[2]));
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    std::fprintf(stderr, "Usage: %s MRF_file mult\n       %s --square t-links.dat [side [penalty]]\n", argv[0],
                 argv[0]);
    return 1;
}
