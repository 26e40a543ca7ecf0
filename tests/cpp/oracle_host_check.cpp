// Runs the oracle's C++ classes (oracle/seeding_algorithm.hpp) the way the
// reference's host seeding example runs traccc::host::seeding_algorithm and
// track_params_estimation: one event from a binary file, default configs,
// seeds and parameters written to an output file; a rejected grid config
// must throw std::domain_error.
#include <cstdio>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "seeding_algorithm.hpp"

template <typename T>
static bool read_n(std::FILE* f, std::vector<T>& v, size_t n) {
    v.resize(n);
    return n == 0 || std::fread(v.data(), sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    uint32_t hdr[2];
    if (std::fread(hdr, sizeof(uint32_t), 2, f) != 2) return 4;
    const uint32_t n = hdr[0], nm = hdr[1];
    std::vector<uint32_t> mi1, mi2;
    std::vector<float> global, zvar, rvar, lp;
    std::vector<uint64_t> sl;
    if (!read_n(f, mi1, n) || !read_n(f, mi2, n) || !read_n(f, global, 3ull * n) ||
        !read_n(f, zvar, n) || !read_n(f, rvar, n) || !read_n(f, lp, 2ull * nm) ||
        !read_n(f, sl, nm))
        return 5;
    std::fclose(f);

    const auto cfg = oracle::seeding_configs::defaults();
    const oracle::host::seeding_algorithm seeding(cfg.finder, cfg.grid, cfg.filter, OR_PHI_CR);
    const or_spacepoints sps{mi1.data(), mi2.data(), global.data(), zvar.data(), rvar.data(), n};
    const std::vector<or_seed> seeds = seeding(sps);

    or_tp_config tp;
    or_tp_config_default(&tp);
    const oracle::host::track_params_estimation params(tp);
    const or_measurements meas{lp.data(), sl.data(), nm};
    const auto pars = params(meas, sps, seeds, {0.f, 0.f, cfg.finder.bFieldInZ});

    // a grid that get_axes rejects (minimum helix radius below rMax / 2,
    // spacepoint_binning_helper.hpp:33-38) throws std::domain_error
    int threw = 0;
    try {
        or_grid_config bad = cfg.grid;
        bad.minPt = cfg.grid.minPt * 1e-3f;
        oracle::host::seeding_algorithm rejected(cfg.finder, bad, cfg.filter);
        (void)rejected;
    } catch (const std::domain_error&) {
        threw = 1;
    }

    std::FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 6;
    const uint32_t ns = static_cast<uint32_t>(seeds.size());
    std::fwrite(&ns, sizeof ns, 1, o);
    if (ns) {
        std::fwrite(seeds.data(), sizeof(or_seed), ns, o);
        std::fwrite(pars.data(), sizeof(or_bound_params), ns, o);
    }
    std::fwrite(&threw, sizeof threw, 1, o);
    std::fclose(o);
    return 0;
}
