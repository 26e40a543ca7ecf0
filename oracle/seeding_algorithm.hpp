/*
 * seeding_algorithm.hpp -- C++ face of the CPU oracle (test infrastructure
 * only: the reference the GPU path is compared with in the tests, never a
 * product path).
 *
 * The reference's host algorithm classes over the C restatement in
 * seeding_oracle.c, with the same constructor arguments and operator():
 *
 *   oracle::host::seeding_algorithm         <- traccc::host::seeding_algorithm
 *       core/include/traccc/seeding/seeding_algorithm.hpp:40-52
 *       (finder, grid, filter configs; spacepoint view -> seed collection)
 *   oracle::host::track_params_estimation   <- traccc::host::track_params_estimation
 *       core/include/traccc/seeding/track_params_estimation.hpp
 *       (config; measurements, spacepoints, seeds, field -> parameters)
 *
 * The views are the oracle's own SoA structs (vecmem is not available); a
 * rejected configuration throws std::domain_error as the reference's
 * get_axes does (spacepoint_binning_helper.hpp:33-38,77-81).  Link with
 * oracle/_lib/libseedoracle.so (built by oracle/Makefile).
 */
#ifndef ORACLE_SEEDING_ALGORITHM_HPP
#define ORACLE_SEEDING_ALGORITHM_HPP

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

extern "C" {
#include "seeding_oracle.h"
}

namespace oracle {

struct seeding_configs {
    or_finder_config finder;
    or_grid_config grid;
    or_filter_config filter;

    /* The reference defaults: seedfinder_config() + setup(), the grid config
     * derived from it, seedfilter_config(). */
    static seeding_configs defaults() {
        seeding_configs c{};
        or_finder_config_default(&c.finder);
        or_finder_config_setup(&c.finder);
        or_grid_config_from_finder(&c.grid, &c.finder);
        or_filter_config_default(&c.filter);
        return c;
    }
};

namespace host {

class seeding_algorithm {
public:
    using output_type = std::vector<or_seed>;

    seeding_algorithm(const or_finder_config& finder, const or_grid_config& grid,
                      const or_filter_config& filter, int phi_mode = OR_PHI_LIBM)
        : finder_(finder), grid_(grid), filter_(filter), phi_mode_(phi_mode) {
        or_axes ax;
        if (or_get_axes(&grid_, &ax) != 0)
            throw std::domain_error("seeding_algorithm: invalid spacepoint grid config");
    }

    /* Seeds of one event, in the reference host seeding's order. */
    output_type operator()(const or_spacepoints& spacepoints) const {
        output_type out(16 + 5ull * spacepoints.size);
        for (int attempt = 0; attempt < 2; ++attempt) {
            uint32_t n = 0;
            const int rc = or_seeding(&finder_, &grid_, &filter_, &spacepoints, phi_mode_,
                                      out.data(), static_cast<uint32_t>(out.size()), &n,
                                      &stats_);
            if (rc == 0) {
                out.resize(n);
                return out;
            }
            if (rc != -1) throw std::domain_error("seeding_algorithm: error " + std::to_string(rc));
            out.resize(n);  // -1: too small, n is the size needed
        }
        throw std::runtime_error("seeding_algorithm: output size");
    }

    /* Work counters of the last call. */
    const or_stats& stats() const { return stats_; }

private:
    or_finder_config finder_;
    or_grid_config grid_;
    or_filter_config filter_;
    int phi_mode_;
    mutable or_stats stats_{};
};

class track_params_estimation {
public:
    using output_type = std::vector<or_bound_params>;

    explicit track_params_estimation(const or_tp_config& config) : config_(config) {}

    output_type operator()(const or_measurements& measurements,
                           const or_spacepoints& spacepoints, const std::vector<or_seed>& seeds,
                           const std::array<float, 3>& bfield) const {
        output_type out(seeds.size());
        if (!seeds.empty() &&
            or_track_params(&config_, &measurements, &spacepoints, seeds.data(),
                            static_cast<uint32_t>(seeds.size()), bfield.data(), out.data()) != 0)
            throw std::runtime_error("track_params_estimation: error");
        return out;
    }

private:
    or_tp_config config_;
};

}  // namespace host
}  // namespace oracle

#endif
