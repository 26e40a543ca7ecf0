// A C++ caller of the whole stage through include/seedgb.hpp, the way a
// traccc-style full chain would use it (examples/run/cuda/src/
// full_chain_algorithm.cpp:230-247): measurements of many events ->
// spacepoint formation (one call) -> seeding (one call) -> parameter
// estimation (one call) -> the track finding's parameter records.  For the
// GPU test in tests/test_gpu_cpp_adapter.py.
//
//   full_chain_check <in.bin> <out.bin>
//
// in.bin: uint32 n_events, uint32 n_surfaces, seedgb_surface[n_surfaces],
//   then per event: uint32 n_meas, f32 local_position[2 n_meas],
//   u64 surface_link[n_meas]
// out.bin, per event: uint32 n_sp, uint32 n_seeds, the formed spacepoints'
//   global f32[3 n_sp], seeds {u32 b, m, t; f32 q}[n_seeds],
//   seedgb_ckf_bound_track_parameters[n_seeds]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "seedgb.hpp"

template <typename T>
static std::vector<T> read_vec(std::FILE* f, std::size_t n) {
    std::vector<T> v(n);
    if (n && std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "short read\n");
        std::exit(2);
    }
    return v;
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t n_events = 0, n_surf = 0;
    if (std::fread(&n_events, 4, 1, f) != 1 || std::fread(&n_surf, 4, 1, f) != 1) return 2;
    const auto surfaces = read_vec<seedgb_surface>(f, n_surf);
    std::vector<seedgb::device_buffer<float>> loc;
    std::vector<seedgb::device_buffer<uint64_t>> link;
    std::vector<seedgb_measurement_view> meas;
    for (uint32_t e = 0; e < n_events; ++e) {
        uint32_t n = 0;
        if (std::fread(&n, 4, 1, f) != 1) return 2;
        const auto l = read_vec<float>(f, 2ull * n);
        const auto s = read_vec<uint64_t>(f, n);
        loc.emplace_back(2ull * n);
        link.emplace_back(n);
        if (n) {
            cudaMemcpy(loc.back().data(), l.data(), 8ull * n, cudaMemcpyHostToDevice);
            cudaMemcpy(link.back().data(), s.data(), 8ull * n, cudaMemcpyHostToDevice);
        }
        meas.push_back(seedgb_measurement_view{loc.back().data(), link.back().data(), n});
    }
    std::fclose(f);

    cudaStream_t stream;
    cudaStreamCreate(&stream);
    seedgb_seedfinder_config finder;
    seedgb_spacepoint_grid_config grid;
    seedgb_seedfilter_config filter;
    seedgb_track_params_estimation_config tp;
    seedgb_seedfinder_config_default(&finder);
    seedgb_spacepoint_grid_config_from_finder(&grid, &finder);
    seedgb_seedfilter_config_default(&filter);
    seedgb_track_params_estimation_config_default(&tp);
    try {
        const seedgb::spacepoint_formation_algorithm formation(surfaces, stream);
        const seedgb::triplet_seeding_algorithm seeding(finder, grid, filter, stream);
        const seedgb::seed_parameter_estimation_algorithm params(tp, stream);
        const auto formed = formation(meas);
        std::vector<seedgb_spacepoint_view> sps;
        for (const auto& b : formed) sps.push_back(b.view(b.count(stream)));
        const auto seeds = seeding(sps);
        const auto pars = params({0.f, 0.f, finder.bFieldInZ}, meas, sps, seeds);
        seeding.check_status();
        std::FILE* o = std::fopen(argv[2], "wb");
        if (!o) return 2;
        for (uint32_t e = 0; e < n_events; ++e) {
            const auto hs = seeds[e].to_host(stream);
            const auto ckf = seedgb::to_ckf(pars[e], stream).to_host(stream);
            if (ckf.size() != hs.size()) return 5;
            std::vector<float> g(3ull * sps[e].size);
            if (!g.empty())
                cudaMemcpy(g.data(), sps[e].global, 4 * g.size(), cudaMemcpyDeviceToHost);
            const uint32_t hdr[2] = {sps[e].size, static_cast<uint32_t>(hs.size())};
            std::fwrite(hdr, 4, 2, o);
            std::fwrite(g.data(), 4, g.size(), o);
            std::fwrite(hs.data(), sizeof(seedgb::seed), hs.size(), o);
            std::fwrite(ckf.data(), sizeof(seedgb_ckf_bound_track_parameters), ckf.size(), o);
        }
        std::fclose(o);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    cudaStreamDestroy(stream);
    return 0;
}
