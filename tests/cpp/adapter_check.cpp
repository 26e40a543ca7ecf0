// Drives the C++ algorithm classes of include/seedgb.hpp the way traccc's
// examples drive theirs (seeding_example_cuda.cpp: construct with configs and
// a stream, call operator(), copy the result back), for the GPU test in
// tests/test_gpu_cpp_adapter.py.
//
//   adapter_check <event.bin> <out.bin>
//
// event.bin: uint32 n_sp, uint32 n_meas, then the columns
//   measurement_index_1 u32[n_sp], measurement_index_2 u32[n_sp],
//   global f32[3 n_sp], z_variance f32[n_sp], radius_variance f32[n_sp],
//   local_position f32[2 n_meas], surface_link u64[n_meas]
// out.bin: uint32 n_seeds, seeds {u32 b, m, t; f32 q}[n_seeds],
//   parameters seedgb_bound_track_parameters[n_seeds],
//   uint32 batch seed counts [2] (the same event twice through the batch call;
//   the batch's parameters, one launch, must equal the single call's: exit 4)
// Also: the parameters handed to the track finding's layout round-trip every
// field (exit 5); the autotuner picks one of its candidates (exit 6); a
// filter trained and gate-calibrated on the event keeps a subset of the
// plain seeds (exit 7).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
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

template <typename T>
static seedgb::device_buffer<T> to_device(const std::vector<T>& v) {
    seedgb::device_buffer<T> d(v.size());
    if (!v.empty()) cudaMemcpy(d.data(), v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
    return d;
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t n_sp = 0, n_meas = 0;
    if (std::fread(&n_sp, 4, 1, f) != 1 || std::fread(&n_meas, 4, 1, f) != 1) return 2;
    const auto mi1 = read_vec<uint32_t>(f, n_sp), mi2 = read_vec<uint32_t>(f, n_sp);
    const auto glob = read_vec<float>(f, 3ull * n_sp);
    const auto zvar = read_vec<float>(f, n_sp), rvar = read_vec<float>(f, n_sp);
    const auto loc = read_vec<float>(f, 2ull * n_meas);
    const auto link = read_vec<uint64_t>(f, n_meas);
    std::fclose(f);

    const auto d_mi1 = to_device(mi1), d_mi2 = to_device(mi2);
    const auto d_glob = to_device(glob), d_zvar = to_device(zvar), d_rvar = to_device(rvar);
    const auto d_loc = to_device(loc);
    const auto d_link = to_device(link);
    const seedgb_spacepoint_view sps{d_mi1.data(), d_mi2.data(), d_glob.data(), d_zvar.data(),
                                     d_rvar.data(), n_sp};
    const seedgb_measurement_view meas{d_loc.data(), d_link.data(), n_meas};

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
        const seedgb::triplet_seeding_algorithm seeding(finder, grid, filter, stream);
        const seedgb::seed_parameter_estimation_algorithm params(tp, stream);
        const seedgb::seed_collection_buffer seeds = seeding(sps);
        const seedgb::track_params_buffer pars =
            params({0.f, 0.f, finder.bFieldInZ}, meas, sps, seeds);
        seeding.check_status();
        const auto hs = seeds.to_host(stream);
        const auto hp = pars.to_host(stream);
        const auto batch = seeding(std::vector<seedgb_spacepoint_view>{sps, sps});
        seeding.check_status();
        uint32_t nb[2] = {static_cast<uint32_t>(batch[0].to_host(stream).size()),
                          static_cast<uint32_t>(batch[1].to_host(stream).size())};
        // parameters of the batch in one launch: the same bytes as the
        // single-event call
        const auto bpars =
            params({0.f, 0.f, finder.bFieldInZ}, std::vector<seedgb_measurement_view>{meas, meas},
                   std::vector<seedgb_spacepoint_view>{sps, sps}, batch);
        for (const auto& bp : bpars) {
            const auto h = bp.to_host(stream);
            if (h.size() != hp.size() ||
                (!h.empty() && std::memcmp(h.data(), hp.data(), sizeof(h[0]) * h.size()) != 0))
                return 4;
        }
        // the CKF hand-off: vector, barcode, column-major covariance
        {
            const auto ckf = seedgb::to_ckf(pars, stream).to_host(stream);
            if (ckf.size() != hp.size()) return 5;
            for (std::size_t i = 0; i < ckf.size(); ++i) {
                if (std::memcmp(ckf[i].vector, hp[i].params, sizeof hp[i].params) != 0 ||
                    ckf[i].barcode != hp[i].surface_link)
                    return 5;
                for (int r = 0; r < 6; ++r)
                    for (int c = 0; c < 6; ++c)
                        if (std::memcmp(&ckf[i].covariance[c * 6 + r], &hp[i].cov[r * 6 + c],
                                        4) != 0)
                            return 5;
            }
        }
        // the autotuner on a two-event batch, two candidate shapes
        {
            seedgb::triplet_seeding_algorithm tuned(finder, grid, filter, stream);
            const std::vector<seedgb_tune> cand{{8, 256, 2048, 1}, {12, 64, 2048, 1}};
            const seedgb_tune best = tuned.autotune({sps, sps}, cand, 2);
            if (!((best.warps_per_cta == 8 && best.middles_per_item == 256) ||
                  (best.warps_per_cta == 12 && best.middles_per_item == 64)))
                return 6;
            tuned.check_status();
        }
        // the learned filter: train, calibrate the gate, seed a subset
        {
            seedgb::triplet_seeding_algorithm learned(finder, grid, filter, stream);
            const seedgb_filter_train_config cfg{2, 4096, 3e-3f, 0.2f, 7u, 1};
            seedgb_doublet_filter f =
                learned.train_filter({sps}, {52.f, 94.f, 144.f, 216.f, 310.f, 430.f}, cfg);
            learned.calibrate_gate(f, {sps}, {}, 0.99f, 0.99f);
            learned.set_filter(&f);
            const auto gated = learned(sps).to_host(stream);
            learned.check_status();
            learned.set_filter(nullptr);
            std::size_t j = 0;  // gated seeds appear in the plain seeds, in order
            for (const auto& g : gated) {
                while (j < hs.size() && std::memcmp(&hs[j], &g, sizeof g) != 0) ++j;
                if (j == hs.size()) return 7;
                ++j;
            }
            if (gated.empty() || gated.size() > hs.size()) return 7;
        }
        // a rejected configuration is a std::domain_error, as in the reference
        bool threw = false;
        try {
            seedgb_spacepoint_grid_config bad = grid;
            bad.minPt = 0.01f;
            seedgb::triplet_seeding_algorithm broken(finder, bad, filter, stream);
        } catch (const std::domain_error&) {
            threw = true;
        }
        if (!threw) return 3;
        std::FILE* o = std::fopen(argv[2], "wb");
        if (!o) return 2;
        const uint32_t n = static_cast<uint32_t>(hs.size());
        std::fwrite(&n, 4, 1, o);
        std::fwrite(hs.data(), sizeof(seedgb::seed), n, o);
        std::fwrite(hp.data(), sizeof(seedgb_bound_track_parameters), hp.size(), o);
        std::fwrite(nb, 4, 2, o);
        std::fclose(o);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    cudaStreamDestroy(stream);
    return 0;
}
