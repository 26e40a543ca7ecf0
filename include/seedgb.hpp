/*
 * seedgb.hpp -- C++ surface of the GB300 seeding library: the reference's
 * algorithm classes and operator() calls over the C ABI of seedgb.h.
 *
 *  seedgb::triplet_seeding_algorithm          <- traccc::cuda::triplet_seeding_algorithm
 *      constructor: device/cuda/include/traccc/cuda/seeding/
 *                   triplet_seeding_algorithm.hpp:35-40 (configs + stream)
 *      operator():  device/common/include/traccc/seeding/device/
 *                   triplet_seeding_algorithm.hpp:68-69 (spacepoint view ->
 *                   seed buffer, asynchronous on the stream)
 *  seedgb::seed_parameter_estimation_algorithm <- traccc::cuda::seed_parameter_estimation_algorithm
 *      operator():  device/common/include/traccc/seeding/device/
 *                   seed_parameter_estimation_algorithm.hpp:48-67
 *  seedgb::spacepoint_formation_algorithm  measurements -> spacepoints for
 *                   many events per call (core/src/seeding/
 *                   silicon_pixel_spacepoint_formation.hpp:31-60 per event)
 *  seedgb::to_ckf   the parameters in the record layout the track finding
 *                   takes (examples/run/cuda/src/full_chain_algorithm.cpp:
 *                   241-247), device-resident
 *  seedgb::gbts_seeding_algorithm           <- traccc::cuda::gbts_seeding_algorithm
 *      constructor: gbts_seedfinder_config::setLinkingScheme (core/src/
 *                   gbts_seeding/gbts_seeding_config.cpp:19-142) + stream
 *      operator():  device/common/include/traccc/gbts_seeding/device/
 *                   gbts_seeding_algorithm.hpp:94-96 (spacepoints and the
 *                   measurements' barcodes and diameters -> seed buffer)
 *      gbts_seedfinder_config::from_directory: the reference's configuration
 *                   directory (examples/options/src/track_gbts_seeding.cpp:
 *                   158-226)
 *  triplet_seeding_algorithm::autotune / train_filter / calibrate_gate /
 *                   set_filter: the library's launch-shape search and learned
 *                   doublet filter (no counterpart in the reference)
 *
 * Header-only, C++17, needs cuda_runtime.h for the device buffers.  Errors
 * are exceptions as in the reference: std::domain_error for a rejected
 * configuration (spacepoint_binning_helper.hpp:33-38), std::runtime_error
 * for CUDA and capacity failures.  Buffers own device memory (cudaMalloc /
 * cudaFree); views are borrowed.  One algorithm object per stream.
 */
#ifndef SEEDGB_HPP
#define SEEDGB_HPP

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "seedgb.h"

namespace seedgb {

inline void check(seedgb_status st, const char* what) {
    if (st == SEEDGB_OK) return;
    const std::string msg = std::string(what) + ": " + seedgb_status_string(st);
    if (st == SEEDGB_BAD_CONFIG) throw std::domain_error(msg);
    throw std::runtime_error(msg);
}

/* Device array owned by the object. */
template <typename T>
class device_buffer {
public:
    device_buffer() = default;
    explicit device_buffer(std::size_t n) : n_(n) {
        if (n && cudaMalloc(&p_, n * sizeof(T)) != cudaSuccess)
            throw std::runtime_error("cudaMalloc failed");
    }
    device_buffer(const device_buffer&) = delete;
    device_buffer& operator=(const device_buffer&) = delete;
    device_buffer(device_buffer&& o) noexcept { swap(o); }
    device_buffer& operator=(device_buffer&& o) noexcept {
        swap(o);
        return *this;
    }
    ~device_buffer() {
        if (p_) cudaFree(p_);
    }
    T* data() const { return p_; }
    std::size_t size() const { return n_; }
    void swap(device_buffer& o) noexcept {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
    }

private:
    T* p_ = nullptr;
    std::size_t n_ = 0;
};

/* One seed on the host (edm::seed: bottom, middle, top, quality). */
struct seed {
    uint32_t bottom, middle, top;
    float quality;
};

/* edm::seed_collection::buffer: four device columns and a device size,
 * resizable like the reference's buffer (triplet_seeding_algorithm.cpp:249-252). */
class seed_collection_buffer {
public:
    explicit seed_collection_buffer(uint32_t capacity)
        : bottom(capacity), middle(capacity), top(capacity), quality(capacity), size(1),
          capacity_(capacity) {}
    seedgb_seed_buffer view() const {
        return seedgb_seed_buffer{bottom.data(), middle.data(), top.data(), quality.data(),
                                  capacity_, size.data()};
    }
    uint32_t capacity() const { return capacity_; }
    /* Copy to the host (synchronises `stream`). */
    std::vector<seed> to_host(cudaStream_t stream) const {
        uint32_t n = 0;
        if (cudaMemcpyAsync(&n, size.data(), sizeof n, cudaMemcpyDeviceToHost, stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            throw std::runtime_error("seed size copy failed");
        n = n < capacity_ ? n : capacity_;
        std::vector<uint32_t> b(n), m(n), t(n);
        std::vector<float> q(n);
        if (n) {
            cudaMemcpyAsync(b.data(), bottom.data(), 4 * n, cudaMemcpyDeviceToHost, stream);
            cudaMemcpyAsync(m.data(), middle.data(), 4 * n, cudaMemcpyDeviceToHost, stream);
            cudaMemcpyAsync(t.data(), top.data(), 4 * n, cudaMemcpyDeviceToHost, stream);
            cudaMemcpyAsync(q.data(), quality.data(), 4 * n, cudaMemcpyDeviceToHost, stream);
            if (cudaStreamSynchronize(stream) != cudaSuccess)
                throw std::runtime_error("seed copy failed");
        }
        std::vector<seed> out(n);
        for (uint32_t i = 0; i < n; ++i) out[i] = seed{b[i], m[i], t[i], q[i]};
        return out;
    }

    device_buffer<uint32_t> bottom, middle, top;
    device_buffer<float> quality;
    device_buffer<uint32_t> size;

private:
    uint32_t capacity_;
};

/* bound_track_parameters_collection_types::buffer. */
class track_params_buffer {
public:
    explicit track_params_buffer(uint32_t capacity) : data(capacity), size(1), capacity_(capacity) {}
    seedgb_params_buffer view() const {
        return seedgb_params_buffer{data.data(), capacity_, size.data()};
    }
    std::vector<seedgb_bound_track_parameters> to_host(cudaStream_t stream) const {
        uint32_t n = 0;
        if (cudaMemcpyAsync(&n, size.data(), sizeof n, cudaMemcpyDeviceToHost, stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            throw std::runtime_error("parameter size copy failed");
        n = n < capacity_ ? n : capacity_;
        std::vector<seedgb_bound_track_parameters> out(n);
        if (n && (cudaMemcpyAsync(out.data(), data.data(), sizeof(out[0]) * n,
                                  cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                  cudaStreamSynchronize(stream) != cudaSuccess))
            throw std::runtime_error("parameter copy failed");
        return out;
    }

    device_buffer<seedgb_bound_track_parameters> data;
    device_buffer<uint32_t> size;

private:
    uint32_t capacity_;
};

/* The parameters in the track finding's record layout, with a device
 * count (bound_track_parameters_collection_types::buffer). */
class ckf_params_buffer {
public:
    explicit ckf_params_buffer(uint32_t capacity) : data(capacity), size(1), capacity_(capacity) {}
    uint32_t capacity() const { return capacity_; }
    std::vector<seedgb_ckf_bound_track_parameters> to_host(cudaStream_t stream) const {
        uint32_t n = 0;
        if (cudaMemcpyAsync(&n, size.data(), sizeof n, cudaMemcpyDeviceToHost, stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            throw std::runtime_error("ckf parameter size copy failed");
        n = n < capacity_ ? n : capacity_;
        std::vector<seedgb_ckf_bound_track_parameters> out(n);
        if (n && (cudaMemcpyAsync(out.data(), data.data(), sizeof(out[0]) * n,
                                  cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                  cudaStreamSynchronize(stream) != cudaSuccess))
            throw std::runtime_error("ckf parameter copy failed");
        return out;
    }

    device_buffer<seedgb_ckf_bound_track_parameters> data;
    device_buffer<uint32_t> size;

private:
    uint32_t capacity_;
};

/* Hands estimated parameters to the track finding: one launch on `stream`,
 * no host synchronisation. */
inline ckf_params_buffer to_ckf(const track_params_buffer& params, cudaStream_t stream) {
    const seedgb_params_buffer in = params.view();
    ckf_params_buffer out(in.capacity);
    check(seedgb_params_to_ckf(&in, out.data.data(), in.capacity, out.size.data(), stream),
          "to_ckf");
    return out;
}

/* Spacepoint collection buffer with room for `capacity` spacepoints and a
 * device count (edm::spacepoint_collection::buffer). */
class spacepoint_collection_buffer {
public:
    explicit spacepoint_collection_buffer(uint32_t capacity)
        : measurement_index_1(capacity), measurement_index_2(capacity), global(3ull * capacity),
          z_variance(capacity), radius_variance(capacity), size(1), capacity_(capacity) {}
    seedgb_spacepoint_buffer buffer() const {
        return seedgb_spacepoint_buffer{measurement_index_1.data(), measurement_index_2.data(),
                                        global.data(), z_variance.data(), radius_variance.data(),
                                        capacity_, size.data()};
    }
    /* A view of the first n spacepoints (n: the count, read back by the caller). */
    seedgb_spacepoint_view view(uint32_t n) const {
        return seedgb_spacepoint_view{measurement_index_1.data(), measurement_index_2.data(),
                                      global.data(), z_variance.data(), radius_variance.data(), n};
    }
    uint32_t count(cudaStream_t stream) const {
        uint32_t n = 0;
        if (cudaMemcpyAsync(&n, size.data(), sizeof n, cudaMemcpyDeviceToHost, stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            throw std::runtime_error("spacepoint count copy failed");
        return n;
    }

    device_buffer<uint32_t> measurement_index_1, measurement_index_2;
    device_buffer<float> global, z_variance, radius_variance;
    device_buffer<uint32_t> size;

private:
    uint32_t capacity_;
};

/* traccc::host::silicon_pixel_spacepoint_formation_algorithm on the device, for
 * many events per call: the surface table uploaded once. */
class spacepoint_formation_algorithm {
public:
    spacepoint_formation_algorithm(const std::vector<seedgb_surface>& surfaces,
                                   cudaStream_t stream)
        : stream_(stream) {
        check(seedgb_formation_create(surfaces.empty() ? nullptr : surfaces.data(),
                                      static_cast<uint32_t>(surfaces.size()), &h_),
              "spacepoint_formation_algorithm");
    }
    spacepoint_formation_algorithm(const spacepoint_formation_algorithm&) = delete;
    spacepoint_formation_algorithm& operator=(const spacepoint_formation_algorithm&) = delete;
    ~spacepoint_formation_algorithm() { seedgb_formation_destroy(h_); }

    /* One buffer per event (room for all its measurements); asynchronous. */
    std::vector<spacepoint_collection_buffer> operator()(
        const std::vector<seedgb_measurement_view>& measurements) const {
        std::vector<spacepoint_collection_buffer> out;
        std::vector<seedgb_spacepoint_buffer> bufs;
        out.reserve(measurements.size());
        for (const auto& m : measurements) {
            out.emplace_back(m.size > 0 ? m.size : 1u);
            bufs.push_back(out.back().buffer());
        }
        if (!measurements.empty())
            check(seedgb_formation_run_batch(h_, measurements.data(), nullptr, bufs.data(),
                                             static_cast<uint32_t>(measurements.size()), stream_),
                  "spacepoint_formation_algorithm()");
        return out;
    }

private:
    cudaStream_t stream_;
    seedgb_formation* h_ = nullptr;
};

/* traccc::cuda::triplet_seeding_algorithm. */
class triplet_seeding_algorithm {
public:
    triplet_seeding_algorithm(const seedgb_seedfinder_config& finder,
                              const seedgb_spacepoint_grid_config& grid,
                              const seedgb_seedfilter_config& filter, cudaStream_t stream)
        : finder_(finder), stream_(stream) {
        check(seedgb_seeding_create(&finder, &grid, &filter, &h_), "triplet_seeding_algorithm");
    }
    triplet_seeding_algorithm(const triplet_seeding_algorithm&) = delete;
    triplet_seeding_algorithm& operator=(const triplet_seeding_algorithm&) = delete;
    ~triplet_seeding_algorithm() { seedgb_seeding_destroy(h_); }

    /* Seeds of one event, in the host seeding's order; asynchronous. */
    seed_collection_buffer operator()(const seedgb_spacepoint_view& spacepoints) const {
        seed_collection_buffer out(capacity(spacepoints.size));
        seedgb_seed_buffer b = out.view();
        check(seedgb_seeding_run(h_, &spacepoints, &b, stream_), "triplet_seeding_algorithm()");
        return out;
    }

    /* Many events in one launch sequence. */
    std::vector<seed_collection_buffer> operator()(
        const std::vector<seedgb_spacepoint_view>& events) const {
        std::vector<seed_collection_buffer> out;
        std::vector<seedgb_seed_buffer> views;
        out.reserve(events.size());
        for (const auto& e : events) {
            out.emplace_back(capacity(e.size));
            views.push_back(out.back().view());
        }
        if (!events.empty())
            check(seedgb_seeding_run_batch(h_, events.data(), static_cast<uint32_t>(events.size()),
                                           views.data(), stream_),
                  "triplet_seeding_algorithm(batch)");
        return out;
    }

    /* Device status of the last call (synchronises the stream). */
    void check_status() const {
        check(seedgb_seeding_last_status(h_, stream_), "triplet_seeding_algorithm status");
    }

    /* Launch-shape search on a representative batch (candidates empty: the
     * library's default grid); leaves the fastest shape set. */
    seedgb_tune autotune(const std::vector<seedgb_spacepoint_view>& events,
                         const std::vector<seedgb_tune>& candidates = {},
                         uint32_t reps = 3) {
        std::vector<seed_collection_buffer> out;
        std::vector<seedgb_seed_buffer> views;
        for (const auto& e : events) {
            out.emplace_back(capacity(e.size));
            views.push_back(out.back().view());
        }
        seedgb_tune best{};
        check(seedgb_seeding_autotune(h_, events.data(), static_cast<uint32_t>(events.size()),
                                      views.data(),
                                      candidates.empty() ? nullptr : candidates.data(),
                                      static_cast<uint32_t>(candidates.size()), reps, &best,
                                      nullptr, stream_),
              "autotune");
        return best;
    }

    /* The learned doublet filter: training on these events' plain seeds,
     * gate calibration on held-out events, installation (nullptr: plain). */
    seedgb_doublet_filter train_filter(const std::vector<seedgb_spacepoint_view>& events,
                                       const std::vector<float>& band_edges,
                                       const seedgb_filter_train_config& cfg) {
        seedgb_doublet_filter f{};
        check(seedgb_filter_train(h_, events.data(), static_cast<uint32_t>(events.size()),
                                  band_edges.data(), static_cast<uint32_t>(band_edges.size()),
                                  &cfg, &f, nullptr, stream_),
              "train_filter");
        return f;
    }
    void calibrate_gate(seedgb_doublet_filter& f, const std::vector<seedgb_spacepoint_view>& events,
                        const std::vector<uint32_t>& class_max, float target, float min_event,
                        float margin = 0.05f) {
        check(seedgb_filter_calibrate_gate(h_, events.data(),
                                           static_cast<uint32_t>(events.size()),
                                           class_max.empty() ? nullptr : class_max.data(),
                                           static_cast<uint32_t>(class_max.size()), target,
                                           min_event, margin, &f, nullptr, nullptr, stream_),
              "calibrate_gate");
    }
    void set_filter(const seedgb_doublet_filter* f) {
        check(seedgb_seeding_set_filter(h_, f), "set_filter");
    }
    seedgb_seeding* handle() const { return h_; }

private:
    uint32_t capacity(uint32_t n_sp) const {
        const uint64_t c = static_cast<uint64_t>(finder_.maxSeedsPerSpM) * n_sp;
        return static_cast<uint32_t>(c > 0 ? (c < 0xFFFFFFFFull ? c : 0xFFFFFFFFull) : 1);
    }
    seedgb_seedfinder_config finder_;
    cudaStream_t stream_;
    seedgb_seeding* h_ = nullptr;
};

/* traccc::cuda::seed_parameter_estimation_algorithm (constant field). */
/* traccc::gbts_seedfinder_config before setLinkingScheme: the parameters and
 * the linking inputs (bin tables unrolled to pairs, layer table, geometry-id
 * binning, minimum pT in MeV, optional tau table). */
struct gbts_seedfinder_config {
    seedgb_gbts_config params{};
    std::vector<seedgb_gbts_layer> layers;
    std::vector<uint32_t> bin_pairs;  // (bin1, bin2) per linked pair
    std::vector<seedgb_gbts_geoid> geoid_binning;
    float min_pt = 900.0f;
    std::vector<float> tau_lut;

    gbts_seedfinder_config() { seedgb_gbts_config_default(&params); }

    /* geoidBinning.txt, binTables.txt and layerInfo.txt of `dir`. */
    static gbts_seedfinder_config from_directory(const std::string& dir, float min_pt = 900.0f) {
        gbts_seedfinder_config c;
        c.min_pt = min_pt;
        uint32_t nl = 0, np = 0, ng = 0;
        check(seedgb_gbts_read_config_dir(dir.c_str(), nullptr, &nl, nullptr, &np, nullptr, &ng),
              "gbts_seedfinder_config::from_directory");
        c.layers.resize(nl);
        c.bin_pairs.resize(2ull * np);
        c.geoid_binning.resize(ng);
        check(seedgb_gbts_read_config_dir(dir.c_str(), c.layers.data(), &nl, c.bin_pairs.data(), &np,
                                          c.geoid_binning.data(), &ng),
              "gbts_seedfinder_config::from_directory");
        return c;
    }
};

/* traccc::cuda::gbts_seeding_algorithm.  The measurements enter as their
 * device columns: surface barcode and cluster diameter. */
class gbts_seeding_algorithm {
public:
    gbts_seeding_algorithm(const gbts_seedfinder_config& cfg, cudaStream_t stream)
        : stream_(stream) {
        check(seedgb_gbts_create(&cfg.params, cfg.layers.data(), static_cast<uint32_t>(cfg.layers.size()),
                                 cfg.bin_pairs.data(), static_cast<uint32_t>(cfg.bin_pairs.size() / 2),
                                 cfg.geoid_binning.data(),
                                 static_cast<uint32_t>(cfg.geoid_binning.size()), cfg.min_pt,
                                 cfg.tau_lut.empty() ? nullptr : cfg.tau_lut.data(),
                                 static_cast<uint32_t>(cfg.tau_lut.size()), &h_),
              "gbts_seeding_algorithm");
    }
    gbts_seeding_algorithm(const gbts_seeding_algorithm&) = delete;
    gbts_seeding_algorithm& operator=(const gbts_seeding_algorithm&) = delete;
    ~gbts_seeding_algorithm() { seedgb_gbts_destroy(h_); }

    seed_collection_buffer operator()(const seedgb_spacepoint_view& spacepoints,
                                      const uint64_t* surface_link, const float* diameter,
                                      uint32_t n_measurements) const {
        seed_collection_buffer out(3u * (spacepoints.size ? spacepoints.size : 1u));
        seedgb_seed_buffer b = out.view();
        check(seedgb_gbts_run(h_, &spacepoints, surface_link, diameter, n_measurements, &b, stream_),
              "gbts_seeding_algorithm()");
        return out;
    }

    /* Many events in one call (seedgb_gbts_run_batch); element e of each
     * vector is event e. */
    std::vector<seed_collection_buffer> operator()(
        const std::vector<seedgb_spacepoint_view>& spacepoints,
        const std::vector<const uint64_t*>& surface_links, const std::vector<const float*>& diameters,
        const std::vector<uint32_t>& n_measurements) const {
        const std::size_t n = spacepoints.size();
        if (surface_links.size() != n || diameters.size() != n || n_measurements.size() != n)
            throw std::invalid_argument("gbts_seeding_algorithm(batch): sizes");
        std::vector<seed_collection_buffer> out;
        std::vector<seedgb_seed_buffer> bufs;
        out.reserve(n);
        for (const auto& sp : spacepoints) {
            out.emplace_back(3u * (sp.size ? sp.size : 1u));
            bufs.push_back(out.back().view());
        }
        if (n)
            check(seedgb_gbts_run_batch(h_, spacepoints.data(), surface_links.data(), diameters.data(),
                                        n_measurements.data(), static_cast<uint32_t>(n), bufs.data(),
                                        stream_),
                  "gbts_seeding_algorithm(batch)");
        return out;
    }

    /* Device status of the last call (synchronises the stream). */
    seedgb_status status() const { return seedgb_gbts_last_status(h_, stream_); }

    std::array<uint64_t, SEEDGB_GBTS_N_COUNTERS> counters() const {
        std::array<uint64_t, SEEDGB_GBTS_N_COUNTERS> c{};
        check(seedgb_gbts_counters(h_, c.data()), "gbts_seeding_algorithm::counters");
        return c;
    }

private:
    seedgb_gbts* h_ = nullptr;
    cudaStream_t stream_;
};

class seed_parameter_estimation_algorithm {
public:
    seed_parameter_estimation_algorithm(const seedgb_track_params_estimation_config& cfg,
                                        cudaStream_t stream)
        : stream_(stream) {
        check(seedgb_params_create(&cfg, &h_), "seed_parameter_estimation_algorithm");
    }
    seed_parameter_estimation_algorithm(const seed_parameter_estimation_algorithm&) = delete;
    seed_parameter_estimation_algorithm& operator=(const seed_parameter_estimation_algorithm&) =
        delete;
    ~seed_parameter_estimation_algorithm() { seedgb_params_destroy(h_); }

    track_params_buffer operator()(const std::array<float, 3>& bfield,
                                   const seedgb_measurement_view& measurements,
                                   const seedgb_spacepoint_view& spacepoints,
                                   const seed_collection_buffer& seeds) const {
        track_params_buffer out(seeds.capacity());
        seedgb_seed_buffer s = seeds.view();
        seedgb_params_buffer p = out.view();
        check(seedgb_params_run(h_, bfield.data(), &measurements, &spacepoints, &s, &p, stream_),
              "seed_parameter_estimation_algorithm()");
        return out;
    }

    /* Many events in one launch (element e of each vector is event e). */
    std::vector<track_params_buffer> operator()(
        const std::array<float, 3>& bfield,
        const std::vector<seedgb_measurement_view>& measurements,
        const std::vector<seedgb_spacepoint_view>& spacepoints,
        const std::vector<seed_collection_buffer>& seeds) const {
        if (measurements.size() != seeds.size() || spacepoints.size() != seeds.size())
            throw std::invalid_argument("seed_parameter_estimation_algorithm(batch): sizes");
        std::vector<track_params_buffer> out;
        std::vector<seedgb_seed_buffer> sv;
        std::vector<seedgb_params_buffer> pv;
        out.reserve(seeds.size());
        for (const auto& sb : seeds) {
            out.emplace_back(sb.capacity());
            sv.push_back(sb.view());
            pv.push_back(out.back().view());
        }
        if (!seeds.empty())
            check(seedgb_params_run_batch(h_, bfield.data(), measurements.data(),
                                          spacepoints.data(), sv.data(), pv.data(),
                                          static_cast<uint32_t>(seeds.size()), stream_),
                  "seed_parameter_estimation_algorithm(batch)");
        return out;
    }

private:
    cudaStream_t stream_;
    seedgb_params* h_ = nullptr;
};

}  // namespace seedgb

#endif
