// A C++ caller of GBTS seeding through include/seedgb.hpp, configured the way
// traccc's examples configure it: the configuration directory read by
// gbts_seedfinder_config::from_directory (geoidBinning.txt, binTables.txt,
// layerInfo.txt), then operator()(spacepoints, measurements).  For the GPU
// test in tests/test_gpu_cpp_adapter.py.
//
//   gbts_check <config dir> <in.bin> <out.bin>
//
// in.bin: uint32 n_sp, uint32 n_meas, u32 measurement_index_1[n_sp],
//   f32 global[3 n_sp], u64 surface_link[n_meas], f32 diameter[n_meas]
// out.bin: uint32 n_seeds, seeds {u32 b, m, t; f32 q}[n_seeds]
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

template <typename T>
static T* to_device(const std::vector<T>& v) {
    T* p = nullptr;
    if (cudaMalloc(&p, sizeof(T) * (v.empty() ? 1 : v.size())) != cudaSuccess) std::exit(3);
    if (!v.empty() && cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        std::exit(3);
    return p;
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    std::FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 2;
    uint32_t n_sp = 0, n_meas = 0;
    if (std::fread(&n_sp, 4, 1, f) != 1 || std::fread(&n_meas, 4, 1, f) != 1) return 2;
    const auto mi = read_vec<uint32_t>(f, n_sp);
    const auto glob = read_vec<float>(f, 3ull * n_sp);
    const auto link = read_vec<uint64_t>(f, n_meas);
    const auto diam = read_vec<float>(f, n_meas);
    std::fclose(f);
    const std::vector<uint32_t> invalid(n_sp, SEEDGB_INVALID_MEASUREMENT_INDEX);
    const std::vector<float> zeros(n_sp, 0.0f);
    uint32_t* d_mi = to_device(mi);
    uint32_t* d_mi2 = to_device(invalid);
    float* d_g = to_device(glob);
    float* d_z = to_device(zeros);
    uint64_t* d_link = to_device(link);
    float* d_diam = to_device(diam);
    cudaStream_t stream;
    cudaStreamCreate(&stream);
    int rc = 0;
    try {
        seedgb::gbts_seedfinder_config cfg = seedgb::gbts_seedfinder_config::from_directory(argv[1]);
        seedgb::gbts_seeding_algorithm gbts(cfg, stream);
        const seedgb_spacepoint_view view{d_mi, d_mi2, d_g, d_z, d_z, n_sp};
        const auto seeds_buf = gbts(view, d_link, d_diam, n_meas);
        if (gbts.status() != SEEDGB_OK) throw std::runtime_error("gbts status");
        const auto seeds = seeds_buf.to_host(stream);
        std::FILE* o = std::fopen(argv[3], "wb");
        const uint32_t ns = static_cast<uint32_t>(seeds.size());
        std::fwrite(&ns, 4, 1, o);
        if (ns) std::fwrite(seeds.data(), sizeof(seedgb::seed), ns, o);
        std::fclose(o);
        // a configuration directory that does not exist is an error, not a crash
        bool threw = false;
        try {
            (void)seedgb::gbts_seedfinder_config::from_directory(std::string(argv[1]) + "/missing");
        } catch (const std::runtime_error&) {
            threw = true;
        }
        if (!threw) throw std::runtime_error("missing directory accepted");
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        rc = 1;
    }
    cudaFree(d_mi);
    cudaFree(d_mi2);
    cudaFree(d_g);
    cudaFree(d_z);
    cudaFree(d_link);
    cudaFree(d_diam);
    cudaStreamDestroy(stream);
    return rc;
}
