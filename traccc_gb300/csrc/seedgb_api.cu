// C-ABI layer of the seeding library: handles, the device work arena and the
// launch sequence.  No call here blocks on the device except the explicit
// status query and arena (re)allocation, which happens only when a batch is
// larger than anything reserved before.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "seedgb.h"
#include "seedgb_internal.h"

using namespace seedgb;

// Pinned host copy of what a launch sequence reads first: the batch header
// (kHdrBytes) followed by the event descriptors, copied to the device in one
// transfer.  `done` is recorded after the transfer that reads it.
constexpr size_t kHdrBytes = 256;

struct Staging {
    uint8_t* host = nullptr;
    uint32_t cap = 0;
    cudaEvent_t done = nullptr;
    BatchHeader* hdr() { return reinterpret_cast<BatchHeader*>(host); }
    EventDesc* desc() { return reinterpret_cast<EventDesc*>(host + kHdrBytes); }
};

struct seedgb_seeding {
    seedgb_seedfinder_config finder;
    seedgb_spacepoint_grid_config grid;
    seedgb_seedfilter_config filter;
    seedgb_grid_axes axes;
    DevConfig dc;
    TuneParams tune;
    int device = 0;
    int num_sms = 0;
    // arena
    void* arena = nullptr;
    size_t arena_bytes = 0;
    uint32_t cap_events = 0;
    uint64_t cap_sp = 0;
    uint32_t cap_chunks = 0;
    Arena a{};
    // staging[0]: direct runs; staging[1], staging[2]: the two graph slots
    Staging staging[3];
    // captured launch sequences (two, alternating, so that the host fills one
    // slot's descriptors while the other slot's graph runs)
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    uint32_t g_events = 0;      // capacity the graphs were captured for
    uint64_t g_sp = 0;
    bool g_valid = false;
    int g_next = 0;
    cudaStream_t cap_stream = nullptr;
    unsigned long long h_counters[kNumCounters] = {};
    // learned doublet filter (device copy of the packed network) and dump
    void* d_mlp = nullptr;
    void* dump = nullptr;
    uint64_t dump_cap = 0;
    void* tdump = nullptr;
    uint64_t tdump_cap = 0;
    bool timing = false;
    bool timed_run = false;
    cudaEvent_t tev[kNumKernels + 1] = {};
};

// Descriptors of a batched parameter estimation: pinned host copy and
// device copy, two slots used in turn so that the host fills one while the
// previous call's copy of the other may still be in flight.
struct ParamsSlot {
    seedgb::ParamsEvent* host = nullptr;
    seedgb::ParamsEvent* dev = nullptr;
    uint32_t cap = 0;
    cudaEvent_t copied = nullptr;
};

struct seedgb_params {
    ParamsConfig pc;
    int num_sms = 0;
    ParamsSlot slot[2];
    int next = 0;
    ~seedgb_params() {
        for (auto& s : slot) {
            if (s.copied) cudaEventDestroy(s.copied);
            if (s.host) cudaFreeHost(s.host);
            if (s.dev) cudaFree(s.dev);
        }
    }
};

namespace seedgb {

DevConfig make_dev_config(const seedgb_seedfinder_config& f,
                          const seedgb_seedfilter_config& fl,
                          const seedgb_grid_axes& ax) {
    DevConfig d{};
    d.zMin = f.zMin;
    d.zMax = f.zMax;
    d.phiMin = f.phiMin;
    d.phiMax = f.phiMax;
    d.beam0 = f.beamPos[0];
    d.beam1 = f.beamPos[1];
    // seedfinder_config::get_num_rbins(), seeding_config.hpp:111-113
    const float nr = f.rMax + std::sqrt(f.beamPos[0] * f.beamPos[0] +
                                        f.beamPos[1] * f.beamPos[1]);
    d.nrbins = (nr >= 0.f && nr < 1.8e19f) ? static_cast<unsigned long long>(nr) : 0ull;
    d.deltaRMin = f.deltaRMin;
    d.deltaRMax = f.deltaRMax;
    d.cotThetaMax = f.cotThetaMax;
    d.collisionRegionMin = f.collisionRegionMin;
    d.collisionRegionMax = f.collisionRegionMax;
    d.deltaZMax = f.deltaZMax;
    d.impactMax = f.impactMax;
    d.minHelixRadius = f.minHelixRadius;
    d.maxScatteringAngle2 = f.maxScatteringAngle2;
    d.sigmaScattering = f.sigmaScattering;
    d.minHelixDiameter2 = f.minHelixDiameter2;
    d.pT2perRadius = f.pT2perRadius;
    d.pTPerHelixRadius = f.pTPerHelixRadius;
    d.maxPtScattering = f.maxPtScattering;
    d.highland = f.highland;
    d.maxSeedsPerSpM = f.maxSeedsPerSpM;
    d.scope0 = f.neighbor_scope[0];
    d.scope1 = f.neighbor_scope[1];
    d.deltaInvHelixDiameter = fl.deltaInvHelixDiameter;
    d.impactWeightFactor = fl.impactWeightFactor;
    d.compatSeedWeight = fl.compatSeedWeight;
    d.filterDeltaRMin = fl.deltaRMin;
    d.compatSeedLimit = static_cast<uint32_t>(fl.compatSeedLimit);
    d.good_spB_min_radius = fl.good_spB_min_radius;
    d.good_spB_weight_increase = fl.good_spB_weight_increase;
    d.good_spT_max_radius = fl.good_spT_max_radius;
    d.good_spT_weight_increase = fl.good_spT_weight_increase;
    d.good_spB_min_weight = fl.good_spB_min_weight;
    d.seed_min_weight = fl.seed_min_weight;
    d.spB_min_radius = fl.spB_min_radius;
    d.phi_bins = ax.phi_bins;
    d.z_bins = ax.z_bins;
    d.nbins = ax.phi_bins * ax.z_bins;
    d.phi_min = ax.phi_min;
    d.phi_max = ax.phi_max;
    d.z_min = ax.z_min;
    d.z_max = ax.z_max;
    d.brute_force_triplets = 0;
    d.last_tier_only = 0;
    d.mlp = nullptr;
    d.band_lo = 0.f;
    d.band_hi = 1.f;
    d.mlp_n_classes = 0;
    return d;
}

}  // namespace seedgb

namespace {

seedgb_status cuda_status(cudaError_t e) {
    return e == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}

size_t align_up(size_t v, size_t a = 256) { return (v + a - 1) / a * a; }

// Longest phi zone over all phi bins (circular::zone_t semantics).
uint32_t max_phi_zone(uint32_t n, uint32_t s0, uint32_t s1) {
    auto remap = [n](uint32_t ibin, int sh) -> uint32_t {
        const int opt = static_cast<int>(ibin) + sh;
        if (opt >= 0 && opt < static_cast<int>(n)) return static_cast<uint32_t>(opt);
        if (opt < 0) return static_cast<uint32_t>(static_cast<int>(n) + opt);
        return static_cast<uint32_t>(opt) - n;
    };
    uint32_t mx = 0;
    for (uint32_t b = 0; b < n; ++b) {
        const uint32_t lo = remap(b, -static_cast<int>(s0)), hi = remap(b, static_cast<int>(s1));
        const uint32_t len = lo < hi ? hi - lo + 1u : n - lo + hi + 1u;
        mx = std::max(mx, len);
    }
    return mx;
}

uint32_t chunks_of(uint32_t n_sp) { return (n_sp + kBinChunk - 1) / kBinChunk; }

uint32_t chunk_capacity(uint32_t events, uint64_t sp) {
    return static_cast<uint32_t>(sp / kBinChunk) + events;
}

uint32_t item_capacity(uint32_t events, uint64_t sp, uint32_t nb, uint32_t mpi) {
    return static_cast<uint32_t>(sp / mpi) + events * nb + 1;
}

void drop_graphs(seedgb_seeding* h) {
    for (auto& g : h->gexec) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
    h->g_valid = false;
}

seedgb_status ensure_staging(Staging& st, uint32_t events) {
    if (!st.done && cudaEventCreateWithFlags(&st.done, cudaEventDisableTiming) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    if (st.cap >= events) return SEEDGB_OK;
    if (cudaEventSynchronize(st.done) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    if (st.host) cudaFreeHost(st.host);
    st.host = nullptr;
    st.cap = 0;
    const size_t bytes = kHdrBytes + sizeof(EventDesc) * events;
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    std::memset(p, 0, bytes);
    st.host = static_cast<uint8_t*>(p);
    st.cap = events;
    return SEEDGB_OK;
}

// Size the arena for a batch; reallocation (which drops the captured graphs)
// only when the batch does not fit what is there.
seedgb_status ensure_arena(seedgb_seeding* h, uint32_t n_events, uint64_t total_sp,
                           uint32_t total_chunks) {
    const uint32_t nb = h->dc.nbins;
    const uint32_t mpi = static_cast<uint32_t>(h->tune.middles_per_item);
    if (h->arena && n_events <= h->cap_events && total_sp <= h->cap_sp &&
        total_chunks <= h->cap_chunks &&
        item_capacity(h->cap_events, h->cap_sp, nb, mpi) <= h->a.max_items)
        return ensure_staging(h->staging[0], h->cap_events);
    const uint32_t ce = std::max(n_events, h->cap_events);
    const uint64_t cs = std::max<uint64_t>(std::max<uint64_t>(total_sp, h->cap_sp), 1);
    if (cs > 0xF0000000ull) return SEEDGB_UNSUPPORTED;
    const uint32_t cc = std::max(chunk_capacity(ce, cs), total_chunks);
    const uint32_t ci = item_capacity(ce, cs, nb, mpi);
    size_t off = 0;
    auto take = [&off](size_t bytes) { const size_t o = off; off = align_up(off + bytes); return o; };
    const size_t o_hdr = take(kHdrBytes);
    const size_t o_events = take(sizeof(EventDesc) * ce);
    const size_t o_spbin = take(sizeof(int32_t) * cs);
    const size_t o_whist = take(sizeof(uint32_t) * static_cast<size_t>(cc) * kBinWarps * nb);
    const size_t o_bs = take(sizeof(uint32_t) * static_cast<size_t>(ce) * (nb + 1));
    const size_t o_nv = take(sizeof(uint32_t) * ce);
    const size_t o_xyzr = take(sizeof(float4) * cs);
    const size_t o_var = take(sizeof(float2) * cs);
    const size_t o_idx = take(sizeof(uint32_t) * cs);
    const size_t o_rs = take(sizeof(float4) * cs);
    const size_t o_rsgp = take(sizeof(uint32_t) * cs);
    const size_t o_uns = take(sizeof(uint8_t) * static_cast<size_t>(ce) * nb);
    const size_t o_items = take(sizeof(uint2) * ci);
    const size_t o_ikey = take(sizeof(uint8_t) * ci);
    const size_t o_iord = take(sizeof(uint2) * ci);
    const size_t o_cnt = take(sizeof(uint8_t) * cs);
    const size_t o_slot = take(sizeof(SeedSlot) * cs * kMaxSeedsPerMiddle);
    const size_t o_cseeds = take(sizeof(uint32_t) * static_cast<size_t>(cc));
    const size_t o_ovf = take(sizeof(uint32_t) * cs * 2);
    const size_t o_ovf2 = take(sizeof(uint32_t) * cs * 2);
    // the counters and the work-item order histogram are zeroed together
    const size_t o_ctr = take(kCounterBytes);
    const size_t o_evf = take(sizeof(uint32_t) * 4 * static_cast<size_t>(ce));
    const size_t o_evm = take(sizeof(uint8_t) * static_cast<size_t>(ce));
    static_assert(kHdrBytes >= sizeof(BatchHeader) && kHdrBytes % 256 == 0,
                  "the descriptors follow the header directly");
    drop_graphs(h);
    if (h->arena) {
        // in-flight work of this handle may still use the old arena
        if (cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
        cudaFree(h->arena);
        h->arena = nullptr;
    }
    void* p = nullptr;
    if (cudaMalloc(&p, off) != cudaSuccess) {
        h->cap_events = 0;
        h->cap_sp = 0;
        h->cap_chunks = 0;
        return SEEDGB_CUDA_ERROR;
    }
    h->arena = p;
    h->arena_bytes = off;
    h->cap_events = ce;
    h->cap_sp = cs;
    h->cap_chunks = cc;
    char* base = static_cast<char*>(p);
    Arena& a = h->a;
    a.hdr = reinterpret_cast<BatchHeader*>(base + o_hdr);
    a.events = reinterpret_cast<EventDesc*>(base + o_events);
    a.sp_bin = reinterpret_cast<int32_t*>(base + o_spbin);
    a.whist = reinterpret_cast<uint32_t*>(base + o_whist);
    a.bin_start = reinterpret_cast<uint32_t*>(base + o_bs);
    a.n_valid = reinterpret_cast<uint32_t*>(base + o_nv);
    a.g_xyzr = reinterpret_cast<float4*>(base + o_xyzr);
    a.g_var = reinterpret_cast<float2*>(base + o_var);
    a.g_idx = reinterpret_cast<uint32_t*>(base + o_idx);
    a.g_rs = reinterpret_cast<float4*>(base + o_rs);
    a.g_rs_gp = reinterpret_cast<uint32_t*>(base + o_rsgp);
    a.bin_unsorted = reinterpret_cast<uint8_t*>(base + o_uns);
    a.items = reinterpret_cast<uint2*>(base + o_items);
    a.item_key = reinterpret_cast<uint8_t*>(base + o_ikey);
    a.items_ord = reinterpret_cast<uint2*>(base + o_iord);
    a.seed_cnt = reinterpret_cast<uint8_t*>(base + o_cnt);
    a.seed_slot = reinterpret_cast<SeedSlot*>(base + o_slot);
    a.chunk_seeds = reinterpret_cast<uint32_t*>(base + o_cseeds);
    a.ovf = reinterpret_cast<uint32_t*>(base + o_ovf);
    a.ovf2 = reinterpret_cast<uint32_t*>(base + o_ovf2);
    a.counters = reinterpret_cast<unsigned long long*>(base + o_ctr);
    a.order_hist = reinterpret_cast<uint32_t*>(base + o_ctr +
                                               sizeof(unsigned long long) * kNumCounters);
    a.ev_filter = reinterpret_cast<uint32_t*>(base + o_evf);
    a.ev_mode = reinterpret_cast<uint8_t*>(base + o_evm);
    a.dump = h->dump;
    a.dump_cap = h->dump_cap;
    a.tdump = static_cast<uint4*>(h->tdump);
    a.tdump_cap = h->tdump_cap;
    a.cap_events = ce;
    a.cap_chunks = cc;
    a.cap_sp = static_cast<uint32_t>(cs);
    a.max_items = ci;
    return ensure_staging(h->staging[0], ce);
}

// Validates a batch and writes its header and descriptors into `st`
// (which the caller has waited for).
seedgb_status stage_batch(Staging& st, const seedgb_spacepoint_view* events, uint32_t n_events,
                          const seedgb_seed_buffer* outs) {
    uint32_t sp_base = 0, chunk_base = 0;
    for (uint32_t e = 0; e < n_events; ++e) {
        const seedgb_spacepoint_view& v = events[e];
        EventDesc& d = st.desc()[e];
        d.mi1 = v.measurement_index_1;
        d.mi2 = v.measurement_index_2;
        d.global = v.global;
        d.zvar = v.z_variance;
        d.rvar = v.radius_variance;
        d.n_sp = v.size;
        d.sp_base = sp_base;
        d.chunk_base = chunk_base;
        d.n_chunks = chunks_of(v.size);
        d.out_b = outs[e].bottom_index;
        d.out_m = outs[e].middle_index;
        d.out_t = outs[e].top_index;
        d.out_q = outs[e].quality;
        d.out_cap = outs[e].capacity;
        d.pad = 0;
        d.out_size = outs[e].size;
        sp_base += v.size;
        chunk_base += d.n_chunks;
    }
    BatchHeader& hb = *st.hdr();
    hb.n_events = n_events;
    hb.total_chunks = chunk_base;
    hb.total_sp = sp_base;
    hb.pad = 0;
    return SEEDGB_OK;
}

// Checks the arguments of a batch and sums its sizes.
seedgb_status check_batch(const seedgb_spacepoint_view* events, uint32_t n_events,
                          const seedgb_seed_buffer* outs, uint64_t* total_sp,
                          uint32_t* total_chunks) {
    if (!events || !outs || n_events == 0) return SEEDGB_INVALID_ARGUMENT;
    if (n_events > kMaxEventsPerBatch) return SEEDGB_UNSUPPORTED;
    uint64_t sp = 0;
    uint64_t chunks = 0;
    for (uint32_t e = 0; e < n_events; ++e) {
        const seedgb_spacepoint_view& v = events[e];
        if (v.size > 0 && !v.global) return SEEDGB_INVALID_ARGUMENT;
        if (!outs[e].size || (outs[e].capacity > 0 &&
                              (!outs[e].bottom_index || !outs[e].middle_index ||
                               !outs[e].top_index || !outs[e].quality)))
            return SEEDGB_INVALID_ARGUMENT;
        sp += v.size;
        chunks += chunks_of(v.size);
    }
    if (sp > 0xF0000000ull) return SEEDGB_UNSUPPORTED;
    *total_sp = sp;
    *total_chunks = static_cast<uint32_t>(chunks);
    return SEEDGB_OK;
}

// Enqueues header + descriptor copy, counter reset and the kernels.
// copied: recorded once the staging buffer has been read (nullptr: none).
cudaError_t enqueue_batch(seedgb_seeding* h, Staging& st, uint32_t staged_events,
                          const BatchHeader& grid, cudaStream_t s, cudaEvent_t copied,
                          cudaEvent_t* timing) {
    cudaError_t err = cudaMemcpyAsync(h->a.hdr, st.host,
                                      kHdrBytes + sizeof(EventDesc) * staged_events,
                                      cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess && copied) err = cudaEventRecord(copied, s);
    if (err == cudaSuccess)
        err = cudaMemsetAsync(h->a.counters, 0, kCounterBytes, s);
    if (err == cudaSuccess && h->dc.mlp)
        err = cudaMemsetAsync(h->a.ev_filter, 0, sizeof(uint32_t) * 4 * grid.n_events, s);
    if (err == cudaSuccess)
        err = launch_seeding(h->dc, h->a, grid, h->tune, h->num_sms, s, timing);
    return err;
}

// Captures the two graph slots for batches up to h->g_events / h->g_sp.
seedgb_status capture_graphs(seedgb_seeding* h) {
    drop_graphs(h);
    const uint32_t ce = h->g_events;
    const uint64_t cs = h->g_sp;
    seedgb_status st = ensure_arena(h, ce, cs, chunk_capacity(ce, cs));
    if (st != SEEDGB_OK) return st;
    if (!h->cap_stream &&
        cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    if (prepare_kernels() != cudaSuccess) return SEEDGB_CUDA_ERROR;
    const BatchHeader grid{ce, chunk_capacity(ce, cs), static_cast<uint32_t>(cs), 0};
    for (int k = 0; k < 2; ++k) {
        Staging& sg = h->staging[1 + k];
        st = ensure_staging(sg, ce);
        if (st != SEEDGB_OK) return st;
        cudaGraph_t g = nullptr;
        cudaError_t err = cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) {
            const cudaError_t e1 = enqueue_batch(h, sg, ce, grid, h->cap_stream, nullptr, nullptr);
            err = cudaStreamEndCapture(h->cap_stream, &g);
            if (e1 != cudaSuccess) err = e1;
        }
        if (err == cudaSuccess) err = cudaGraphInstantiate(&h->gexec[k], g, 0);
        if (g) cudaGraphDestroy(g);
        if (err != cudaSuccess) {
            drop_graphs(h);
            return SEEDGB_CUDA_ERROR;
        }
    }
    h->g_valid = true;
    h->g_next = 0;
    return SEEDGB_OK;
}

}  // namespace

extern "C" {

seedgb_status seedgb_seeding_create(const seedgb_seedfinder_config* finder,
                                    const seedgb_spacepoint_grid_config* grid,
                                    const seedgb_seedfilter_config* filter,
                                    seedgb_seeding** out) {
    if (!finder || !grid || !filter || !out) return SEEDGB_INVALID_ARGUMENT;
    *out = nullptr;
    seedgb_grid_axes ax;
    const seedgb_status st = seedgb_get_axes(grid, &ax);
    if (st != SEEDGB_OK) return st;
    const uint64_t nbins = static_cast<uint64_t>(ax.phi_bins) * ax.z_bins;
    if (ax.phi_bins == 0 || nbins > static_cast<uint64_t>(kMaxBins)) return SEEDGB_UNSUPPORTED;
    if (finder->neighbor_scope[0] >= ax.phi_bins || finder->neighbor_scope[1] >= ax.phi_bins)
        return SEEDGB_UNSUPPORTED;
    const uint32_t zl = std::min<uint32_t>(ax.z_bins,
                                           finder->neighbor_scope[0] + finder->neighbor_scope[1] + 1);
    if (static_cast<uint64_t>(max_phi_zone(ax.phi_bins, finder->neighbor_scope[0],
                                           finder->neighbor_scope[1])) * zl >
        static_cast<uint64_t>(kMaxSegments))
        return SEEDGB_UNSUPPORTED;
    if (finder->maxSeedsPerSpM > kMaxSeedsPerMiddle) return SEEDGB_UNSUPPORTED;
    if (filter->compatSeedLimit > 8) return SEEDGB_UNSUPPORTED;

    seedgb_seeding* h = new (std::nothrow) seedgb_seeding();
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    h->finder = *finder;
    h->grid = *grid;
    h->filter = *filter;
    h->axes = ax;
    h->dc = make_dev_config(*finder, *filter, ax);
    if (cudaGetDevice(&h->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device) !=
            cudaSuccess ||
        ensure_staging(h->staging[0], 1) != SEEDGB_OK) {
        seedgb_seeding_destroy(h);
        return SEEDGB_CUDA_ERROR;
    }
    h->tune.fast_warps = 16;  // clamped below to what fits in shared memory
    h->tune.middles_per_item = 256;
    h->tune.nb_cap = 2048;
    h->tune.ctas_per_sm = 1;
    if (const char* s = std::getenv("SEEDGB_TUNE")) {
        int w, m, nb, c;
        if (std::sscanf(s, "%d,%d,%d,%d", &w, &m, &nb, &c) == 4 && w >= 1 && w <= 16 &&
            m >= 1 && m <= 4096 && nb >= 256 && nb <= 8192 && c >= 1 && c <= 8) {
            h->tune = TuneParams{w, m, nb, c};
        }
    }
    const int mw = fast_kernel_max_warps(h->tune.nb_cap, h->tune.ctas_per_sm);
    if (mw < 1) {
        seedgb_seeding_destroy(h);
        return SEEDGB_UNSUPPORTED;
    }
    h->tune.fast_warps = std::min(h->tune.fast_warps, mw);
    *out = h;
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_destroy(seedgb_seeding* h) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    drop_graphs(h);
    if (h->arena) {
        cudaDeviceSynchronize();
        cudaFree(h->arena);
    }
    for (auto& st : h->staging) {
        if (st.done) {
            cudaEventSynchronize(st.done);
            cudaEventDestroy(st.done);
        }
        if (st.host) cudaFreeHost(st.host);
    }
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    if (h->d_mlp) cudaFree(h->d_mlp);
    for (auto& e : h->tev)
        if (e) cudaEventDestroy(e);
    delete h;
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_reserve(seedgb_seeding* h, uint32_t max_events,
                                     uint64_t max_total_spacepoints) {
    if (!h || max_events == 0) return SEEDGB_INVALID_ARGUMENT;
    if (max_total_spacepoints > 0xF0000000ull) return SEEDGB_UNSUPPORTED;
    return ensure_arena(h, max_events, max_total_spacepoints,
                        chunk_capacity(max_events, max_total_spacepoints));
}

seedgb_status seedgb_seeding_run_batch(seedgb_seeding* h, const seedgb_spacepoint_view* events,
                                       uint32_t n_events, seedgb_seed_buffer* outs,
                                       void* stream) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    uint64_t total_sp = 0;
    uint32_t total_chunks = 0;
    seedgb_status st = check_batch(events, n_events, outs, &total_sp, &total_chunks);
    if (st != SEEDGB_OK) return st;
    st = ensure_arena(h, n_events, total_sp, total_chunks);
    if (st != SEEDGB_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Staging& sg = h->staging[0];
    // the staging buffer may still feed the previous call's copy
    if (cudaEventSynchronize(sg.done) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    stage_batch(sg, events, n_events, outs);
    const BatchHeader grid = *sg.hdr();
    const cudaError_t err =
        enqueue_batch(h, sg, n_events, grid, s, sg.done, h->timing ? h->tev : nullptr);
    h->timed_run = h->timing && err == cudaSuccess;
    return cuda_status(err);
}

seedgb_status seedgb_seeding_graph_create(seedgb_seeding* h, uint32_t max_events,
                                          uint64_t max_total_spacepoints) {
    if (!h || max_events == 0 || max_events > kMaxEventsPerBatch)
        return SEEDGB_INVALID_ARGUMENT;
    if (max_total_spacepoints > 0xF0000000ull) return SEEDGB_UNSUPPORTED;
    h->g_events = max_events;
    h->g_sp = std::max<uint64_t>(max_total_spacepoints, 1);
    return capture_graphs(h);
}

seedgb_status seedgb_seeding_graph_launch(seedgb_seeding* h,
                                          const seedgb_spacepoint_view* events,
                                          uint32_t n_events, seedgb_seed_buffer* outs,
                                          void* stream) {
    if (!h || h->g_events == 0) return SEEDGB_INVALID_ARGUMENT;
    uint64_t total_sp = 0;
    uint32_t total_chunks = 0;
    seedgb_status st = check_batch(events, n_events, outs, &total_sp, &total_chunks);
    if (st != SEEDGB_OK) return st;
    if (n_events > h->g_events || total_sp > h->g_sp) return SEEDGB_SIZE_LIMIT;
    if (!h->g_valid) {
        // a configuration change or a larger direct run replaced the arena
        st = capture_graphs(h);
        if (st != SEEDGB_OK) return st;
    }
    const int k = h->g_next;
    Staging& sg = h->staging[1 + k];
    if (cudaEventSynchronize(sg.done) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    stage_batch(sg, events, n_events, outs);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t err = cudaGraphLaunch(h->gexec[k], s);
    if (err == cudaSuccess) err = cudaEventRecord(sg.done, s);
    h->g_next = k ^ 1;
    h->timed_run = false;
    return cuda_status(err);
}

seedgb_status seedgb_seeding_set_tune(seedgb_seeding* h, const seedgb_tune* t) {
    if (!h || !t) return SEEDGB_INVALID_ARGUMENT;
    if (t->warps_per_cta < 1 || t->warps_per_cta > 16 || t->middles_per_item < 1 ||
        t->middles_per_item > 4096 || t->neighbourhood_capacity < 256 ||
        t->neighbourhood_capacity > 8192 || t->ctas_per_sm < 1 || t->ctas_per_sm > 8)
        return SEEDGB_INVALID_ARGUMENT;
    const int mw = fast_kernel_max_warps(t->neighbourhood_capacity, t->ctas_per_sm);
    if (mw < 1) return SEEDGB_UNSUPPORTED;
    const TuneParams tp{std::min(t->warps_per_cta, mw), t->middles_per_item,
                        t->neighbourhood_capacity, t->ctas_per_sm};
    if (h->arena && cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
    h->tune = tp;
    h->g_valid = false;
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_set_filter(seedgb_seeding* h, const seedgb_doublet_filter* f) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    // kernels in flight may read the current network
    if (cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
    h->g_valid = false;
    if (!f) {
        h->dc.mlp = nullptr;
        return SEEDGB_OK;
    }
    if (f->n_edges > 15 || !(f->band[0] <= f->band[1])) return SEEDGB_INVALID_ARGUMENT;
    if (f->prune_bottom > SEEDGB_FILTER_PRUNE_DOUBLETS || f->prune_top > SEEDGB_FILTER_GATE_MIDDLE)
        return SEEDGB_INVALID_ARGUMENT;
    for (int i = 0; i < 8; ++i)
        if (!std::isfinite(f->mu[i]) || !std::isfinite(f->isd[i])) return SEEDGB_INVALID_ARGUMENT;
    for (uint32_t i = 1; i < f->n_edges; ++i)
        if (!(f->edges[i - 1] <= f->edges[i])) return SEEDGB_INVALID_ARGUMENT;
    std::vector<uint8_t> frag(mlp_frag_bytes());
    pack_mlp_frag(*f, *reinterpret_cast<MlpFrag*>(frag.data()));
    if (!h->d_mlp && cudaMalloc(&h->d_mlp, frag.size()) != cudaSuccess) {
        h->d_mlp = nullptr;
        return SEEDGB_CUDA_ERROR;
    }
    if (cudaMemcpy(h->d_mlp, frag.data(), frag.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    h->dc.mlp = static_cast<const MlpFrag*>(h->d_mlp);
    h->dc.band_lo = f->band[0];
    h->dc.band_hi = f->band[1];
    for (int i = 0; i < 8; ++i) {
        h->dc.mlp_mu[i] = f->mu[i];
        h->dc.mlp_isd[i] = f->isd[i];
    }
    h->dc.mlp_thr[0] = f->threshold[0];
    h->dc.mlp_thr[1] = f->threshold[1];
    h->dc.mlp_n_edges = f->n_edges;
    for (uint32_t i = 0; i < 15; ++i) h->dc.mlp_edges[i] = i < f->n_edges ? f->edges[i] : 0.f;
    h->dc.mlp_prune_bottom = f->prune_bottom;
    h->dc.mlp_prune_top = f->prune_top;
    h->dc.mlp_gate_max_tops = f->gate_max_tops;
    if (f->n_size_classes > 8) return SEEDGB_INVALID_ARGUMENT;
    h->dc.mlp_n_classes = f->n_size_classes;
    for (uint32_t k = 0; k < 8; ++k) {
        const bool on = k < f->n_size_classes;
        if (on && k > 0 && !(f->size_class_max[k - 1] <= f->size_class_max[k]))
            return SEEDGB_INVALID_ARGUMENT;
        h->dc.mlp_class_max[k] = on ? f->size_class_max[k] : 0u;
        for (int r = 0; r < 2; ++r) {
            h->dc.mlp_class_thr[k][r] = on ? f->size_class_threshold[k][r] : 0.f;
            h->dc.mlp_class_band[k][r] = on ? f->size_class_band[k][r] : 0.f;
        }
    }
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_set_doublet_dump(seedgb_seeding* h, void* records,
                                              uint64_t capacity) {
    if (!h || (records && (reinterpret_cast<uintptr_t>(records) % 16))) return SEEDGB_INVALID_ARGUMENT;
    if (cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
    h->dump = records;
    h->dump_cap = records ? capacity : 0;
    h->a.dump = h->dump;
    h->a.dump_cap = h->dump_cap;
    h->g_valid = false;  // the arena view is baked into the graphs
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_set_triplet_dump(seedgb_seeding* h, void* records,
                                               uint64_t capacity) {
    if (!h || (records && (reinterpret_cast<uintptr_t>(records) % 16))) return SEEDGB_INVALID_ARGUMENT;
    if (cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
    h->tdump = records;
    h->tdump_cap = records ? capacity : 0;
    h->a.tdump = static_cast<uint4*>(h->tdump);
    h->a.tdump_cap = h->tdump_cap;
    h->g_valid = false;
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_filter_stats(seedgb_seeding* h, uint32_t n_events,
                                          uint32_t* per_event, uint8_t* fell_back,
                                          uint64_t* n_records, uint64_t* n_triplet_records,
                                          void* stream) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    if (!h->arena) return SEEDGB_INVALID_ARGUMENT;
    if ((per_event || fell_back) && n_events > h->cap_events) return SEEDGB_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t err = cudaSuccess;
    if (per_event && n_events)
        err = cudaMemcpyAsync(per_event, h->a.ev_filter, sizeof(uint32_t) * 4 * n_events,
                              cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess && fell_back && n_events)
        err = cudaMemcpyAsync(fell_back, h->a.ev_mode, n_events, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(h->h_counters, h->a.counters,
                              sizeof(unsigned long long) * kNumCounters, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return SEEDGB_CUDA_ERROR;
    if (fell_back && !h->dc.mlp) std::memset(fell_back, 0, n_events);
    if (n_records) *n_records = h->h_counters[kDumpCount];
    if (n_triplet_records) *n_triplet_records = h->h_counters[kTripDumpCount];
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_get_tune(seedgb_seeding* h, seedgb_tune* t) {
    if (!h || !t) return SEEDGB_INVALID_ARGUMENT;
    t->warps_per_cta = h->tune.fast_warps;
    t->middles_per_item = h->tune.middles_per_item;
    t->neighbourhood_capacity = h->tune.nb_cap;
    t->ctas_per_sm = h->tune.ctas_per_sm;
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_run(seedgb_seeding* h, const seedgb_spacepoint_view* sps,
                                 seedgb_seed_buffer* out, void* stream) {
    return seedgb_seeding_run_batch(h, sps, 1, out, stream);
}

seedgb_status seedgb_seeding_last_status(seedgb_seeding* h, void* stream) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    if (!h->arena) return SEEDGB_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t err = cudaMemcpyAsync(h->h_counters, h->a.counters,
                                      sizeof(unsigned long long) * kNumCounters,
                                      cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return SEEDGB_CUDA_ERROR;
    const unsigned long long bits = h->h_counters[kStatus];
    if (bits & (1ull << SEEDGB_CAPACITY_OVERFLOW)) return SEEDGB_CAPACITY_OVERFLOW;
    if (bits & (1ull << SEEDGB_TIMEOUT)) return SEEDGB_TIMEOUT;
    if (bits & (1ull << SEEDGB_BAD_CONFIG)) return SEEDGB_BAD_CONFIG;
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_counters(seedgb_seeding* h, uint64_t out[9]) {
    if (!h || !out) return SEEDGB_INVALID_ARGUMENT;
    out[0] = h->h_counters[kNumValid];
    out[1] = h->h_counters[kOvfCount];
    out[2] = h->h_counters[kNumMB];
    out[3] = h->h_counters[kNumMT];
    out[4] = h->h_counters[kNumTriplets];
    out[5] = h->h_counters[kNumSeeds];
    out[6] = h->h_counters[kPhiUndecided];
    out[7] = h->h_counters[kItemTotal];
    out[8] = h->h_counters[kOvf2Count];
    return SEEDGB_OK;
}

seedgb_status seedgb_seeding_copy_grid(seedgb_seeding* h, uint32_t event,
                                       uint32_t* bin_offsets, uint32_t* bin_sps,
                                       uint32_t bin_sps_capacity, uint32_t* n_valid,
                                       void* stream) {
    if (!h || !bin_offsets || !n_valid) return SEEDGB_INVALID_ARGUMENT;
    if (!h->arena || event >= h->cap_events) return SEEDGB_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t nb = h->dc.nbins;
    std::vector<uint32_t> bs(nb + 1);
    EventDesc d;
    cudaError_t err = cudaMemcpyAsync(bs.data(), h->a.bin_start + static_cast<size_t>(event) * (nb + 1),
                                      sizeof(uint32_t) * (nb + 1), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(&d, h->a.events + event, sizeof(EventDesc), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return SEEDGB_CUDA_ERROR;
    const uint32_t nv = bs[nb] - bs[0];
    *n_valid = nv;
    for (uint32_t b = 0; b <= nb; ++b) bin_offsets[b] = bs[b] - bs[0];
    if (nv > 0) {
        if (!bin_sps || bin_sps_capacity < nv) return SEEDGB_INVALID_ARGUMENT;
        err = cudaMemcpyAsync(bin_sps, h->a.g_idx + bs[0], sizeof(uint32_t) * nv,
                              cudaMemcpyDeviceToHost, s);
        if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    }
    return cuda_status(err);
}

seedgb_status seedgb_seeding_set_option(seedgb_seeding* h, seedgb_option opt, int64_t value) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    switch (opt) {
        case SEEDGB_OPTION_EXHAUSTIVE_TRIPLETS:
            h->dc.brute_force_triplets = value ? 1u : 0u;
            h->g_valid = false;  // the configuration is baked into the graphs
            return SEEDGB_OK;
        case SEEDGB_OPTION_LAST_TIER_ONLY:
            h->dc.last_tier_only = value ? 1u : 0u;
            h->g_valid = false;
            return SEEDGB_OK;
        case SEEDGB_OPTION_KERNEL_TIMING:
            if (value && !h->tev[0]) {
                for (auto& e : h->tev)
                    if (cudaEventCreate(&e) != cudaSuccess) return SEEDGB_CUDA_ERROR;
            }
            h->timing = value != 0;
            return SEEDGB_OK;
    }
    return SEEDGB_INVALID_ARGUMENT;
}

seedgb_status seedgb_seeding_kernel_times(seedgb_seeding* h, float ms[10]) {
    if (!h || !ms || !h->timed_run) return SEEDGB_INVALID_ARGUMENT;
    if (cudaEventSynchronize(h->tev[kNumKernels]) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    for (int i = 0; i < kNumKernels; ++i) {
        if (cudaEventElapsedTime(&ms[i], h->tev[i], h->tev[i + 1]) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
    }
    return SEEDGB_OK;
}

seedgb_status seedgb_params_create(const seedgb_track_params_estimation_config* cfg,
                                   seedgb_params** out) {
    if (!cfg || !out) return SEEDGB_INVALID_ARGUMENT;
    seedgb_params* h = new (std::nothrow) seedgb_params();
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    for (int i = 0; i < 6; ++i) {
        h->pc.initial_sigma[i] = cfg->initial_sigma[i];
        h->pc.initial_inflation[i] = cfg->initial_inflation[i];
    }
    h->pc.initial_sigma_qopt = cfg->initial_sigma_qopt;
    h->pc.initial_sigma_pt_rel = cfg->initial_sigma_pt_rel;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev) !=
            cudaSuccess) {
        delete h;
        return SEEDGB_CUDA_ERROR;
    }
    *out = h;
    return SEEDGB_OK;
}

seedgb_status seedgb_params_destroy(seedgb_params* h) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    delete h;
    return SEEDGB_OK;
}

seedgb_status seedgb_params_run(seedgb_params* h, const float bfield[3],
                                const seedgb_measurement_view* meas,
                                const seedgb_spacepoint_view* sps,
                                const seedgb_seed_buffer* seeds, seedgb_params_buffer* out,
                                void* stream) {
    if (!h || !bfield || !meas || !sps || !seeds || !out || !seeds->size || !out->size)
        return SEEDGB_INVALID_ARGUMENT;
    return cuda_status(launch_params(h->pc, bfield, *meas, *sps, *seeds, *out, h->num_sms,
                                     static_cast<cudaStream_t>(stream)));
}

seedgb_status seedgb_params_run_batch(seedgb_params* h, const float bfield[3],
                                      const seedgb_measurement_view* meas,
                                      const seedgb_spacepoint_view* sps,
                                      const seedgb_seed_buffer* seeds,
                                      seedgb_params_buffer* outs, uint32_t n_events,
                                      void* stream) {
    if (!h || !bfield || (n_events && (!meas || !sps || !seeds || !outs)))
        return SEEDGB_INVALID_ARGUMENT;
    if (n_events == 0) return SEEDGB_OK;
    if (n_events > 65535u) return SEEDGB_SIZE_LIMIT;
    for (uint32_t e = 0; e < n_events; ++e)
        if (!seeds[e].size || !outs[e].size) return SEEDGB_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ParamsSlot& sl = h->slot[h->next];
    // the previous copy out of this slot's pinned descriptors must be done
    if (sl.copied && cudaEventSynchronize(sl.copied) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    if (sl.cap < n_events) {
        // in-flight launches may still read the old device descriptors
        if (sl.dev && cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.dev) cudaFree(sl.dev);
        sl.host = nullptr;
        sl.dev = nullptr;
        sl.cap = 0;
        const uint32_t cap = std::max(n_events, 64u);
        if (cudaMallocHost(reinterpret_cast<void**>(&sl.host), sizeof(seedgb::ParamsEvent) * cap) !=
                cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&sl.dev), sizeof(seedgb::ParamsEvent) * cap) !=
                cudaSuccess)
            return SEEDGB_CUDA_ERROR;
        sl.cap = cap;
    }
    if (!sl.copied && cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    for (uint32_t e = 0; e < n_events; ++e)
        sl.host[e] = seedgb::ParamsEvent{meas[e], sps[e], seeds[e], outs[e]};
    if (cudaMemcpyAsync(sl.dev, sl.host, sizeof(seedgb::ParamsEvent) * n_events,
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaEventRecord(sl.copied, s) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    h->next ^= 1;
    return cuda_status(launch_params_batch(h->pc, bfield, sl.dev, n_events, h->num_sms, s));
}

}  // extern "C"
