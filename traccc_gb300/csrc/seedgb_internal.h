// Internal structures shared by the seeding kernels and the C-ABI layer.
//
// Device data layout of one batch (all arrays live in one arena owned by the
// seeding handle; "grid position" = position in the binned spacepoint grid of
// the whole batch, event e owning [sp_base[e], sp_base[e] + n_valid[e])):
//
//   sp_bin      int32 [total_sp]            grid bin of each input spacepoint or -1
//   whist       uint32[chunks][NWB][nbins]  per-warp bin histograms -> offsets
//   bin_start   uint32[E][nbins+1]          grid-position range of each bin
//   g_xyzr      float4[total_sp]            binned x, y, z, r (r = sqrt(x^2+y^2))
//   g_var       float2[total_sp]            binned z / radius variances
//   g_idx       uint32[total_sp]            binned spacepoint index within its event
//   g_rs        float4[total_sp]            each bin's spacepoints sorted by radius
//   g_rs_gp     uint32[total_sp]            grid position of each g_rs entry
//   bin_unsorted uint8[E][nbins]            bin too large to sort in shared memory
//   items       uint2 [max_items]           (event, bin | chunk<<16) work items
//   item_key    uint8 [max_items]           cost bucket of each work item
//   items_ord   uint2 [max_items]           work items, most costly first
//   seed_cnt    uint8 [total_sp]            seeds per middle spacepoint
//   seed_slot   SeedSlot[total_sp][KMAX]    seeds per middle, in final order
//   chunk_seeds uint32[chunks]              seeds of each 2048-middle chunk
//   ovf         uint32[2 total_sp]          middles the fast kernel hands to the general path
//   ovf2        uint32[2 total_sp]          middles beyond the general path's middle tier
//   counters    uint64[kNumCounters]
#pragma once

#include <cstddef>
#include <cstdint>

#include "seedgb.h"

namespace seedgb {

constexpr int kMaxSeedsPerMiddle = SEEDGB_MAX_SEEDS_PER_MIDDLE;
constexpr int kMaxSegments = 64;      // neighbourhood bins per middle
constexpr int kMaxBins = 4096;        // phi x z bins
constexpr uint32_t kMaxEventsPerBatch = 65535;
constexpr uint32_t kOrderBuckets = 256;  // log-scale cost buckets of the work items

// Binning chunk geometry: NWB warps x RB rounds x 32 spacepoints, each warp a
// contiguous run of spacepoints (stable order inside a bin).
constexpr int kBinWarps = 8;
constexpr int kBinRounds = 8;
constexpr int kBinChunk = kBinWarps * kBinRounds * 32;  // 2048

enum Counter : int {
    kStatus = 0,        // bit mask of seedgb_status values (1 << status)
    kItemFetch = 1,     // work-item counter of the fast seeding kernel
    kItemTotal = 2,     // number of work items
    kOvfCount = 3,      // middles queued for the large-capacity path
    kOvfFetch = 4,
    kNumMB = 5,
    kNumMT = 6,
    kNumTriplets = 7,
    kNumSeeds = 8,
    kNumValid = 9,
    kAnyVariance = 10,  // nonzero if any spacepoint has a nonzero variance
    kPhiUndecided = 11, // correctly rounded phi not decidable from double
    kItemFetch2 = 12,   // work-item counter of the fallback (plain) pass
    kDumpCount = 13,    // doublet records written (may exceed the capacity)
    kFallbackEvents = 14,  // events re-seeded without the learned filter
    kOvfFetch2 = 15,    // large-capacity queue counter of the fallback pass
    kTripDumpCount = 16,  // triplet records written (may exceed the capacity)
    kOvf2Count = 17,    // middles queued for the last (large-capacity) tier
    kOvf2Fetch = 18,
    kOvf2Fetch2 = 19,   // last-tier queue counter of the fallback pass
    kNumCounters = 24
};
// bytes of the per-batch counters and the work-item order histogram
// (zeroed with one memset at the start of every batch)
constexpr size_t kCounterBytes =
    sizeof(unsigned long long) * kNumCounters + sizeof(uint32_t) * 2 * kOrderBuckets;

struct MlpFrag;  // seedgb_mlp.cuh

// Kernel-side copy of the configuration (host-derived, passed by value).
struct DevConfig {
    // seedfinder_config
    float zMin, zMax, phiMin, phiMax;
    float beam0, beam1;
    unsigned long long nrbins;  // (size_t)(rMax + |beamPos|)
    float deltaRMin, deltaRMax, cotThetaMax, collisionRegionMin,
        collisionRegionMax, deltaZMax, impactMax, minHelixRadius;
    float maxScatteringAngle2, sigmaScattering, minHelixDiameter2, pT2perRadius,
        pTPerHelixRadius, maxPtScattering, highland;
    uint32_t maxSeedsPerSpM;
    uint32_t scope0, scope1;
    // seedfilter_config
    float deltaInvHelixDiameter, impactWeightFactor, compatSeedWeight,
        filterDeltaRMin;
    uint32_t compatSeedLimit;
    float good_spB_min_radius, good_spB_weight_increase, good_spT_max_radius,
        good_spT_weight_increase, good_spB_min_weight, seed_min_weight,
        spB_min_radius;
    // axes
    uint32_t phi_bins, z_bins, nbins;
    float phi_min, phi_max, z_min, z_max;
    // behaviour switches (tests)
    uint32_t brute_force_triplets;  // 1: test every MB x MT pair (no cot window)
    uint32_t last_tier_only;        // 1: the general path's middle tier passes every middle on
    // learned doublet filter: nullptr = plain seeding
    const MlpFrag* mlp;         // weight fragments and biases (device)
    float band_lo, band_hi;     // pruned-fraction band; outside it: plain re-run
    float mlp_mu[8], mlp_isd[8];
    float mlp_thr[2];           // keep when logit >= mlp_thr[role], role 1 = top
    float mlp_edges[15];        // radial band edges of the layer-pair feature
    uint32_t mlp_n_edges;
    uint32_t mlp_prune_bottom, mlp_prune_top;
    // per-event-size classes of thresholds and band (0 classes: the above)
    uint32_t mlp_n_classes;
    uint32_t mlp_class_max[8];
    float mlp_class_thr[8][2];
    float mlp_class_band[8][2];
    uint32_t mlp_gate_max_tops;  // middle gate: larger middles kept unscored (0: none)
};

// One event of a batch, as the kernels see it.
struct EventDesc {
    const uint32_t* mi1;
    const uint32_t* mi2;
    const float* global;
    const float* zvar;
    const float* rvar;
    uint32_t n_sp;
    uint32_t sp_base;     // first grid position / internal index of the event
    uint32_t chunk_base;  // first binning chunk of the event
    uint32_t n_chunks;
    uint32_t* out_b;
    uint32_t* out_m;
    uint32_t* out_t;
    float* out_q;
    uint32_t out_cap;
    uint32_t pad;
    uint32_t* out_size;
};

// Sizes of the batch in flight, device-resident so that a CUDA graph captured
// with capacity-sized grids serves any batch up to its capacity.
struct BatchHeader {
    uint32_t n_events;
    uint32_t total_chunks;
    uint32_t total_sp;
    uint32_t pad;
};

struct SeedSlot {
    uint32_t b, m, t;
    float q;
};

// Pointers into the work arena.
struct Arena {
    BatchHeader* hdr;       // sizes of the batch (device)
    EventDesc* events;      // [E]
    uint32_t* chunk_event;  // [total_chunks]
    int32_t* sp_bin;
    uint32_t* whist;
    uint32_t* bin_start;
    uint32_t* n_valid;      // [E]
    float4* g_xyzr;
    float2* g_var;
    uint32_t* g_idx;
    float4* g_rs;           // [total_sp] every bin sorted by radius
    uint32_t* g_rs_gp;      // [total_sp] grid position of each g_rs entry
    uint8_t* bin_unsorted;  // [E][nbins] bin too large to sort
    uint2* items;
    uint8_t* item_key;      // [max_items] cost bucket of each item
    uint2* items_ord;       // [max_items] items, most costly first
    uint32_t* order_hist;   // [2 * kOrderBuckets] items per bucket, scatter cursors
    uint8_t* seed_cnt;
    SeedSlot* seed_slot;
    uint32_t* chunk_seeds;  // [cap_chunks] seeds of each binning chunk of middles
    uint32_t* ovf;          // [2 * cap_sp] middles for the general path (middle tier)
    uint32_t* ovf2;         // [2 * cap_sp] middles for its last, large-capacity tier
    unsigned long long* counters;
    uint32_t* ev_filter;    // [E][4] scored / pruned middle-bottom, scored / pruned middle-top
    uint8_t* ev_mode;       // [E] 1: re-seed without the filter (fallback pass)
    void* dump;             // doublet records (48 B each) or nullptr
    unsigned long long dump_cap;
    uint4* tdump;           // triplet records {middle, bottom, top, event} or nullptr
    unsigned long long tdump_cap;
    uint32_t cap_events;    // capacities of the arena (launch grids of a graph)
    uint32_t cap_chunks;
    uint32_t cap_sp;
    uint32_t max_items;
};

// Launch shapes picked by the autotuner (see seedgb_api.cu).
struct TuneParams {
    int fast_warps;        // warps per CTA of the fast seeding kernel
    int middles_per_item;  // middles per work item
    int nb_cap;            // neighbourhood spacepoints staged in shared memory
    int ctas_per_sm;
};

// Kernel-side config from the reference config structs and the grid axes.
DevConfig make_dev_config(const seedgb_seedfinder_config& f,
                          const seedgb_seedfilter_config& fl,
                          const seedgb_grid_axes& ax);

// Kernel launchers (seedgb_kernels.cu).  All asynchronous on `stream`.
// timing: nullptr, or kNumKernels+1 events recorded around the kernels.
// grid: the batch sizes that size the launch grids (the actual batch, or the
// arena capacities when capturing a graph); the kernels read the actual
// sizes from a.hdr.
constexpr int kNumKernels = 10;
// Sets the kernels' shared-memory attributes on the current device (once).
cudaError_t prepare_kernels();
cudaError_t launch_seeding(const DevConfig& cfg, const Arena& a, const BatchHeader& grid,
                           const TuneParams& tp, int num_sms,
                           cudaStream_t stream, cudaEvent_t* timing = nullptr);

struct ParamsConfig {
    float initial_sigma[6];
    float initial_sigma_qopt, initial_sigma_pt_rel;
    float initial_inflation[6];
};

cudaError_t launch_params(const ParamsConfig& cfg, const float bfield[3],
                          const seedgb_measurement_view& meas,
                          const seedgb_spacepoint_view& sps,
                          const seedgb_seed_buffer& seeds,
                          const seedgb_params_buffer& out, int num_sms,
                          cudaStream_t stream);

// One event of a batched parameter estimation (device-side descriptor).
struct ParamsEvent {
    seedgb_measurement_view meas;
    seedgb_spacepoint_view sps;
    seedgb_seed_buffer seeds;
    seedgb_params_buffer out;
};
cudaError_t launch_params_batch(const ParamsConfig& cfg, const float bfield[3],
                                const ParamsEvent* events, uint32_t n_events, int num_sms,
                                cudaStream_t stream);

size_t fast_kernel_smem(const TuneParams& tp);
// Packs the host-side network into the fragment layout the kernels read.
void pack_mlp_frag(const seedgb_doublet_filter& m, MlpFrag& f);
size_t mlp_frag_bytes();
// Most warps per CTA whose scratch fits next to an nb_cap staging buffer with
// ctas_per_sm CTAs resident on one SM.
int fast_kernel_max_warps(int nb_cap, int ctas_per_sm = 1);

}  // namespace seedgb
