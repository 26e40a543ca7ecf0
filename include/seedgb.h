/*
 * seedgb.h -- C ABI of the GB300-native triplet seeding library.
 *
 * A drop-in for traccc's triplet seeding stage (spacepoint binning, doublet
 * finding, triplet finding, seed filtering) and its track-parameter
 * estimation, running on one GB300 (sm_103a).  Plain pointers and sizes only:
 * every pointer marked "device" is a CUDA device address, streams are passed
 * as void* holding a cudaStream_t.
 *
 * Reference interfaces replaced (paths in the traccc 1.6.0 tree):
 *  - seedgb_seeding_*  <- traccc::cuda::triplet_seeding_algorithm
 *      (device/cuda/include/traccc/cuda/seeding/triplet_seeding_algorithm.hpp:35-40,
 *       operator() at device/common/include/traccc/seeding/device/
 *       triplet_seeding_algorithm.hpp:68-69), with the results of
 *      traccc::host::seeding_algorithm (core/include/traccc/seeding/
 *       seeding_algorithm.hpp:40-52).
 *  - seedgb_params_*   <- traccc::cuda::seed_parameter_estimation_algorithm
 *      (device/cuda/include/traccc/cuda/seeding/
 *       seed_parameter_estimation_algorithm.hpp:33-37, operator() at
 *       device/common/include/traccc/seeding/device/
 *       seed_parameter_estimation_algorithm.hpp:48-67) and
 *      traccc::host::track_params_estimation (core/include/traccc/seeding/
 *       track_params_estimation.hpp:31-67).
 *
 * Semantics: all work is enqueued on the caller's stream and the calls return
 * before it finishes (as the reference's device algorithms do); no call of the
 * run functions blocks on the device, except that growing a handle's work
 * space (a batch larger than anything reserved before) waits for the device.
 * set_tune, set_filter and the dump setters wait for the device before they
 * change what kernels in flight read (set_option applies to the next run);
 * status, counter and grid queries synchronise the given stream;
 * seedgb_form_spacepoints returns after its stream has finished the call.
 * Errors are status codes, never exceptions.  A handle is not thread-safe:
 * use one handle per host thread / stream, as the reference uses one
 * algorithm object per thread.
 */
#ifndef SEEDGB_H
#define SEEDGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEEDGB_ABI_VERSION 1u
#define SEEDGB_INVALID_MEASUREMENT_INDEX 0xFFFFFFFFu
/* Largest number of seeds kept per middle spacepoint (maxSeedsPerSpM). */
#define SEEDGB_MAX_SEEDS_PER_MIDDLE 8u

typedef enum {
    SEEDGB_OK = 0,
    /* empty input: nothing was launched except writing size 0 (the reference
     * returns an empty buffer, triplet_seeding_algorithm.cpp:75-77) */
    SEEDGB_EMPTY = 1,
    /* the configuration is rejected (the reference throws std::domain_error,
     * spacepoint_binning_helper.hpp:33-38,77-81) */
    SEEDGB_BAD_CONFIG = 2,
    /* a CUDA runtime call failed (the reference throws std::runtime_error,
     * device/cuda/src/utils/cuda_error_handling.hpp:14-21) */
    SEEDGB_CUDA_ERROR = 3,
    /* a device-side buffer was too small; the result is incomplete */
    SEEDGB_CAPACITY_OVERFLOW = 4,
    /* a bounded device-side wait ran out */
    SEEDGB_TIMEOUT = 5,
    SEEDGB_INVALID_ARGUMENT = 6,
    SEEDGB_UNSUPPORTED = 7,
    /* the input exceeds the fixed capacity of an allocation-free entry point */
    SEEDGB_SIZE_LIMIT = 8
} seedgb_status;

/* traccc::seedfinder_config (core/include/traccc/seeding/detail/
 * seeding_config.hpp:17-139), same fields, same order, same units
 * (mm, GeV, T = 0.000299792458 GeV/(e mm)). */
typedef struct {
    float zMin, zMax, rMax, rMin;
    float collisionRegionMin, collisionRegionMax;
    float phiMin, phiMax;
    float minPt, cotThetaMax, deltaRMin, deltaRMax, deltaZMax;
    float impactMax, sigmaScattering, maxPtScattering;
    uint32_t maxSeedsPerSpM;
    float bFieldInZ;
    float beamPos[2];
    float radLengthPerSeed, zAlign, rAlign, sigmaError;
    float highland, maxScatteringAngle2, pTPerHelixRadius, minHelixDiameter2,
        minHelixRadius, pT2perRadius;
    int32_t phiBinDeflectionCoverage;
    uint32_t neighbor_scope[2];
} seedgb_seedfinder_config;

/* traccc::spacepoint_grid_config (seeding_config.hpp:142-189). */
typedef struct {
    float bFieldInZ, minPt, rMax, zMax, zMin, deltaRMax, cotThetaMax, impactMax;
    float phiMin, phiMax;
    int32_t phiBinDeflectionCoverage;
} seedgb_spacepoint_grid_config;

/* traccc::seedfilter_config (seeding_config.hpp:191-219). */
typedef struct {
    float deltaInvHelixDiameter, impactWeightFactor, compatSeedWeight, deltaRMin;
    uint64_t compatSeedLimit;
    float good_spB_min_radius, good_spB_weight_increase;
    float good_spT_max_radius, good_spT_weight_increase;
    float good_spB_min_weight, seed_min_weight, spB_min_radius;
} seedgb_seedfilter_config;

/* traccc::track_params_estimation_config
 * (core/include/traccc/seeding/detail/track_params_estimation_config.hpp:18-33) */
typedef struct {
    float initial_sigma[6];
    float initial_sigma_qopt;
    float initial_sigma_pt_rel;
    float initial_inflation[6];
} seedgb_track_params_estimation_config;

/* The reference's config constructors: defaults + setup()
 * (seeding_config.hpp:19,120-138,146-157,191-219). */
void seedgb_seedfinder_config_default(seedgb_seedfinder_config* c);
/* seedfinder_config::setup(): recompute the derived members after a change. */
void seedgb_seedfinder_config_setup(seedgb_seedfinder_config* c);
void seedgb_spacepoint_grid_config_from_finder(seedgb_spacepoint_grid_config* g,
                                               const seedgb_seedfinder_config* f);
void seedgb_seedfilter_config_default(seedgb_seedfilter_config* c);
void seedgb_track_params_estimation_config_default(
    seedgb_track_params_estimation_config* c);

/* Grid axes from get_axes (core/include/traccc/seeding/
 * spacepoint_binning_helper.hpp:22-110): circular phi axis, regular z axis. */
typedef struct {
    uint32_t phi_bins;
    float phi_min, phi_max;
    uint32_t z_bins;
    float z_min, z_max;
} seedgb_grid_axes;
seedgb_status seedgb_get_axes(const seedgb_spacepoint_grid_config* g,
                              seedgb_grid_axes* out);

/* edm::spacepoint_collection view (core/include/traccc/edm/
 * spacepoint_collection.hpp:222-234): five device columns; global holds x, y, z
 * interleaved (std::array<float,3>, 12-byte stride). */
typedef struct {
    const uint32_t* measurement_index_1;
    const uint32_t* measurement_index_2;
    const float* global;
    const float* z_variance;
    const float* radius_variance;
    uint32_t size;
} seedgb_spacepoint_view;

/* edm::seed_collection buffer (core/include/traccc/edm/seed_collection.hpp:
 * 142-146): four device columns of `capacity` elements and a device-resident
 * element count, like the reference's resizable buffer
 * (triplet_seeding_algorithm.cpp:249-252).  Seed indices are spacepoint
 * indices of the input view. */
typedef struct {
    uint32_t* bottom_index;
    uint32_t* middle_index;
    uint32_t* top_index;
    float* quality;
    uint32_t capacity;
    uint32_t* size; /* device */
} seedgb_seed_buffer;

/* The measurement columns parameter estimation reads (edm::
 * measurement_collection, core/include/traccc/edm/measurement_collection.hpp:
 * 240-259): local_position (2 floats each) and surface_link (64-bit id). */
typedef struct {
    const float* local_position;
    const uint64_t* surface_link;
    uint32_t size;
} seedgb_measurement_view;

/* bound_track_parameters: surface link, {loc0, loc1, phi, theta, q/p, time},
 * 6x6 covariance (row-major; the diagonal is set, the rest is zero). */
typedef struct {
    uint64_t surface_link;
    float params[6];
    float cov[36];
} seedgb_bound_track_parameters;

typedef struct {
    seedgb_bound_track_parameters* data; /* device */
    uint32_t capacity;
    uint32_t* size; /* device */
} seedgb_params_buffer;

/* ------------------------------------------------------------------------ */
/* Seeding                                                                   */
/* ------------------------------------------------------------------------ */

typedef struct seedgb_seeding seedgb_seeding;

/* Replaces triplet_seeding_algorithm(finder, grid, filter, mr, copy, stream)
 * (triplet_seeding_algorithm.hpp:35-40).  Validates the grid (get_axes) and
 * returns SEEDGB_BAD_CONFIG where the reference throws.  Allocates nothing on
 * the device until the first run or seedgb_seeding_reserve. */
seedgb_status seedgb_seeding_create(const seedgb_seedfinder_config* finder,
                                    const seedgb_spacepoint_grid_config* grid,
                                    const seedgb_seedfilter_config* filter,
                                    seedgb_seeding** out);
seedgb_status seedgb_seeding_destroy(seedgb_seeding* h);

/* Size the device work space for batches of up to max_events events holding up
 * to max_total_spacepoints spacepoints together.  Runs that fit need no
 * further allocation (which is what makes them capturable in a CUDA graph). */
seedgb_status seedgb_seeding_reserve(seedgb_seeding* h, uint32_t max_events,
                                     uint64_t max_total_spacepoints);

/* Replaces edm::seed_collection::buffer operator()(spacepoint view)
 * (device/common/include/traccc/seeding/device/triplet_seeding_algorithm.hpp:
 * 68-69).  Seeds are written in the host seeding order (grid bin, then middle
 * spacepoint index, then seed rank), identical to traccc::host::
 * seeding_algorithm.  out->capacity must be >= maxSeedsPerSpM * sps->size to
 * be safe; a smaller buffer is filled up to capacity and the status word
 * reports SEEDGB_CAPACITY_OVERFLOW.  Asynchronous on `stream`. */
seedgb_status seedgb_seeding_run(seedgb_seeding* h,
                                 const seedgb_spacepoint_view* sps,
                                 seedgb_seed_buffer* out, void* stream);

/* Many events with uneven sizes in one launch sequence (the GB300 form of the
 * reference's one-stream-per-thread event concurrency, examples/run/common/
 * include/traccc/examples/impl/throughput_mt.ipp:171-179). */
seedgb_status seedgb_seeding_run_batch(seedgb_seeding* h,
                                       const seedgb_spacepoint_view* events,
                                       uint32_t n_events,
                                       seedgb_seed_buffer* outs, void* stream);

/* Synchronise `stream` and return the device status of the last run
 * (SEEDGB_OK, SEEDGB_CAPACITY_OVERFLOW, SEEDGB_TIMEOUT). */
seedgb_status seedgb_seeding_last_status(seedgb_seeding* h, void* stream);

/* Work counters of the last run (after seedgb_seeding_last_status):
 * out[0] valid spacepoints, out[1] middles the fast kernel handed to the
 * general path, out[2] middle-bottom doublets, out[3] middle-top doublets,
 * out[4] triplets, out[5] seeds, out[6] spacepoints whose correctly rounded
 * phi the double-precision atan2 could not decide (expected 0), out[7] work
 * items, out[8] middles that reached the general path's last
 * (large-capacity) tier. */
seedgb_status seedgb_seeding_counters(seedgb_seeding* h, uint64_t out[9]);

/* Copy the phi-z grid of event `event` of the last run to host memory
 * (synchronises `stream`): bin_offsets[nbins+1] (CSR) and bin_sps[n_valid] =
 * spacepoint indices in grid order.  The same grid as
 * traccc::host::details::spacepoint_binning::operator()
 * (core/src/seeding/spacepoint_binning.cpp:27-53): bins in serial order
 * phi + nphi * z, spacepoints of a bin in ascending index order.
 * bin_sps_capacity must be >= the event's spacepoint count. */
seedgb_status seedgb_seeding_copy_grid(seedgb_seeding* h, uint32_t event,
                                       uint32_t* bin_offsets, uint32_t* bin_sps,
                                       uint32_t bin_sps_capacity,
                                       uint32_t* n_valid, void* stream);

/* Behaviour options (not part of the reference interface). */
typedef enum {
    /* 1: test every middle-bottom x middle-top doublet pair for triplets
     * instead of the cot(theta) window (verification of the window; the
     * results are identical, only slower). */
    SEEDGB_OPTION_EXHAUSTIVE_TRIPLETS = 1,
    /* 1: record CUDA events around every kernel of a run on the run's stream
     * (read back with seedgb_seeding_kernel_times) */
    SEEDGB_OPTION_KERNEL_TIMING = 2,
    /* 1: the general path's middle tier (k_seed_mid) hands every middle it
     * receives on to the last, large-capacity tier (verification of that
     * tier; the results are identical, only slower) */
    SEEDGB_OPTION_LAST_TIER_ONLY = 3
} seedgb_option;
seedgb_status seedgb_seeding_set_option(seedgb_seeding* h, seedgb_option opt,
                                        int64_t value);

/* Device durations (ms) of the kernels of the last run with
 * SEEDGB_OPTION_KERNEL_TIMING on, in launch order: bin_count, bin_scan,
 * item_order, bin_scatter, bin_rsort, seed_fast, seed_mid, seed_slow,
 * seed_count, seed_compact (with the learned filter, seed_slow also covers
 * the fallback pass).  Waits for the last recorded event.  Returns
 * SEEDGB_INVALID_ARGUMENT if timing was off. */
seedgb_status seedgb_seeding_kernel_times(seedgb_seeding* h, float ms[10]);

/* ------------------------------------------------------------------------ */
/* Spacepoint formation (the step in front of the seeding path)              */
/* ------------------------------------------------------------------------ */

/* A measurement surface: local -> global placement and shape, the part of
 * detray's tracking_surface::local_to_global that spacepoint formation uses
 * (core/include/traccc/seeding/impl/spacepoint_formation.ipp:30-38).
 *  type 0, plane:    (l0, l1)      -> R (l0, l1, 0) + t
 *  type 1, cylinder: (r phi, z)    -> R (r cos phi, r sin phi, z) + t,
 *                    phi = l0 / radius
 * R is row-major; each global coordinate is (R[i][0] a + R[i][1] b) +
 * R[i][2] c + t[i] in float arithmetic without contraction; cos and sin of
 * the cylinder angle are evaluated in double and rounded to float. */
typedef struct {
    uint32_t type;
    float radius;
    float rotation[9];
    float translation[3];
} seedgb_surface;

/* Replaces silicon_pixel_spacepoint_formation (core/src/seeding/
 * silicon_pixel_spacepoint_formation.hpp:31-60; device form_spacepoints,
 * device/common/include/traccc/seeding/device/impl/form_spacepoints.ipp):
 * one spacepoint per 2-dimensional measurement (dimensions == NULL: all
 * are), global position from its surface, measurement_index_1 = the
 * measurement's index, measurement_index_2 = SEEDGB_INVALID_MEASUREMENT_INDEX,
 * variances 0.  The surface of a measurement is surfaces[surface_link];
 * measurements whose surface_link is >= n_surfaces form no spacepoint.
 * Spacepoints are written in measurement order (the host algorithm's order;
 * the reference's device version appends in no fixed order).  All pointers
 * are device memory except `surfaces_host`, copied on the stream; outputs
 * have room for meas->size spacepoints; *n_out (device) receives the count.
 * Returns after the stream has finished the call (the surface table is then
 * free to change); calls from one host thread share a scratch area. */
seedgb_status seedgb_form_spacepoints(const seedgb_surface* surfaces_host, uint32_t n_surfaces,
                                      const seedgb_measurement_view* meas,
                                      const uint8_t* dimensions,
                                      uint32_t* measurement_index_1,
                                      uint32_t* measurement_index_2, float* global,
                                      float* z_variance, float* radius_variance,
                                      uint32_t* n_out, void* stream);

/* Spacepoint formation for many events per call, without host
 * synchronisation: the surface table is uploaded once, at creation, and
 * stays on the device; each batch is one launch sequence (descriptor copy
 * from pinned memory, count, scan, write) over all its events.  Same
 * spacepoints, in the same order, as seedgb_form_spacepoints per event.  No
 * counterpart in the reference, whose algorithm forms one event per call
 * (silicon_pixel_spacepoint_formation.hpp:31-60). */
typedef struct {
    uint32_t* measurement_index_1;
    uint32_t* measurement_index_2;
    float* global;          /* x, y, z interleaved */
    float* z_variance;
    float* radius_variance;
    uint32_t capacity;      /* >= the event's measurement count */
    uint32_t* size;         /* device: spacepoints formed */
} seedgb_spacepoint_buffer;

typedef struct seedgb_formation seedgb_formation;
seedgb_status seedgb_formation_create(const seedgb_surface* surfaces_host, uint32_t n_surfaces,
                                      seedgb_formation** out);
seedgb_status seedgb_formation_destroy(seedgb_formation* h);
/* Element e of each array belongs to event e; dimensions may be NULL (all
 * measurements 2-dimensional), else an array of n_events device pointers
 * (each may be NULL).  Asynchronous on `stream`; the descriptors travel
 * through two pinned slots used in turn (a call waits only for the copy of
 * the call before the previous one).  SEEDGB_INVALID_ARGUMENT when an
 * output's capacity is below its event's measurement count; SEEDGB_SIZE_LIMIT
 * above 65535 events.  One stream per handle. */
seedgb_status seedgb_formation_run_batch(seedgb_formation* h, const seedgb_measurement_view* meas,
                                         const uint8_t* const* dimensions,
                                         seedgb_spacepoint_buffer* outs, uint32_t n_events,
                                         void* stream);

/* ------------------------------------------------------------------------ */
/* CSV input (traccc's on-disk event format)                                 */
/* ------------------------------------------------------------------------ */

/* Number of data rows of a CSV file (its header line excluded), or -1. */
int64_t seedgb_csv_rows(const char* path);

/* Replaces traccc::io::csv::read_spacepoints (io/src/csv/read_spacepoints.cpp:
 * 25-77): one spacepoint per row of the hit file (columns tx, ty, tz, found
 * by name), measurement_index_1 = the measurement whose measurement-hit-id
 * row names this hit's row index (else SEEDGB_INVALID_MEASUREMENT_INDEX),
 * measurement_index_2 = invalid, variances 0.  Host memory, capacity rows;
 * *n gets the row count.  meas_hit_map_path may be NULL (all invalid).
 * Measurements keep file order (the reader's sort_measurements = false). */
seedgb_status seedgb_csv_read_spacepoints(const char* hits_path, const char* meas_hit_map_path,
                                          uint64_t capacity, uint32_t* measurement_index_1,
                                          uint32_t* measurement_index_2, float* global,
                                          float* z_variance, float* radius_variance,
                                          uint64_t* n);

/* The measurement columns parameter estimation reads, from a measurement
 * file (io/include/traccc/io/csv/measurement.hpp: measurement_id,
 * geometry_id, local_key, local0, local1, ...): local_position = (local0,
 * local1), surface_link = geometry_id as written (the reference maps the
 * ACTS geometry id to a detray barcode through the detector description,
 * which is not part of this library), dimensions from local_key as
 * make_measurement_edm.cpp:36-52 decodes it (bit 1: loc0 active, bit 2:
 * loc1 active; inactive local coordinates are 0).  Host memory. */
seedgb_status seedgb_csv_read_measurements(const char* meas_path, uint64_t capacity,
                                           float* local_position, uint64_t* surface_link,
                                           uint8_t* dimensions, uint64_t* n);

/* ------------------------------------------------------------------------ */
/* Batched, graph-captured launches.  No counterpart in the reference, which */
/* overlaps events with one CUDA stream per host thread (throughput_mt.ipp:  */
/* 171-179); here a whole batch of uneven events runs as one captured launch */
/* sequence whose persistent seeding kernel load-balances across events.     */
/* ------------------------------------------------------------------------ */

/* Capture the launch sequence (descriptor copy, counter reset, the seven
 * kernels) for batches of up to max_events events with up to
 * max_total_spacepoints spacepoints together.  Grids are sized for that
 * capacity; the kernels read the batch's actual sizes from device memory, so
 * one captured graph serves every batch within it.  Allocates the arena for
 * the capacity; later runs within it allocate nothing. */
seedgb_status seedgb_seeding_graph_create(seedgb_seeding* h, uint32_t max_events,
                                          uint64_t max_total_spacepoints);

/* Same contract and output as seedgb_seeding_run_batch, through the captured
 * graph: one cudaGraphLaunch per batch.  SEEDGB_SIZE_LIMIT when the batch
 * exceeds the captured capacity.  Two graph slots alternate, so the host
 * prepares batch k+1 while batch k runs; it waits only for batch k-1.
 * Changing the options or the tuning re-captures on the next launch. */
seedgb_status seedgb_seeding_graph_launch(seedgb_seeding* h,
                                          const seedgb_spacepoint_view* events,
                                          uint32_t n_events, seedgb_seed_buffer* outs,
                                          void* stream);

/* Launch shape of the seeding kernel (the autotuner's search space).  No
 * counterpart in the reference.  warps_per_cta is clamped to what fits in
 * shared memory with the given neighbourhood capacity (read it back with
 * seedgb_seeding_get_tune).  Results do not depend on the tuning. */
typedef struct {
    int32_t warps_per_cta;          /* 1..16: warps (middle spacepoints in flight) per CTA */
    int32_t middles_per_item;       /* 1..4096: middle spacepoints per work item */
    int32_t neighbourhood_capacity; /* 256..8192: spacepoints staged in shared memory */
    int32_t ctas_per_sm;            /* 1..8: resident CTAs per SM of the persistent grid */
} seedgb_tune;
seedgb_status seedgb_seeding_set_tune(seedgb_seeding* h, const seedgb_tune* t);
seedgb_status seedgb_seeding_get_tune(seedgb_seeding* h, seedgb_tune* t);

/* The autotuner (no counterpart in the reference): for the batch `events`
 * (device views; seeds into `outs`), sets each candidate shape (NULL: the
 * default grid of 3 x 5 x 4 x 2 shapes -- warps {8, 12, 16}, middles per item
 * {64, 256, 384, 512, 1024}, neighbourhood {1536, 2048, 2560, 3072}, CTAs per SM
 * {1, 2}), captures the graph for the batch and times `reps` launches with
 * CUDA events on `stream` (median, after one warm-up launch).  Shapes that do
 * not fit in shared memory, or that are clamped to a shape already measured,
 * are skipped (times_ms[i] = -1; times_ms may be NULL, else n_candidates --
 * or 120 for the default grid -- entries).  Leaves the fastest shape set (and
 * in *best) with the graph captured for the batch.  Every measured launch
 * must end with status OK.  Synchronises `stream`. */
seedgb_status seedgb_seeding_autotune(seedgb_seeding* h, const seedgb_spacepoint_view* events,
                                      uint32_t n_events, seedgb_seed_buffer* outs,
                                      const seedgb_tune* candidates, uint32_t n_candidates,
                                      uint32_t reps, seedgb_tune* best, float* times_ms,
                                      void* stream);

/* ------------------------------------------------------------------------ */
/* Learned doublet filter.  No counterpart in the reference.                 */
/*                                                                          */
/* For every middle spacepoint with both middle-bottom and middle-top       */
/* doublets (after all doublet cuts), each doublet is described by 8        */
/* features, computed in float arithmetic without contraction:             */
/*   0 r_m  1 z_m  2 r_o - r_m  3 z_o - z_m  4 cot(theta) of the doublet's  */
/*   lin_circle  5 y / |dxy| in the lin_circle's frame (the sine of the     */
/*   doublet's azimuthal angle to the middle spacepoint's radial direction) */
/*   6 the lin_circle's z-intercept Zo  7 layer-pair id = band(r_m) *       */
/*   (n_edges + 1) + band(r_o), band(r) = number of edges <= r              */
/* and scored by an MLP 8 -> 32 -> 32 -> 1 on the tensor cores: inputs     */
/* (f - mu) * isd rounded to bf16, bf16 weights, fp32 biases and            */
/* accumulation, ReLU, bf16 hidden activations, a logit out.  Doublets of   */
/* a role the filter may prune are dropped when logit < threshold[role]     */
/* (role 0 middle-bottom, 1 middle-top); the unchanged triplet finding and  */
/* seed filtering run on the survivors.  Per event, when the pruned         */
/* fraction of the scored doublets lies outside [band[0], band[1]], the     */
/* event is seeded again without the filter inside the same launch          */
/* sequence (fallback).                                                      */
/*                                                                          */
/* prune_top = SEEDGB_FILTER_GATE_MIDDLE gates whole middles instead: a     */
/* middle none of whose middle-top doublets reaches threshold[1] yields no  */
/* seed (its middle-top doublets count as pruned), every other middle is   */
/* seeded with all its doublets.  The reference selects seeds per middle   */
/* from that middle's triplets alone (core/src/seeding/seed_finding.cpp:    */
/* 76-116), so the gated output is a subset of the plain seeds by           */
/* construction.                                                             */
/* ------------------------------------------------------------------------ */
#define SEEDGB_FILTER_KEEP 0u           /* score only */
#define SEEDGB_FILTER_PRUNE_DOUBLETS 1u /* drop doublets below the threshold */
#define SEEDGB_FILTER_GATE_MIDDLE 2u    /* prune_top only: gate whole middles */
typedef struct {
    float mu[8], isd[8];
    float w1[8 * 32];   /* [input][output], rounded to bf16 when loaded */
    float b1[32];
    float w2[32 * 32];  /* [input][output] */
    float b2[32];
    float w3[32];
    float b3;
    float threshold[2];
    uint32_t n_edges;   /* <= 15 */
    float edges[15];    /* ascending radial band edges (mm) */
    uint32_t prune_bottom, prune_top; /* SEEDGB_FILTER_* */
    float band[2];
    /* Optional per-event-size classes (n_size_classes <= 8; 0: threshold and
     * band above apply to every event).  An event with n spacepoints belongs
     * to the first class k with n <= size_class_max[k] (ascending), else to
     * the last; its thresholds and band are that class's. */
    uint32_t n_size_classes;
    uint32_t size_class_max[8];
    float size_class_threshold[8][2];
    float size_class_band[8][2];
    /* Middle gate only: a middle with more than gate_max_tops middle-top
     * doublets is always kept, unscored (0: every middle is scored).  Middles
     * without a seed are nearly all small (on the 100k-spacepoint events 96 %
     * of them have at most 32 middle-top doublets, together 0.7 % of the
     * doublet pairs), so the limit keeps almost every gating opportunity and
     * spares the large middles the scoring. */
    uint32_t gate_max_tops;
} seedgb_doublet_filter;

/* Install (copy) a filter on the handle, or remove it with f == NULL. */
seedgb_status seedgb_seeding_set_filter(seedgb_seeding* h, const seedgb_doublet_filter* f);

/* Record every scored doublet of the following runs into `records` (device
 * memory, `capacity` records of 48 bytes: uint32 middle, uint32 other,
 * uint32 role | event << 1, float features[8], float logit; indices are the
 * event's spacepoint indices).  Scoring needs an installed filter (with
 * prune flags 0 the seeds stay those of plain seeding).  records == NULL
 * stops recording.  Records are written in no particular order. */
seedgb_status seedgb_seeding_set_doublet_dump(seedgb_seeding* h, void* records,
                                              uint64_t capacity);

/* Record every triplet (before seed filtering) of the middles the filter
 * scores into `records` (device memory, `capacity` records of 16 bytes:
 * uint32 middle, bottom, top, event; the event's spacepoint indices).  With
 * an installed filter that prunes nothing, these are the triplets of plain
 * seeding: a doublet in none of them can change no seed (the training
 * label).  records == NULL stops recording. */
seedgb_status seedgb_seeding_set_triplet_dump(seedgb_seeding* h, void* records,
                                              uint64_t capacity);

/* After a run (synchronises `stream`): per event {scored middle-bottom,
 * pruned middle-bottom, scored middle-top, pruned middle-top} into
 * per_event[4 * n_events], 1 in fell_back[e] if event e was re-seeded
 * without the filter (either may be NULL), and the numbers of doublet and
 * triplet records the run produced (may exceed the dump capacities). */
seedgb_status seedgb_seeding_filter_stats(seedgb_seeding* h, uint32_t n_events,
                                          uint32_t* per_event, uint8_t* fell_back,
                                          uint64_t* n_records, uint64_t* n_triplet_records,
                                          void* stream);

/* Host drivers of the filter for C++ callers (no counterpart in the
 * reference).  Training: plain seeding of the events on this handle, in
 * passes of events_per_pass, with the doublet dump on; every middle-top
 * doublet of a middle with both roles is a sample, labelled 1 when it is the
 * (middle, top) pair of an accepted seed; all positives and a share
 * neg_keep of the negatives (chosen by a hash of seed, event, middle and
 * partner) are kept; inputs standardised over the samples; He-uniform
 * initial weights; `epochs` epochs of mini-batch Adam (lr, 0.9, 0.999, 1e-8)
 * on the weighted logistic loss (positives weighted by the negative /
 * positive ratio) with seedgb_mlp_grad / seedgb_mlp_adam, the samples
 * shuffled every epoch.  The same events, configuration and seed give the
 * same network bit for bit.  *out receives the network, the band edges,
 * thresholds -inf, band [0, 1], prune_top = SEEDGB_FILTER_GATE_MIDDLE and
 * gate_max_tops = 32.
 * loss_per_epoch (may be NULL): `epochs` mean losses.  Allocates its own
 * device buffers and synchronises `stream`. */
typedef struct {
    uint32_t epochs;          /* >= 1, e.g. 4 */
    uint32_t batch;           /* samples per step, e.g. 16384 */
    float learning_rate;      /* e.g. 3e-3 */
    float neg_keep;           /* share of the negative doublets kept, e.g. 0.05 */
    uint64_t seed;
    uint32_t events_per_pass; /* events seeded per dump pass, e.g. 8 */
} seedgb_filter_train_config;
seedgb_status seedgb_filter_train(seedgb_seeding* h, const seedgb_spacepoint_view* events,
                                  uint32_t n_events, const float* band_edges, uint32_t n_edges,
                                  const seedgb_filter_train_config* cfg,
                                  seedgb_doublet_filter* out, float* loss_per_epoch,
                                  void* stream);

/* Calibration of the middle gate on held-out events: one scored plain run
 * gives every middle's best middle-top logit and plain seed count, from
 * which the gate's seed recall at any threshold follows exactly (a gated run
 * keeps precisely the plain seeds of the middles it keeps).  Per size class
 * (class_max ascending, n_classes <= 8; 0: one class), the highest threshold
 * whose recall over the class's events is >= target and >= min_event on each
 * of them (middles above f->gate_max_tops middle-top doublets count as kept); the band is the class's range of gated middle-top fractions
 * widened by `margin`.  *f (the network, in) gets thresholds, bands, size
 * classes and prune_top = SEEDGB_FILTER_GATE_MIDDLE.  recall_out /
 * pruned_out (may be NULL): per event, the calibrated recall and gated
 * fraction.  Synchronises `stream`. */
seedgb_status seedgb_filter_calibrate_gate(seedgb_seeding* h, const seedgb_spacepoint_view* events,
                                           uint32_t n_events, const uint32_t* class_max,
                                           uint32_t n_classes, float target, float min_event,
                                           float margin, seedgb_doublet_filter* f,
                                           float* recall_out, float* pruned_out, void* stream);

/* Training and stand-alone inference of the network on the tensor cores.
 * params: device fp32 block of seedgb_mlp_num_params() values laid out as
 * w1[8][32], b1[32], w2[32][32], b2[32], w3[32], b3 (bf16-rounded when
 * used); norm: device {mu[8], isd[8]}; features: device n x 8 floats
 * (16-byte aligned); labels: device n floats in {0, 1}. */
uint32_t seedgb_mlp_num_params(void);
seedgb_status seedgb_mlp_forward(const float* params, const float* norm,
                                 const float* features, uint32_t n, float* logits,
                                 void* stream);
/* grad (device, num_params floats) and loss (device, 1 float) are
 * overwritten with the gradient and value of the mean weighted logistic loss
 * -(p y log s(z) + (1 - y) log(1 - s(z))), p = pos_weight.  The sums run in a
 * fixed order (no atomics): the same inputs give bit-identical results on
 * the same device.  Keeps a per-thread device scratch of one gradient row per
 * SM, allocated on the first call. */
seedgb_status seedgb_mlp_grad(const float* params, const float* norm,
                              const float* features, const float* labels, uint32_t n,
                              float pos_weight, float* grad, float* loss, void* stream);
/* One Adam step (bias-corrected, step >= 1) on n parameters. */
seedgb_status seedgb_mlp_adam(float* params, const float* grad, float* m, float* v,
                              uint32_t n, uint32_t step, float lr, float beta1,
                              float beta2, float eps, void* stream);

/* ------------------------------------------------------------------------ */
/* Track parameter estimation                                                */
/* ------------------------------------------------------------------------ */

typedef struct seedgb_params seedgb_params;

/* Replaces seed_parameter_estimation_algorithm(config, mr, copy, stream)
 * (seed_parameter_estimation_algorithm.hpp:33-37). */
seedgb_status seedgb_params_create(
    const seedgb_track_params_estimation_config* cfg, seedgb_params** out);
seedgb_status seedgb_params_destroy(seedgb_params* h);

/* Replaces operator()(magnetic_field, measurements, spacepoints, seeds)
 * (seed_parameter_estimation_algorithm.hpp:48-67) for a constant field
 * bfield = {Bx, By, Bz} in GeV/(e mm).  One parameter set per seed, in seed
 * order; reads the seed count from seeds->size on the device. */
seedgb_status seedgb_params_run(seedgb_params* h, const float bfield[3],
                                const seedgb_measurement_view* meas,
                                const seedgb_spacepoint_view* sps,
                                const seedgb_seed_buffer* seeds,
                                seedgb_params_buffer* out, void* stream);

/* n_events calls of seedgb_params_run in one launch (no counterpart in the
 * reference, whose operator() takes one event): element e of each host
 * array describes event e.  Same results as the per-event calls.  The
 * descriptors travel in one copy from a pinned buffer of the handle (two
 * used in turn: the call waits only for the copy of the call before the
 * previous one).  One stream per handle.  SEEDGB_SIZE_LIMIT above 65535
 * events. */
seedgb_status seedgb_params_run_batch(seedgb_params* h, const float bfield[3],
                                      const seedgb_measurement_view* meas,
                                      const seedgb_spacepoint_view* sps,
                                      const seedgb_seed_buffer* seeds,
                                      seedgb_params_buffer* outs, uint32_t n_events,
                                      void* stream);

/* ------------------------------------------------------------------------ */
/* Hand-off to the combinatorial Kalman filter                               */
/* ------------------------------------------------------------------------ */

/* The record the reference's track finding takes as seeds:
 * bound_track_parameters_collection_types::buffer, whose element is detray's
 * bound_track_parameters over the array algebra
 * (core/include/traccc/edm/track_parameters.hpp:29-49; consumed by
 * combinatorial_kalman_filter_algorithm at
 * examples/run/cuda/src/full_chain_algorithm.cpp:241-247).  detray is not
 * vendored, so this layout follows its published definition and is NOT
 * pinned against a build of it: the bound parameter vector (a 6 x 1 matrix:
 * loc0, loc1, phi, theta, q/p, time), the surface barcode (64 bits), then the
 * 6 x 6 covariance as the array algebra stores matrices, an array of columns
 * (element (row, col) at covariance[col * 6 + row]). */
typedef struct {
    float vector[6];
    uint64_t barcode;
    float covariance[36];
} seedgb_ckf_bound_track_parameters;

/* Converts a parameter buffer (seedgb_params_run / _run_batch output) into
 * the CKF's record layout on the device, keeping the parameters device-
 * resident: reads the count from in->size on the device, writes
 * min(count, capacity) records to `out` (device, 16-byte aligned) and that
 * number to *out_size (device; may be NULL).  Asynchronous on `stream`; one
 * launch, no host synchronisation (graph-capturable like the seeding
 * launches).  No counterpart in the reference, which estimates parameters
 * directly in this layout. */
seedgb_status seedgb_params_to_ckf(const seedgb_params_buffer* in,
                                   seedgb_ckf_bound_track_parameters* out, uint32_t capacity,
                                   uint32_t* out_size, void* stream);

/* ------------------------------------------------------------------------ */

/* ------------------------------------------------------------------------ */
/* Binning without device allocation                                         */
/* ------------------------------------------------------------------------ */

/* Largest event and fixed device scratch of seedgb_spacepoint_binning_noalloc.
 * The scratch is a static array in the library's device image: every GPU that
 * loads the library holds SEEDGB_NOALLOC_SCRATCH_BYTES (768.25 KiB) until the
 * process exits. */
#define SEEDGB_NOALLOC_MAX_SPACEPOINTS 65536u
#define SEEDGB_NOALLOC_SCRATCH_BYTES (256u + 4u * 65536u + 4u * 32u * 4096u)

/* No counterpart in the reference.  Bins one event into the phi-z grid like
 * the reference's spacepoint binning and this library's seeding path
 * (seedgb_seeding_copy_grid gives the same grid), without allocating device
 * memory: for callers that cannot call cudaMalloc on their event path -- code
 * running during stream capture, trigger processes that reserve all memory
 * at start-up, plugins of frameworks that own every device allocation.
 *
 *   sps          device spacepoint columns, at most
 *                SEEDGB_NOALLOC_MAX_SPACEPOINTS (else SEEDGB_SIZE_LIMIT)
 *   bin_offsets  device, nbins + 1 entries (nbins = phi bins x z bins of
 *                get_axes, at most 4096, else SEEDGB_SIZE_LIMIT): CSR offsets
 *   bin_sps      device, >= sps->size entries: spacepoint indices, bins in
 *                serial order, ascending index inside a bin
 *
 * Returns SEEDGB_BAD_CONFIG, before launching anything, when the grid's phi
 * axis cannot place every phi the finder accepts (a grid phi range much
 * narrower than the finder's: ibin = int((phi - min) / (max - min) * n)
 * outside [-n, 2n) at an end of the finder's range); such spacepoints would
 * otherwise be left out of the grid.
 *
 * Asynchronous on `stream`.  The kernel's scratch is one static device array
 * shared by every call, which keeps the last call's contents (the kernel
 * clears what must start at zero): calls that overlap on the GPU -- on two
 * streams, or from two host threads -- race and corrupt each other's result;
 * serialise them.  Every call made outside stream capture looks up the
 * array's device address (cudaGetSymbolAddress) with the current device;
 * a call during capture reuses the address found by the last call outside
 * capture on that device, so make a first call on each device before any
 * stream capture (and again after a device reset).  Device ordinals of 64 or
 * more get SEEDGB_UNSUPPORTED.  Allocates nothing: no cudaMalloc, no
 * cudaFree. */
seedgb_status seedgb_spacepoint_binning_noalloc(
    const seedgb_seedfinder_config* finder, const seedgb_spacepoint_grid_config* grid,
    const seedgb_spacepoint_view* sps, uint32_t* bin_offsets, uint32_t* bin_sps,
    void* stream);

/* ------------------------------------------------------------------------ */
/* GBTS seeding (graph-based track seeding)                                  */
/* ------------------------------------------------------------------------ */

/* traccc::gbts_seedfinder_config (core/include/traccc/gbts_seeding/
 * gbts_seeding_config.hpp:67-276): the per-kernel parameter structs
 * flattened in declaration order, the config's scalars, then the bit layout
 * of the measurements' surface barcode (volume = (link >> volume_shift) &
 * (2^volume_bits - 1), surface index likewise; the defaults are detray's
 * barcode layout, volume in bits 52-63 and surface index in bits 27-47). */
typedef struct {
    /* gbts_sort_nodes_params */
    float tMin_slope, offset, tMax_min, tMax_correction, tMax_slope, maxTau;
    int32_t useTauLUT;
    float tau_lut_inv_bin;
    uint32_t tauLutSize;
    /* gbts_make_graph_edges_params */
    float minDeltaRadius, min_z0, max_z0, maxOuterRadius, tau_roi, cut_zMinU, cut_zMaxU,
        max_Kappa, low_Kappa_d0, high_Kappa_d0;
    /* gbts_match_graph_edges_params */
    float cut_dphi_max, cut_dcurv_max, cut_tau_ratio_max;
    /* gbts_dphi_window_params */
    float min_delta_phi, dphi_coeff, min_delta_phi_low_dr, dphi_coeff_low_dr,
        low_dr_threshold;
    /* gbts_count_spacepoints_by_layer_params */
    float type1_max_width;
    int32_t doTauCut;
    /* gbts_fit_segments_params */
    float sigmaMS, radLen, sigma_x, sigma_y, weight_x, weight_y, maxDChi2_x, maxDChi2_y,
        add_hit, qual_scale, inv_max_curvature;
    /* gbts_convert_seeds_params */
    int32_t use_dropout;
    float dropout_dcurv_m, force_dropout_max_curv_m, best_hit_frac, tight_bid_cot_threshold;
    /* gbts_seedfinder_config scalars */
    uint32_t n_phi_bins, max_num_neighbours, minLevel, max_edges_factor, edge_bidding_rounds;
    /* surface barcode layout */
    uint32_t volume_shift, volume_bits, index_shift, index_bits;
} seedgb_gbts_config;

/* One layer of gbts_layerInfo (gbts_seeding_config.hpp:24-44): type (0
 * barrel, 1 / 2 end-caps), first eta bin and number of eta bins, minimum eta
 * and eta bin width. */
typedef struct {
    int32_t type;
    uint32_t eta_bin0, n_eta_bins;
    float min_eta, eta_bin_width;
} seedgb_gbts_layer;

/* One (detray geometry id, layer) pair of the geometry-id binning. */
typedef struct {
    uint64_t barcode;
    int32_t layer;
} seedgb_gbts_geoid;

/* The reference's defaults (gbts_seeding_config.hpp member initialisers). */
void seedgb_gbts_config_default(seedgb_gbts_config* c);

typedef struct seedgb_gbts seedgb_gbts;

/* Replaces gbts_seedfinder_config::setLinkingScheme(binTables, layerInfo,
 * geoIDBinning, minPt) (core/src/gbts_seeding/gbts_seeding_config.cpp:19-142)
 * followed by the construction of traccc::cuda::gbts_seeding_algorithm(config,
 * mr, copy, stream) (device/cuda/include/traccc/cuda/gbts_seeding/
 * gbts_seeding_algorithm.hpp).  `bin_pairs` holds n_pairs (bin1, bin2) pairs,
 * the linked layer-eta bins already unrolled; `tau_lut` (n_tau_lut floats,
 * a multiple of 5) is used when config->useTauLUT is set, else may be NULL.
 * The pT-dependent cuts of the config are scaled by 900 MeV / min_pt (MeV),
 * as setLinkingScheme does.  SEEDGB_BAD_CONFIG where setLinkingScheme returns
 * false, and for tables the kernels cannot index (a layer index outside the
 * layer table, a bin pair outside the eta bins, a malformed tau table) or
 * more than 49 bidding rounds. */
seedgb_status seedgb_gbts_create(const seedgb_gbts_config* config,
                                 const seedgb_gbts_layer* layers, uint32_t n_layers,
                                 const uint32_t* bin_pairs, uint32_t n_pairs,
                                 const seedgb_gbts_geoid* geoids, uint32_t n_geoids,
                                 float min_pt, const float* tau_lut, uint32_t n_tau_lut,
                                 seedgb_gbts** out);
seedgb_status seedgb_gbts_destroy(seedgb_gbts* h);

/* The config after setLinkingScheme's scaling, and the sizes of the derived
 * tables (eta bins, volume map entries, surface map entries). */
seedgb_status seedgb_gbts_get_config(const seedgb_gbts* h, seedgb_gbts_config* config,
                                     uint32_t* n_eta_bins, uint32_t* n_volumes,
                                     uint32_t* n_surfaces);

/* Replaces edm::seed_collection::buffer operator()(spacepoints, measurements)
 * (device/common/include/traccc/gbts_seeding/device/gbts_seeding_algorithm.
 * hpp:94-96).  surface_link / diameter: device measurement columns (n_meas
 * entries) indexed by the spacepoints' measurement_index_1.  Seeds (bottom =
 * innermost, top = outermost spacepoint, quality = the path's fit quality)
 * are written in a canonical order: by seed proposal (path-store order), up
 * to three per proposal in the reference's emission order; the reference's
 * own order depends on its atomics.  Enqueued on `stream`; the call waits
 * once for the device in the middle (to size the path store, as the
 * reference reads its path counts back) and returns with the rest in flight.
 * A seed buffer smaller than the result is filled to capacity and the status
 * reports SEEDGB_CAPACITY_OVERFLOW. */
seedgb_status seedgb_gbts_run(seedgb_gbts* h, const seedgb_spacepoint_view* sps,
                              const uint64_t* surface_link, const float* diameter,
                              uint32_t n_meas, seedgb_seed_buffer* out, void* stream);

/* Many events in one call, the same seeds as one seedgb_gbts_run per event:
 * event e is (events[e], surface_links[e], diameters[e], n_meas[e]) ->
 * outs[e].  All work stays in order on `stream`; the call enqueues event
 * e + 1's kernels before it waits for event e's path-store size, so the GPU
 * keeps working while the host waits (two events' work areas are kept). */
seedgb_status seedgb_gbts_run_batch(seedgb_gbts* h, const seedgb_spacepoint_view* events,
                                    const uint64_t* const* surface_links,
                                    const float* const* diameters, const uint32_t* n_meas,
                                    uint32_t n_events, seedgb_seed_buffer* outs, void* stream);

/* Synchronise `stream` and return the worst device status of the last call
 * (over all events of a batch). */
seedgb_status seedgb_gbts_last_status(seedgb_gbts* h, void* stream);

/* Counters of the last event (synchronises the handle's last stream): nodes,
 * edges created, edge connections, connected edges, terminus edges, path
 * store entries below the terminus edges, seed proposals, proposals rejected
 * by the bidding, seeds. */
#define SEEDGB_GBTS_N_COUNTERS 9u
seedgb_status seedgb_gbts_counters(seedgb_gbts* h, uint64_t* counters);

/* The reference's GBTS configuration directory (examples/options/src/
 * track_gbts_seeding.cpp:158-226): geoidBinning.txt, binTables.txt and
 * layerInfo.txt.  Call with NULL arrays to get the counts, then with arrays
 * of at least those sizes; bin_pairs gets 2 * n_pairs entries.  SEEDGB_
 * INVALID_ARGUMENT when a file is missing or malformed. */
seedgb_status seedgb_gbts_read_config_dir(const char* dir, seedgb_gbts_layer* layers,
                                          uint32_t* n_layers, uint32_t* bin_pairs,
                                          uint32_t* n_pairs, seedgb_gbts_geoid* geoids,
                                          uint32_t* n_geoids);

const char* seedgb_status_string(seedgb_status s);
uint32_t seedgb_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
