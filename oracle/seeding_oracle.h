/*
 * seeding_oracle.h -- CPU restatement of traccc's host triplet seeding and
 * track-parameter estimation.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GB300 seeding path.  Only the test-suite, the smoke check and the timed CPU
 * baseline of bench.py may load it; the product library never links or calls
 * it, and nothing in the product falls back to it.
 *
 * Every routine restates the reference algorithm in plain C, in the same
 * floating-point operation order as the reference (float arithmetic, no FMA
 * contraction: build with -O2 -ffp-contract=off).  Each function names the
 * reference file:line it follows.  Paths are relative to the traccc source
 * tree (traccc 1.6.0).
 *
 * Parity pins (tests/test_oracle_kat.py):
 *   - tests/cpu/test_seeding.cpp:35-181 (two 5-spacepoint muon events, exactly
 *     one seed each, with the same config tweaks);
 *   - tests/cpu/test_track_params_estimation.cpp:34-144 (helix spacepoints,
 *     |p - sqrt(2) GeV| < 2e-4 and the q/p sign);
 *   - tests/cpu/test_axis.cpp:26-87 and the circular-axis cases that follow
 *     (bin, range, zone and remap known answers).
 */
#ifndef SEEDING_ORACLE_H
#define SEEDING_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* traccc::seedfinder_config (core/include/traccc/seeding/detail/
 * seeding_config.hpp:17-139), field for field. */
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
    /* derived by or_finder_config_setup() */
    float highland, maxScatteringAngle2, pTPerHelixRadius, minHelixDiameter2,
        minHelixRadius, pT2perRadius;
    int32_t phiBinDeflectionCoverage;
    uint32_t neighbor_scope[2];
} or_finder_config;

/* traccc::spacepoint_grid_config (seeding_config.hpp:142-189). */
typedef struct {
    float bFieldInZ, minPt, rMax, zMax, zMin, deltaRMax, cotThetaMax, impactMax;
    float phiMin, phiMax;
    int32_t phiBinDeflectionCoverage;
} or_grid_config;

/* traccc::seedfilter_config (seeding_config.hpp:191-219). */
typedef struct {
    float deltaInvHelixDiameter, impactWeightFactor, compatSeedWeight, deltaRMin;
    uint64_t compatSeedLimit;
    float good_spB_min_radius, good_spB_weight_increase;
    float good_spT_max_radius, good_spT_weight_increase;
    float good_spB_min_weight, seed_min_weight, spB_min_radius;
} or_filter_config;

/* traccc::track_params_estimation_config
 * (core/include/traccc/seeding/detail/track_params_estimation_config.hpp:18-33) */
typedef struct {
    float initial_sigma[6];
    float initial_sigma_qopt;
    float initial_sigma_pt_rel;
    float initial_inflation[6];
} or_tp_config;

/* The two axes of the phi-z grid (axis2::circular / axis2::regular). */
typedef struct {
    uint32_t phi_bins;
    float phi_min, phi_max;
    uint32_t z_bins;
    float z_min, z_max;
} or_axes;

/* spacepoint_collection SoA (core/include/traccc/edm/spacepoint_collection.hpp:
 * 222-234): global is xyz interleaved (std::array<float,3>). */
typedef struct {
    const uint32_t* measurement_index_1;
    const uint32_t* measurement_index_2;
    const float* global;
    const float* z_variance;
    const float* radius_variance;
    uint32_t size;
} or_spacepoints;

/* The measurement columns that parameter estimation reads. */
typedef struct {
    const float* local_position; /* 2 floats per measurement */
    const uint64_t* surface_link;
    uint32_t size;
} or_measurements;

/* edm::seed (core/include/traccc/edm/seed_collection.hpp:28-146). */
typedef struct {
    uint32_t bottom, middle, top;
    float quality;
} or_seed;

/* bound_track_parameters: vector {loc0, loc1, phi, theta, qop, time},
 * diagonal-filled 6x6 covariance (row-major), surface link. */
typedef struct {
    uint64_t surface_link;
    float params[6];
    float cov[36];
} or_bound_params;

/* How the azimuth of a spacepoint is evaluated.
 *  OR_PHI_LIBM: atan2f of the C library, as the reference host code does.
 *  OR_PHI_CR  : the correctly rounded float atan2, i.e. the reference host code
 *               on a C library whose atan2f is correctly rounded. */
enum { OR_PHI_LIBM = 0, OR_PHI_CR = 1 };

/* Work counters and near-threshold counts of one seeding call. */
typedef struct {
    uint64_t n_sp, n_valid;
    uint64_t n_pair_tests;            /* (middle, neighbour) visits         */
    uint64_t n_mb, n_mt;              /* doublets                            */
    uint64_t n_middles_with_mb;       /* middles whose MT search ran         */
    uint64_t n_middles_both;          /* middles with MB and MT doublets     */
    uint64_t n_triplet_tests;         /* sum n_mb * n_mt                     */
    uint64_t n_triplets;              /* compatible triplets                 */
    uint64_t n_triplets_after_cut;    /* after the single-seed cut           */
    uint64_t n_seeds;
    uint64_t max_mb_per_middle, max_mt_per_middle, max_triplets_per_mb;
    uint64_t max_triplets_per_middle;
    uint64_t max_bin_size, max_neighbourhood;
    /* decisions whose deciding quantity lies within 1e-6 relative of its cut */
    uint64_t near_doublet_cuts, near_triplet_cuts, near_bin_edges;
    uint64_t phi_cr_undecided;        /* CR atan2 too close to a float midpoint */
    /* learned doublet filter (or_seeding_ex with a filter) */
    uint64_t n_scored_mb, n_scored_mt;  /* doublets of middles with both roles */
    uint64_t n_pruned_mb, n_pruned_mt;  /* of those, dropped by the filter     */
    /* algorithmic work: pairs passing the doublet window (first stage), and
     * the FP32 operations (+ - * / sqrt, one each) executed by the doublet
     * and triplet tests */
    uint64_t n_window_pairs, ops_doublet_tests, ops_triplet_tests;
} or_stats;

/* Config construction: defaults and setup() (seeding_config.hpp:19,120-138). */
void or_finder_config_default(or_finder_config* c);
void or_finder_config_setup(or_finder_config* c);
void or_grid_config_from_finder(or_grid_config* g, const or_finder_config* f);
void or_filter_config_default(or_filter_config* c);
void or_tp_config_default(or_tp_config* c);

/* get_axes (core/include/traccc/seeding/spacepoint_binning_helper.hpp:22-110).
 * Returns 0, or 1/2 for the two std::domain_error conditions. */
int or_get_axes(const or_grid_config* g, or_axes* out);

/* Axis primitives (core/include/traccc/seeding/grids/axis.hpp). */
uint32_t or_regular_bin(uint32_t n, float mn, float mx, float v);
void or_regular_range(uint32_t n, float mn, float mx, float v,
                      const uint32_t nh[2], uint32_t out[2]);
uint32_t or_regular_zone(uint32_t n, float mn, float mx, float v,
                         const uint32_t nh[2], uint32_t* out, uint32_t cap);
uint32_t or_circular_bin(uint32_t n, float mn, float mx, float v);
uint32_t or_circular_remap(uint32_t n, uint32_t ibin, int32_t shood);
void or_circular_range(uint32_t n, float mn, float mx, float v,
                       const uint32_t nh[2], uint32_t out[2]);
uint32_t or_circular_zone(uint32_t n, float mn, float mx, float v,
                          const uint32_t nh[2], uint32_t* out, uint32_t cap);

/* Spacepoint azimuth and validity (spacepoint_collection.ipp:52-63,
 * spacepoint_binning_helper.hpp:112-127). */
float or_sp_phi(float x, float y, int phi_mode, int* undecided);
int or_is_valid_sp(const or_finder_config* c, float x, float y, float z,
                   int phi_mode);

/* Binning (core/src/seeding/spacepoint_binning.cpp:27-53).
 * bin_offsets[nbins+1] (CSR), bin_sps[n_valid] = spacepoint indices. */
int or_binning(const or_finder_config* c, const or_axes* axes,
               const or_spacepoints* sps, int phi_mode, uint32_t* bin_offsets,
               uint32_t* bin_sps, uint32_t* n_valid, or_stats* stats);

/* Full host seeding (core/src/seeding/seeding_algorithm.cpp:24-28 ->
 * seed_finding.cpp:58-121).  Returns 0 on success, -1 if cap is too small
 * (n_out then holds the required size), >0 for config errors. */
int or_seeding(const or_finder_config* fc, const or_grid_config* gc,
               const or_filter_config* flt, const or_spacepoints* sps,
               int phi_mode, or_seed* out, uint32_t cap, uint32_t* n_out,
               or_stats* stats);

/* ------------------------------------------------------------------------ */
/* Learned doublet filter (no counterpart in the reference).                 */
/*                                                                          */
/* A doublet (middle m, other o) of a middle spacepoint that has both       */
/* middle-bottom and middle-top doublets is described by 8 features, in     */
/* float arithmetic without contraction:                                    */
/*   0 r_m   1 z_m   2 dr = r_o - r_m   3 dz = z_o - z_m                    */
/*   4 cot(theta) of the doublet's lin_circle (bottom-to-top direction)     */
/*   5 s = y * iDeltaR of the lin_circle's frame: the sine of the angle     */
/*     between the doublet and the middle spacepoint's radial direction    */
/*     (the azimuthal bending feature)                                       */
/*   6 z-intercept at r = 0 of the lin_circle (Zo)                           */
/*   7 layer-pair id = band(r_m) * (n_edges + 1) + band(r_o), band(r) =     */
/*     number of radial band edges <= r                                     */
/* The network is an MLP 8 -> 32 -> 32 -> 1: inputs standardised          */
/* ((f - mu) * isd) and rounded to bf16, bf16 weights, float biases and     */
/* accumulation (bias first, then inputs in index order), ReLU, hidden      */
/* activations rounded to bf16; the output is a logit.  A doublet is kept   */
/* when logit >= threshold[role] (role 0 middle-bottom, 1 middle-top).       */
/* ------------------------------------------------------------------------ */
#define OR_MLP_IN 8
#define OR_MLP_H 32
#define OR_MAX_BAND_EDGES 15
typedef struct {
    float mu[OR_MLP_IN], isd[OR_MLP_IN];
    float w1[OR_MLP_IN * OR_MLP_H];   /* [in][out], rounded to bf16 when used */
    float b1[OR_MLP_H];
    float w2[OR_MLP_H * OR_MLP_H];    /* [in][out] */
    float b2[OR_MLP_H];
    float w3[OR_MLP_H];
    float b3;
    float threshold[2];               /* keep when logit >= threshold[top] */
    uint32_t n_edges;
    float edges[OR_MAX_BAND_EDGES];   /* ascending radial band edges */
    uint32_t prune_bottom, prune_top; /* 0 keep, 1 drop doublets below the
                                       * threshold, 2 (prune_top only) gate
                                       * whole middles: no seed unless a
                                       * middle-top doublet reaches it */
    uint32_t gate_max_tops;           /* gate: middles with more middle-top
                                       * doublets are kept (0: no limit) */
} or_doublet_filter;

/* One scored doublet (dump of or_seeding_ex). */
typedef struct {
    uint32_t middle, other;
    uint32_t top;                     /* 0 middle-bottom, 1 middle-top */
    float feat[OR_MLP_IN];
    float logit;                      /* 0 when no filter was given */
} or_doublet_rec;

/* One triplet of a scored middle (dump of or_seeding_ex). */
typedef struct {
    uint32_t middle, bottom, top, event;
} or_triplet_rec;

float or_bf16_round(float x);
void or_doublet_features(int top, const float m[6], const float o[6],
                         const float lc[6], const or_doublet_filter* f,
                         float feat[OR_MLP_IN]);
float or_mlp_logit(const or_doublet_filter* f, const float feat[OR_MLP_IN]);

/* or_seeding with the learned filter: the doublets of every middle that has
 * both roles are scored, those below the threshold (of the roles the filter
 * may prune) dropped, and the unchanged triplet finding and seed filtering
 * run on the survivors.  filt == NULL: plain seeding.  dump != NULL: every
 * scored doublet is written (up to dump_cap; n_dump = the count).
 * tdump != NULL: every triplet (before seed filtering) of the middles that
 * have both roles is written (up to tdump_cap; n_tdump = the count). */
int or_seeding_ex(const or_finder_config* fc, const or_grid_config* gc,
                  const or_filter_config* flt, const or_spacepoints* sps,
                  int phi_mode, const or_doublet_filter* filt,
                  or_doublet_rec* dump, uint64_t dump_cap, uint64_t* n_dump,
                  or_triplet_rec* tdump, uint64_t tdump_cap, uint64_t* n_tdump,
                  or_seed* out, uint32_t cap, uint32_t* n_out, or_stats* stats);

/* Spacepoint formation (core/src/seeding/silicon_pixel_spacepoint_formation.hpp:
 * 31-60, core/include/traccc/seeding/impl/spacepoint_formation.ipp:20-47):
 * one spacepoint per 2-dimensional measurement, in measurement order, global
 * position = the surface's local_to_global.  Surfaces: type 0 plane,
 * (l0, l1) -> R (l0, l1, 0) + t; type 1 cylinder, (r phi, z) ->
 * R (r cos phi, r sin phi, z) + t with phi = l0 / radius (cos, sin in
 * double, rounded to float); each coordinate (R[i][0] a + R[i][1] b) +
 * R[i][2] c + t[i] in float.  (detray's algebra is not vendored: the
 * placement arithmetic is this definition; parity unpinned against detray.)
 * dims == NULL: all measurements are 2-dimensional.  Measurements whose
 * surface_link >= n_surfaces form no spacepoint.  Returns the count. */
typedef struct {
    uint32_t type;
    float radius;
    float rotation[9];
    float translation[3];
} or_surface;
uint32_t or_form_spacepoints(const or_surface* surfaces, uint32_t n_surfaces,
                             const or_measurements* meas, const uint8_t* dims,
                             uint32_t* mi1, uint32_t* mi2, float* global,
                             float* zvar, float* rvar);

/* Host track-parameter estimation (core/src/seeding/
 * track_params_estimation.cpp:23-91). */
int or_track_params(const or_tp_config* c, const or_measurements* meas,
                    const or_spacepoints* sps, const or_seed* seeds,
                    uint32_t n_seeds, const float bfield[3],
                    or_bound_params* out);

/* Doublet/triplet helpers, exposed for unit tests.
 * m/o = {x, y, z, r, var_z, var_r}. */
int or_doublet_compatible(int top, const float m[6], const float o[6],
                          const or_finder_config* c);
void or_transform_coordinates(int top, const float m[6], const float o[6],
                              float lc[6] /* Zo,cot,iDR,Er,U,V */);
int or_triplet_compatible(const float m[6], const float lb[6],
                          const float lt[6], const or_finder_config* c,
                          float iSinTheta2, float scatteringInRegion2,
                          float* curvature, float* impact);

#ifdef __cplusplus
}
#endif
#endif
