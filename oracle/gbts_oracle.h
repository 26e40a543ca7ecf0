/* CPU oracle of traccc's GBTS seeding (graph-based track seeding).
 *
 * TEST INFRASTRUCTURE ONLY: the tests, the smoke check and bench.py's CPU
 * baseline call it as the checker; the product library never links it.
 *
 * The reference implements GBTS only as device kernels
 * (the .ipp files of device/common/include/traccc/gbts_seeding/device/impl, driven by
 * device/common/src/gbts_seeding/gbts_seeding_algorithm.cpp); it has no host
 * implementation and no tests, so this restatement is "parity unpinned": it
 * follows the kernels' arithmetic expression for expression, and fixes one
 * canonical order wherever the reference's result depends on the order in
 * which its atomics land (node order inside an (eta, phi) cell, edge order,
 * the link lists, the connected-edge numbering, the path store, the order of
 * the seed proposals and of the output seeds).
 */
#ifndef GBTS_ORACLE_H
#define GBTS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* gbts_seedfinder_config and its per-kernel parameter structs
 * (core/include/traccc/gbts_seeding/gbts_seeding_config.hpp:67-276), flattened;
 * plus the bit layout of the surface barcode (volume and surface index). */
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
    float min_delta_phi, dphi_coeff, min_delta_phi_low_dr, dphi_coeff_low_dr, low_dr_threshold;
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
    /* surface barcode layout: volume = (link >> volume_shift) & (2^volume_bits - 1),
     * surface index = (link >> index_shift) & (2^index_bits - 1) */
    uint32_t volume_shift, volume_bits, index_shift, index_bits;
} or_gbts_config;

/* The linking scheme after gbts_seedfinder_config::setLinkingScheme
 * (core/src/gbts_seeding/gbts_seeding_config.cpp:19-142). */
typedef struct {
    uint32_t n_layers;
    const int8_t* layer_type;
    const uint32_t* eta_bin0;
    const uint32_t* n_eta;
    const float* min_eta;
    const float* eta_width;
    uint32_t n_pairs;
    const uint32_t* pairs; /* [bin1, bin2] per pair */
    uint32_t n_volumes;
    const int16_t* volume_map;
    uint32_t n_surfaces;
    const uint32_t* surface_map; /* [surface index, layer] per entry */
    uint32_t n_tau_lut;
    const float* tau_lut;
    uint32_t n_eta_bins;
} or_gbts_tables;

/* Counters of one run (the reference's gbts_counter, plus nodes and seeds). */
enum {
    OR_GBTS_NODES = 0,
    OR_GBTS_EDGES,            /* edges created (before the nMaxEdges cap) */
    OR_GBTS_CONNECTIONS,      /* edge-to-edge links */
    OR_GBTS_CONNECTED_EDGES,  /* edges kept for the CCA */
    OR_GBTS_TERMINUS,         /* terminus edges */
    OR_GBTS_PATHS,            /* path-store entries below the terminus edges */
    OR_GBTS_PROPS,            /* seed proposals */
    OR_GBTS_REJECTED,         /* proposals rejected by the bidding */
    OR_GBTS_SEEDS,            /* output seeds */
    OR_GBTS_N_COUNTERS
};

/* The reference defaults (gbts_seeding_config.hpp member initialisers) and the
 * detray barcode layout (volume in bits 52-63, surface index in bits 27-47). */
void or_gbts_config_default(or_gbts_config* c);

/* setLinkingScheme: geometry-id binning (barcode, layer) pairs -> volume map
 * and surface map; scales the pT-dependent cuts of `c` by 900 MeV / minPt.
 * `geoid` / `geoid_layer` are copied and sorted internally.  volume_map must
 * hold 2 * (largest volume + 1) entries, surface_map 2 * (n + 1).  Returns 0,
 * or -1 when the reference's checks fail. */
int or_gbts_linking(or_gbts_config* c, float minPt, const uint64_t* geoid,
                    const int16_t* geoid_layer, uint32_t n, int16_t* volume_map,
                    uint32_t volume_cap, uint32_t* n_volumes, uint32_t* surface_map,
                    uint32_t surface_cap, uint32_t* n_surfaces);

typedef struct {
    uint32_t bottom, middle, top;
    float quality;
} or_gbts_seed;

/* The whole chain on one event.  Spacepoints: xyz (3 floats each) and their
 * first measurement index; measurements: surface barcode and cluster
 * diameter.  Seeds go to `out` up to `cap`; `*n_out` gets the total.
 * Returns 0, or 1 when `cap` was too small, or 2 when a measurement index is
 * out of range (that spacepoint is skipped). */
int or_gbts_run(const or_gbts_config* c, const or_gbts_tables* t, uint32_t n_sp,
                const float* xyz, const uint32_t* meas_idx, uint32_t n_meas,
                const uint64_t* surface_link, const float* diameter, or_gbts_seed* out,
                uint64_t cap, uint64_t* n_out, uint64_t* counters);

#ifdef __cplusplus
}
#endif

#endif
