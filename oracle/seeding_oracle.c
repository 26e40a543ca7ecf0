/*
 * seeding_oracle.c -- CPU restatement of traccc's host triplet seeding and
 * track-parameter estimation.
 *
 * TEST INFRASTRUCTURE ONLY: the correctness oracle for the GB300 path (and
 * the timed CPU baseline of bench.py).  The product library never links or
 * calls this file.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (see oracle/Makefile).
 * All arithmetic is float, in the reference's expression order; no FMA.
 * File:line citations are into the traccc 1.6.0 source tree.
 */
#include "seeding_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* detray units as used by traccc (core/include/traccc/definitions/common.hpp:
 * 18-25 aliases detray::unit; detray is not vendored, these are its published
 * values: native units mm, GeV, e; T = GeV/(e*mm) * 0.000299792458;
 * time in mm of light travel). */
#define U_MM 1.f
#define U_MEV 1e-3f
#define U_GEV 1.f
#define U_T 0.000299792458f
#define U_DEGREE 0.017453292519943295f
#define U_NS 299.792458f
#define U_E 1.f

/* ------------------------------------------------------------------------ */
/* Configs                                                                   */
/* ------------------------------------------------------------------------ */

/* seedfinder_config::setup(), seeding_config.hpp:120-138. */
void or_finder_config_setup(or_finder_config* c) {
    c->highland = 13.6f * U_MEV * sqrtf(c->radLengthPerSeed) *
                  (1.f + 0.038f * logf(c->radLengthPerSeed));
    float maxScatteringAngle = c->highland / c->minPt;
    c->maxScatteringAngle2 = maxScatteringAngle * maxScatteringAngle;
    c->pTPerHelixRadius = c->bFieldInZ;
    c->minHelixDiameter2 = powf(c->minPt * 2.f / c->pTPerHelixRadius, 2.f);
    c->minHelixRadius = sqrtf(c->minHelixDiameter2) / 2.f;
    c->pT2perRadius = powf(c->highland / c->pTPerHelixRadius, 2.f);
}

/* seedfinder_config defaults, seeding_config.hpp:19-118. */
void or_finder_config_default(or_finder_config* c) {
    memset(c, 0, sizeof(*c));
    c->zMin = -2000.f * U_MM;
    c->zMax = 2000.f * U_MM;
    c->rMax = 200.f * U_MM;
    c->rMin = 33.f * U_MM;
    c->collisionRegionMin = -250 * U_MM;
    c->collisionRegionMax = +250 * U_MM;
    c->phiMin = (float)(-M_PI);
    c->phiMax = (float)(M_PI);
    c->minPt = 500.f * U_MEV;
    c->cotThetaMax = 27.2845f;
    c->deltaRMin = 20 * U_MM;
    c->deltaRMax = 80 * U_MM;
    c->deltaZMax = 450 * U_MM;
    c->impactMax = 10.f * U_MM;
    c->sigmaScattering = 3.0f;
    c->maxPtScattering = 10.f * U_GEV;
    c->maxSeedsPerSpM = 5;
    c->bFieldInZ = 1.99724f * U_T;
    c->beamPos[0] = -.0f * U_MM;
    c->beamPos[1] = -.0f * U_MM;
    c->radLengthPerSeed = 0.05f;
    c->zAlign = 0 * U_MM;
    c->rAlign = 0 * U_MM;
    c->sigmaError = 5;
    c->phiBinDeflectionCoverage = 1;
    c->neighbor_scope[0] = 1;
    c->neighbor_scope[1] = 1;
    or_finder_config_setup(c);
}

/* spacepoint_grid_config(const seedfinder_config&), seeding_config.hpp:146-157 */
void or_grid_config_from_finder(or_grid_config* g, const or_finder_config* f) {
    g->bFieldInZ = f->bFieldInZ;
    g->minPt = f->minPt;
    g->rMax = f->rMax;
    g->zMax = f->zMax;
    g->zMin = f->zMin;
    g->deltaRMax = f->deltaRMax;
    g->cotThetaMax = f->cotThetaMax;
    g->impactMax = f->impactMax;
    g->phiMin = f->phiMin;
    g->phiMax = f->phiMax;
    g->phiBinDeflectionCoverage = f->phiBinDeflectionCoverage;
}

/* seedfilter_config defaults, seeding_config.hpp:191-219. */
void or_filter_config_default(or_filter_config* c) {
    c->deltaInvHelixDiameter = 0.00003f / U_MM;
    c->impactWeightFactor = 1.f;
    c->compatSeedWeight = 200.f;
    c->deltaRMin = 5.f * U_MM;
    c->compatSeedLimit = 2;
    c->good_spB_min_radius = 150.f * U_MM;
    c->good_spB_weight_increase = 400.f;
    c->good_spT_max_radius = 150.f * U_MM;
    c->good_spT_weight_increase = 200.f;
    c->good_spB_min_weight = 380.f;
    c->seed_min_weight = 200.f;
    c->spB_min_radius = 43.f * U_MM;
}

/* track_params_estimation_config, track_params_estimation_config.hpp:18-33. */
void or_tp_config_default(or_tp_config* c) {
    c->initial_sigma[0] = 1.f * U_MM;
    c->initial_sigma[1] = 1.f * U_MM;
    c->initial_sigma[2] = 1.f * U_DEGREE;
    c->initial_sigma[3] = 1.f * U_DEGREE;
    c->initial_sigma[4] = 0.f * U_E / U_GEV;
    c->initial_sigma[5] = 1.f * U_NS;
    c->initial_sigma_qopt = 0.1f * U_E / U_GEV;
    c->initial_sigma_pt_rel = 0.1f;
    for (int i = 0; i < 6; ++i) c->initial_inflation[i] = 1.f;
    c->initial_inflation[5] = 100.f;
}

/* get_axes, spacepoint_binning_helper.hpp:22-110. */
int or_get_axes(const or_grid_config* g, or_axes* out) {
    uint32_t phiBins;
    if (g->bFieldInZ == 0) {
        phiBins = 100;
    } else {
        float minHelixRadius = g->minPt / g->bFieldInZ;
        if (minHelixRadius < g->rMax / 2) return 1;
        float maxR2 = g->rMax * g->rMax;
        float xOuter = maxR2 / (2 * minHelixRadius);
        float yOuter = sqrtf(maxR2 - xOuter * xOuter);
        float outerAngle = atanf(xOuter / yOuter);
        float innerAngle = 0;
        float rMin = g->rMax;
        if (g->rMax > g->deltaRMax) {
            rMin = g->rMax - g->deltaRMax;
            float innerCircleR2 =
                (g->rMax - g->deltaRMax) * (g->rMax - g->deltaRMax);
            float xInner = innerCircleR2 / (2 * minHelixRadius);
            float yInner = sqrtf(innerCircleR2 - xInner * xInner);
            innerAngle = atanf(xInner / yInner);
        }
        float deltaAngleWithMaxD0 =
            fabsf(asinf(g->impactMax / (rMin)) - asinf(g->impactMax / g->rMax));
        float deltaPhi = (outerAngle - innerAngle + deltaAngleWithMaxD0) /
                         (float)(g->phiBinDeflectionCoverage);
        if (deltaPhi <= 0.) return 2;
        phiBins = (uint32_t)llround(2 * M_PI / deltaPhi + 0.5);
    }
    float zBinSize = g->cotThetaMax * g->deltaRMax;
    uint32_t zb = (uint32_t)floorf((g->zMax - g->zMin) / zBinSize);
    out->phi_bins = phiBins;
    out->phi_min = g->phiMin;
    out->phi_max = g->phiMax;
    out->z_bins = zb > 1u ? zb : 1u;
    out->z_min = g->zMin;
    out->z_max = g->zMax;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Axes (core/include/traccc/seeding/grids/axis.hpp)                         */
/* ------------------------------------------------------------------------ */

/* regular::bin, axis.hpp:87-100 */
uint32_t or_regular_bin(uint32_t n, float mn, float mx, float v) {
    int ibin = (int)((v - mn) / (mx - mn) * (float)n);
    if (ibin >= 0 && ibin < (int)n) return (uint32_t)ibin;
    return ibin < 0 ? 0u : n - 1u;
}

/* regular::range (binned neighbourhood), axis.hpp:110-123 */
void or_regular_range(uint32_t n, float mn, float mx, float v,
                      const uint32_t nh[2], uint32_t out[2]) {
    int ibin = (int)((v - mn) / (mx - mn) * (float)n);
    int ibinmin = ibin - (int)nh[0];
    int ibinmax = ibin + (int)nh[1];
    out[0] = (ibinmin >= 0) ? (uint32_t)ibinmin : 0u;
    out[1] = (ibinmax < (int)n) ? (uint32_t)ibinmax : n - 1u;
}

/* regular::zone_t, axis.hpp:155-166 */
uint32_t or_regular_zone(uint32_t n, float mn, float mx, float v,
                         const uint32_t nh[2], uint32_t* out, uint32_t cap) {
    uint32_t r[2];
    or_regular_range(n, mn, mx, v, nh, r);
    uint32_t len = r[1] - r[0] + 1u;
    for (uint32_t i = 0; i < len && i < cap; ++i) out[i] = r[0] + i;
    return len;
}

/* circular::bin, axis.hpp:277-289 */
uint32_t or_circular_bin(uint32_t n, float mn, float mx, float v) {
    int ibin = (int)((v - mn) / (mx - mn) * (float)n);
    if (ibin >= 0 && ibin < (int)n) return (uint32_t)ibin;
    if (ibin < 0) return n + (uint32_t)ibin;
    return (uint32_t)ibin - n;
}

/* circular::remap, axis.hpp:394-404 */
uint32_t or_circular_remap(uint32_t n, uint32_t ibin, int32_t shood) {
    int opt_bin = (int)ibin + shood;
    if (opt_bin >= 0 && opt_bin < (int)n) return (uint32_t)opt_bin;
    if (opt_bin < 0) return (uint32_t)((int)n + opt_bin);
    return (uint32_t)opt_bin - n;
}

/* circular::range (binned neighbourhood), axis.hpp:299-306 */
void or_circular_range(uint32_t n, float mn, float mx, float v,
                       const uint32_t nh[2], uint32_t out[2]) {
    uint32_t gbin = or_circular_bin(n, mn, mx, v);
    out[0] = or_circular_remap(n, gbin, -(int32_t)nh[0]);
    out[1] = or_circular_remap(n, gbin, (int32_t)nh[1]);
}

/* circular::zone_t, axis.hpp:333-358 (including its wrap-around order) */
uint32_t or_circular_zone(uint32_t n, float mn, float mx, float v,
                          const uint32_t nh[2], uint32_t* out, uint32_t cap) {
    uint32_t r[2];
    or_circular_range(n, mn, mx, v, nh, r);
    if (r[0] < r[1]) {
        uint32_t len = r[1] - r[0] + 1u;
        for (uint32_t i = 0; i < len && i < cap; ++i) out[i] = r[0] + i;
        return len;
    }
    uint32_t vl = n - r[0] + r[1] + 1u;
    uint32_t mi = 0, mo = 0;
    for (uint32_t i = 0; i < vl; ++i) {
        uint32_t b = r[0] + mi++;
        if (b > n - 1u) b = mo++;
        if (i < cap) out[i] = b;
    }
    return vl;
}

/* ------------------------------------------------------------------------ */
/* Spacepoint helpers                                                        */
/* ------------------------------------------------------------------------ */

static inline float sp_radius(float x, float y) {
    /* spacepoint::radius, spacepoint_collection.ipp:52-57 */
    return sqrtf(x * x + y * y);
}

/* spacepoint::phi (spacepoint_collection.ipp:59-63) = atan2(y, x).
 * OR_PHI_CR rounds the double-precision atan2 to float and reports inputs
 * whose double result lies too close to a float rounding midpoint to decide
 * the correctly rounded value from it. */
float or_sp_phi(float x, float y, int phi_mode, int* undecided) {
    if (phi_mode == OR_PHI_LIBM) return atan2f(y, x);
    double r = atan2((double)y, (double)x);
    float f = (float)r;
    if (undecided && isfinite(r) && r != 0.0) {
        double lo = (double)nextafterf(f, -INFINITY);
        double hi = (double)nextafterf(f, INFINITY);
        double m1 = 0.5 * ((double)f + lo), m2 = 0.5 * ((double)f + hi);
        double tol = fabs(r) * 0x1p-44;
        if (fabs(r - m1) <= tol || fabs(r - m2) <= tol) *undecided = 1;
    }
    return f;
}

/* is_valid_sp, spacepoint_binning_helper.hpp:112-127.  The reference casts
 * perp() to size_t; a non-finite or out-of-range perp is undefined behaviour
 * there and is treated as invalid here (what x86-64 produces). */
int or_is_valid_sp(const or_finder_config* c, float x, float y, float z,
                   int phi_mode) {
    if (z > c->zMax || z < c->zMin) return 0;
    float spPhi = or_sp_phi(x, y, phi_mode, NULL);
    if (spPhi > c->phiMax || spPhi < c->phiMin) return 0;
    float bx = x - c->beamPos[0], by = y - c->beamPos[1];
    float perp = sqrtf(bx * bx + by * by);
    float nb = c->rMax + sqrtf(c->beamPos[0] * c->beamPos[0] +
                               c->beamPos[1] * c->beamPos[1]);
    if (!(perp >= 0.f) || !(perp < 1.8e19f)) return 0;
    if (!(nb >= 0.f) || !(nb < 1.8e19f)) return 0;
    return (uint64_t)perp < (uint64_t)nb;
}

static inline int near_rel(float q, float t) {
    float d = fabsf(q - t);
    float s = fabsf(t) > fabsf(q) ? fabsf(t) : fabsf(q);
    return s > 0.f && d <= 1e-6f * s;
}

/* Distance of the scaled phi value to the nearest bin edge (for the report of
 * spacepoints whose bin a one-ulp change of phi would move). */
static int near_phi_edge(uint32_t n, float mn, float mx, float phi) {
    float v = (phi - mn) / (mx - mn) * (float)n;
    float k = floorf(v + 0.5f);
    return fabsf(v - k) <= 1e-6f * (float)n;
}

/* spacepoint_binning::operator(), core/src/seeding/spacepoint_binning.cpp:
 * 27-53: loop in spacepoint order, push valid ones to their (phi, z) bin. */
int or_binning(const or_finder_config* c, const or_axes* a,
               const or_spacepoints* sps, int phi_mode, uint32_t* bin_offsets,
               uint32_t* bin_sps, uint32_t* n_valid, or_stats* st) {
    uint32_t nbins = a->phi_bins * a->z_bins;
    uint32_t* bin_of = (uint32_t*)malloc(sizeof(uint32_t) * (sps->size + 1));
    if (!bin_of) return -2;
    memset(bin_offsets, 0, sizeof(uint32_t) * (nbins + 1));
    for (uint32_t i = 0; i < sps->size; ++i) {
        float x = sps->global[3 * i], y = sps->global[3 * i + 1],
              z = sps->global[3 * i + 2];
        bin_of[i] = UINT32_MAX;
        if (!or_is_valid_sp(c, x, y, z, phi_mode)) continue;
        int und = 0;
        float phi = or_sp_phi(x, y, phi_mode, &und);
        if (st) {
            st->phi_cr_undecided += (uint64_t)und;
            st->near_bin_edges +=
                (uint64_t)near_phi_edge(a->phi_bins, a->phi_min, a->phi_max, phi);
        }
        uint32_t b = or_circular_bin(a->phi_bins, a->phi_min, a->phi_max, phi) +
                     a->phi_bins * or_regular_bin(a->z_bins, a->z_min, a->z_max, z);
        bin_of[i] = b;
        bin_offsets[b + 1]++;
    }
    for (uint32_t b = 0; b < nbins; ++b) bin_offsets[b + 1] += bin_offsets[b];
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * (nbins + 1));
    if (!fill) { free(bin_of); return -2; }
    memcpy(fill, bin_offsets, sizeof(uint32_t) * (nbins + 1));
    for (uint32_t i = 0; i < sps->size; ++i)
        if (bin_of[i] != UINT32_MAX) bin_sps[fill[bin_of[i]]++] = i;
    *n_valid = bin_offsets[nbins];
    if (st) {
        st->n_sp += sps->size;
        st->n_valid += *n_valid;
        for (uint32_t b = 0; b < nbins; ++b) {
            uint64_t s = bin_offsets[b + 1] - bin_offsets[b];
            if (s > st->max_bin_size) st->max_bin_size = s;
        }
    }
    free(fill);
    free(bin_of);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Doublet / triplet helpers                                                 */
/* ------------------------------------------------------------------------ */

/* per-call scratch counters (per host thread) */
static _Thread_local uint64_t g_near_doublet, g_near_triplet;
/* FP32 operations (+ - * / sqrt, one each) of the doublet and triplet tests
 * as written, every operation of a stage counted once the stage is reached
 * (short-circuited comparisons included), and the pairs that pass the
 * doublet window (first stage) */
static _Thread_local uint64_t g_ops_doublet, g_ops_triplet, g_window_pass;

/* doublet_finding_helper::isCompatible, core/include/traccc/seeding/
 * doublet_finding_helper.hpp:51-216.  m = middle, o = bottom or top.
 * std::min keeps its (b < a) ? b : a semantics, so NaN radii do not reject. */
int or_doublet_compatible(int top, const float m[6], const float o[6],
                          const or_finder_config* c) {
    float deltaR, cotTheta, zOrigin;
    if (!top) {
        deltaR = m[3] - o[3];
        cotTheta = m[2] - o[2];
        zOrigin = m[2] * deltaR - m[3] * cotTheta;
    } else {
        deltaR = o[3] - m[3];
        cotTheta = (o[2] - m[2]);
        zOrigin = m[2] * deltaR - m[3] * cotTheta;
    }
    if ((deltaR >= c->deltaRMax) || (deltaR <= c->deltaRMin) ||
        (fabsf(cotTheta) >= c->cotThetaMax * deltaR) ||
        (zOrigin <= c->collisionRegionMin * deltaR) ||
        (zOrigin >= c->collisionRegionMax * deltaR) ||
        fabsf(cotTheta) >= c->deltaZMax) {
        g_ops_doublet += 8;
        if (near_rel(deltaR, c->deltaRMax) || near_rel(deltaR, c->deltaRMin) ||
            near_rel(fabsf(cotTheta), c->cotThetaMax * deltaR) ||
            near_rel(zOrigin, c->collisionRegionMin * deltaR) ||
            near_rel(zOrigin, c->collisionRegionMax * deltaR) ||
            near_rel(fabsf(cotTheta), c->deltaZMax))
            g_near_doublet++;
        return 0;
    }
    /* window: 5 for deltaR, cotTheta, zOrigin + 3 products in the cuts;
     * helix stage: 39 */
    g_ops_doublet += 8 + 39;
    g_window_pass++;
    float midX = 0.5f * (m[0] + o[0]);
    float midY = 0.5f * (m[1] + o[1]);
    float slope = (o[1] - m[1]) / (o[0] - m[0]);
    float deltaX = o[0] - m[0];
    float deltaY = o[1] - m[1];
    float deltaXY2 = deltaX * deltaX + deltaY * deltaY;
    float sagittaLength =
        sqrtf(c->minHelixRadius * c->minHelixRadius - deltaXY2 / 4.f);
    float denom = sqrtf((slope * slope + 1) / (slope * slope));
    float cosCentralAngle = 1.f / denom;
    float sinCentralAngle = -1.f / (slope * denom);
    float mpDeltaX = sagittaLength * cosCentralAngle;
    float mpDeltaY = sagittaLength * sinCentralAngle;
    float mp1X = midX + mpDeltaX;
    float mp2X = midX - mpDeltaX;
    float mp1Y = midY + mpDeltaY;
    float mp2Y = midY - mpDeltaY;
    float mp1R2 = mp1X * mp1X + mp1Y * mp1Y;
    float mp2R2 = mp2X * mp2X + mp2Y * mp2Y;
    float mn = (mp2R2 < mp1R2) ? mp2R2 : mp1R2;
    float lim = ((c->minHelixRadius - c->impactMax) *
                 (c->minHelixRadius - c->impactMax));
    if (near_rel(mn, lim)) g_near_doublet++;
    if (mn <= lim) return 0;
    return 1;
}

/* doublet_finding_helper::transform_coordinates, doublet_finding_helper.hpp:
 * 218-272.  lc = {Zo, cotTheta, iDeltaR, Er, U, V} (lin_circle.hpp:18-49). */
void or_transform_coordinates(int top, const float m[6], const float o[6],
                              float lc[6]) {
    const float xM = m[0], yM = m[1], zM = m[2], rM = m[3];
    const float varianceZM = m[4], varianceRM = m[5];
    float cosPhiM = xM / rM;
    float sinPhiM = yM / rM;
    float deltaX = o[0] - xM;
    float deltaY = o[1] - yM;
    float deltaZ = o[2] - zM;
    float x = deltaX * cosPhiM + deltaY * sinPhiM;
    float y = deltaY * cosPhiM - deltaX * sinPhiM;
    float iDeltaR2 = 1.f / (deltaX * deltaX + deltaY * deltaY);
    float iDeltaR = sqrtf(iDeltaR2);
    float cot_theta = deltaZ * iDeltaR;
    if (!top) cot_theta = -cot_theta;
    lc[1] = cot_theta;
    lc[0] = zM - rM * cot_theta;
    lc[2] = iDeltaR;
    lc[4] = x * iDeltaR2;
    lc[5] = y * iDeltaR2;
    lc[3] = ((varianceZM + o[4]) +
             (cot_theta * cot_theta) * (varianceRM + o[5])) *
            iDeltaR2;
}

/* triplet_finding_helper::isCompatible, core/include/traccc/seeding/
 * triplet_finding_helper.hpp:42-133. */
int or_triplet_compatible(const float m[6], const float lb[6],
                          const float lt[6], const or_finder_config* c,
                          float iSinTheta2, float scatteringInRegion2,
                          float* curvature, float* impact_parameter) {
    const float lbZo = lb[0], lbCot = lb[1], lbIDR = lb[2], lbEr = lb[3],
                lbU = lb[4], lbV = lb[5];
    const float ltCot = lt[1], ltIDR = lt[2], ltEr = lt[3], ltU = lt[4],
                ltV = lt[5];
    (void)lbZo;
    float error2 = ltEr + lbEr +
                   2.f * (lbCot * ltCot * m[5] + m[4]) * lbIDR * ltIDR;
    float deltaCotTheta = lbCot - ltCot;
    float deltaCotTheta2 = deltaCotTheta * deltaCotTheta;
    float error = 0.f;
    float dCotThetaMinusError2 = 0.f;
    g_ops_triplet += 11; /* error2 8, deltaCotTheta 1, its square 1, the gate 1 */
    if (deltaCotTheta2 - error2 > 0) {
        g_ops_triplet += 5; /* sqrt, 2 products, 2 sums */
        deltaCotTheta = fabsf(deltaCotTheta);
        error = sqrtf(error2);
        dCotThetaMinusError2 =
            deltaCotTheta2 + error2 - 2.f * deltaCotTheta * error;
        if (near_rel(dCotThetaMinusError2, scatteringInRegion2))
            g_near_triplet++;
        if (dCotThetaMinusError2 > scatteringInRegion2) return 0;
    }
    float dU = ltU - lbU;
    g_ops_triplet += 1;
    if (dU == 0.f) return 0;
    g_ops_triplet += 8; /* A 2, S2 2, B 2, B2 1, the cut's product 1 */
    float A = (ltV - lbV) / dU;
    float S2 = 1.f + A * A;
    float B = lbV - A * lbU;
    float B2 = B * B;
    if (near_rel(S2, B2 * c->minHelixDiameter2)) g_near_triplet++;
    if (S2 < B2 * c->minHelixDiameter2) return 0;
    g_ops_triplet += 15; /* pT-dependent scattering 10, curvature 2, impact 3 */
    float iHelixDiameter2 = B2 / S2;
    float pT2scatter = 4.f * iHelixDiameter2 * c->pT2perRadius;
    float pT = c->pTPerHelixRadius * sqrtf(S2 / B2) / 2.f;
    if (pT > c->maxPtScattering) {
        float pTscatter = c->highland / c->maxPtScattering;
        pT2scatter = pTscatter * pTscatter;
    }
    float p2scatter = pT2scatter * iSinTheta2;
    float lim2 = p2scatter * c->sigmaScattering * c->sigmaScattering;
    if ((deltaCotTheta2 - error2 > 0.f) && near_rel(dCotThetaMinusError2, lim2))
        g_near_triplet++;
    if ((deltaCotTheta2 - error2 > 0.f) && (dCotThetaMinusError2 > lim2))
        return 0;
    *curvature = B / sqrtf(S2);
    *impact_parameter = fabsf((A - B * m[3]) * m[3]);
    if (near_rel(*impact_parameter, c->impactMax)) g_near_triplet++;
    if (*impact_parameter > c->impactMax) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Seed finding                                                              */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint32_t sp;   /* spacepoint index of the bottom / top */
    float lc[6];
} dbl_t;

typedef struct {
    uint32_t spB, spT;
    uint32_t order; /* position in the middle's triplet list (host order) */
    float curvature, weight, z_vertex;
} trip_t;

typedef struct {
    void* p;
    size_t n, cap, esz;
} vec_t;

static int vec_push(vec_t* v, const void* e) {
    if (v->n == v->cap) {
        size_t nc = v->cap ? 2 * v->cap : 64;
        void* np = realloc(v->p, nc * v->esz);
        if (!np) return -1;
        v->p = np;
        v->cap = nc;
    }
    memcpy((char*)v->p + v->n * v->esz, e, v->esz);
    v->n++;
    return 0;
}

static void load_sp(const or_spacepoints* s, uint32_t i, float o[6]) {
    o[0] = s->global[3 * i];
    o[1] = s->global[3 * i + 1];
    o[2] = s->global[3 * i + 2];
    o[3] = sp_radius(o[0], o[1]);
    o[4] = s->z_variance ? s->z_variance[i] : 0.f;
    o[5] = s->radius_variance ? s->radius_variance[i] : 0.f;
}

/* triplet_sorter, core/include/traccc/seeding/detail/triplet_sorter.hpp:39-71:
 * weight descending, then the sum y^2+z^2 of bottom and top descending.  The
 * reference leaves the order of exact ties to std::sort; here they keep their
 * host list order, which makes the order total. */
typedef struct {
    const or_spacepoints* s;
} sort_ctx_t;

static float tie_sum(const or_spacepoints* s, uint32_t b, uint32_t t) {
    float yb = s->global[3 * b + 1], zb = s->global[3 * b + 2];
    float yt = s->global[3 * t + 1], zt = s->global[3 * t + 2];
    return yb * yb + zb * zb + yt * yt + zt * zt;
}

/* returns 1 if a sorts before b */
static int trip_before(const trip_t* a, const trip_t* b, const or_spacepoints* s) {
    if (a->weight != b->weight) return a->weight > b->weight;
    float sa = tie_sum(s, a->spB, a->spT), sb = tie_sum(s, b->spB, b->spT);
    if (sa != sb) return sa > sb;
    return a->order < b->order;
}

static void merge_sort(uint32_t* idx, uint32_t* tmp, size_t n, const trip_t* t,
                       const or_spacepoints* s) {
    if (n < 2) return;
    size_t h = n / 2;
    merge_sort(idx, tmp, h, t, s);
    merge_sort(idx + h, tmp, n - h, t, s);
    size_t i = 0, j = h, k = 0;
    while (i < h && j < n) {
        if (trip_before(&t[idx[j]], &t[idx[i]], s)) tmp[k++] = idx[j++];
        else tmp[k++] = idx[i++];
    }
    while (i < h) tmp[k++] = idx[i++];
    while (j < n) tmp[k++] = idx[j++];
    memcpy(idx, tmp, n * sizeof(uint32_t));
}

typedef struct {
    const or_finder_config* fc;
    const or_filter_config* flt;
    const or_spacepoints* sps;
    const or_axes* ax;
    const uint32_t* bin_off;
    const uint32_t* bin_sps;
    int phi_mode;
} seed_ctx_t;

/* doublet_finding<T>::operator(), core/src/seeding/doublet_finding.hpp:51-110:
 * phi zone (outer) x z zone (inner), in-bin order. */
static int find_doublets(const seed_ctx_t* x, uint32_t spM, const float m[6],
                         int top, vec_t* out, or_stats* st) {
    uint32_t phis[64], zs[64];
    float phi = or_sp_phi(m[0], m[1], x->phi_mode, NULL);
    uint32_t np = or_circular_zone(x->ax->phi_bins, x->ax->phi_min,
                                   x->ax->phi_max, phi, x->fc->neighbor_scope,
                                   phis, 64);
    uint32_t nz = or_regular_zone(x->ax->z_bins, x->ax->z_min, x->ax->z_max,
                                  m[2], x->fc->neighbor_scope, zs, 64);
    if (np > 64 || nz > 64) return -3;
    (void)spM;
    uint64_t nb = 0;
    for (uint32_t ip = 0; ip < np; ++ip) {
        for (uint32_t iz = 0; iz < nz; ++iz) {
            uint32_t b = phis[ip] + zs[iz] * x->ax->phi_bins;
            for (uint32_t k = x->bin_off[b]; k < x->bin_off[b + 1]; ++k) {
                uint32_t o = x->bin_sps[k];
                float ov[6];
                load_sp(x->sps, o, ov);
                nb++;
                if (or_doublet_compatible(top, m, ov, x->fc)) {
                    dbl_t d;
                    d.sp = o;
                    or_transform_coordinates(top, m, ov, d.lc);
                    if (vec_push(out, &d)) return -2;
                }
            }
        }
    }
    if (st) {
        st->n_pair_tests += nb;
        if (nb > st->max_neighbourhood) st->max_neighbourhood = nb;
    }
    return 0;
}

/* seed_finding::operator() with triplet_finding, seed_filtering:
 * core/src/seeding/seed_finding.cpp:58-121,
 * core/src/seeding/triplet_finding.hpp:60-183,
 * core/src/seeding/seed_filtering.cpp:28-123,
 * core/include/traccc/seeding/seed_selecting_helper.hpp:27-80. */
/* ------------------------------------------------------------------------ */
/* Learned doublet filter                                                    */
/* ------------------------------------------------------------------------ */

/* float -> bf16 -> float, round to nearest even (NaN stays NaN). */
float or_bf16_round(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x007fffffu)) {
        u |= 0x00400000u;
        u &= 0xffff0000u;
    } else {
        u += 0x7fffu + ((u >> 16) & 1u);
        u &= 0xffff0000u;
    }
    memcpy(&x, &u, 4);
    return x;
}

static uint32_t band_of(const or_doublet_filter* f, float r) {
    uint32_t b = 0;
    for (uint32_t i = 0; i < f->n_edges; ++i)
        if (f->edges[i] <= r) ++b;
    return b;
}

void or_doublet_features(int top, const float m[6], const float o[6],
                         const float lc[6], const or_doublet_filter* f,
                         float feat[OR_MLP_IN]) {
    (void)top;
    feat[0] = m[3];
    feat[1] = m[2];
    feat[2] = o[3] - m[3];
    feat[3] = o[2] - m[2];
    feat[4] = lc[1];
    /* y * iDeltaR with the operations of or_transform_coordinates */
    const float cosPhiM = m[0] / m[3], sinPhiM = m[1] / m[3];
    const float deltaX = o[0] - m[0], deltaY = o[1] - m[1];
    const float y = deltaY * cosPhiM - deltaX * sinPhiM;
    const float iDeltaR2 = 1.f / (deltaX * deltaX + deltaY * deltaY);
    feat[5] = y * sqrtf(iDeltaR2);
    feat[6] = lc[0];
    const uint32_t nb = f ? f->n_edges + 1 : 1;
    feat[7] = f ? (float)(band_of(f, m[3]) * nb + band_of(f, o[3])) : 0.f;
}

float or_mlp_logit(const or_doublet_filter* f, const float feat[OR_MLP_IN]) {
    float x[OR_MLP_IN], h1[OR_MLP_H], h2[OR_MLP_H];
    for (int i = 0; i < OR_MLP_IN; ++i) x[i] = or_bf16_round((feat[i] - f->mu[i]) * f->isd[i]);
    for (int j = 0; j < OR_MLP_H; ++j) {
        float a = f->b1[j];
        for (int i = 0; i < OR_MLP_IN; ++i) a += x[i] * or_bf16_round(f->w1[i * OR_MLP_H + j]);
        h1[j] = or_bf16_round(a > 0.f ? a : 0.f);
    }
    for (int j = 0; j < OR_MLP_H; ++j) {
        float a = f->b2[j];
        for (int i = 0; i < OR_MLP_H; ++i) a += h1[i] * or_bf16_round(f->w2[i * OR_MLP_H + j]);
        h2[j] = or_bf16_round(a > 0.f ? a : 0.f);
    }
    float a = f->b3;
    for (int i = 0; i < OR_MLP_H; ++i) a += h2[i] * or_bf16_round(f->w3[i]);
    return a;
}

/* Scores the doublets of one role, dumps them, and (if the filter may prune
 * this role) keeps those with logit >= threshold, in order. */
static int score_role(const or_doublet_filter* filt, int top, uint32_t spM,
                      const float m[6], const or_spacepoints* sps, vec_t* v,
                      or_doublet_rec* dump, uint64_t dump_cap, uint64_t* n_dump,
                      uint64_t* n_scored, uint64_t* n_pruned, int* reach) {
    dbl_t* D = (dbl_t*)v->p;
    size_t w = 0;
    const uint32_t mode = filt ? (top ? filt->prune_top : filt->prune_bottom) : 0u;
    const int may_prune = mode == 1u;
    *reach = 0;
    for (size_t k = 0; k < v->n; ++k) {
        float ov[6], feat[OR_MLP_IN];
        load_sp(sps, D[k].sp, ov);
        or_doublet_features(top, m, ov, D[k].lc, filt, feat);
        const float logit = filt ? or_mlp_logit(filt, feat) : 0.f;
        if (dump && n_dump) {
            if (*n_dump < dump_cap) {
                or_doublet_rec* r = &dump[*n_dump];
                r->middle = spM;
                r->other = D[k].sp;
                r->top = (uint32_t)top;
                memcpy(r->feat, feat, sizeof feat);
                r->logit = logit;
            }
            ++*n_dump;
        }
        (*n_scored)++;
        if (filt && logit >= filt->threshold[top ? 1 : 0]) *reach = 1;
        if (may_prune && !(logit >= filt->threshold[top ? 1 : 0])) {
            (*n_pruned)++;
            continue;
        }
        D[w++] = D[k];
    }
    v->n = w;
    return 0;
}

int or_seeding(const or_finder_config* fc, const or_grid_config* gc,
               const or_filter_config* flt, const or_spacepoints* sps,
               int phi_mode, or_seed* out, uint32_t cap, uint32_t* n_out,
               or_stats* st) {
    return or_seeding_ex(fc, gc, flt, sps, phi_mode, NULL, NULL, 0, NULL, NULL, 0, NULL,
                         out, cap, n_out, st);
}

int or_seeding_ex(const or_finder_config* fc, const or_grid_config* gc,
                  const or_filter_config* flt, const or_spacepoints* sps,
                  int phi_mode, const or_doublet_filter* filt,
                  or_doublet_rec* dump, uint64_t dump_cap, uint64_t* n_dump,
                  or_triplet_rec* tdump, uint64_t tdump_cap, uint64_t* n_tdump,
                  or_seed* out, uint32_t cap, uint32_t* n_out, or_stats* st) {
    or_stats st_local;
    if (!st && (filt || dump)) {
        memset(&st_local, 0, sizeof st_local);
        st = &st_local;
    }
    if (n_dump) *n_dump = 0;
    if (n_tdump) *n_tdump = 0;
    or_axes ax;
    int rc = or_get_axes(gc, &ax);
    if (rc) return rc;
    uint32_t nbins = ax.phi_bins * ax.z_bins;
    uint32_t* bin_off = (uint32_t*)malloc(sizeof(uint32_t) * (nbins + 1));
    uint32_t* bin_sps = (uint32_t*)malloc(sizeof(uint32_t) * (sps->size + 1));
    if (!bin_off || !bin_sps) { free(bin_off); free(bin_sps); return -2; }
    uint32_t n_valid = 0;
    g_near_doublet = g_near_triplet = 0;
    g_ops_doublet = g_ops_triplet = g_window_pass = 0;
    rc = or_binning(fc, &ax, sps, phi_mode, bin_off, bin_sps, &n_valid, st);
    if (rc) { free(bin_off); free(bin_sps); return rc; }

    seed_ctx_t x = {fc, flt, sps, &ax, bin_off, bin_sps, phi_mode};
    vec_t mb = {0, 0, 0, sizeof(dbl_t)}, mt = {0, 0, 0, sizeof(dbl_t)};
    vec_t tr = {0, 0, 0, sizeof(trip_t)};
    vec_t sel = {0, 0, 0, sizeof(uint32_t)}, tmp = {0, 0, 0, sizeof(uint32_t)};
    vec_t cr = {0, 0, 0, sizeof(float)};
    uint32_t n_seeds = 0;
    rc = 0;

    for (uint32_t b = 0; b < nbins && rc == 0; ++b) {
        for (uint32_t j = bin_off[b]; j < bin_off[b + 1] && rc == 0; ++j) {
            uint32_t spM = bin_sps[j];
            float m[6];
            load_sp(sps, spM, m);
            mb.n = 0;
            if ((rc = find_doublets(&x, spM, m, 0, &mb, st))) break;
            if (mb.n == 0) continue;
            if (st) st->n_middles_with_mb++;
            mt.n = 0;
            if ((rc = find_doublets(&x, spM, m, 1, &mt, st))) break;
            if (st) {
                st->n_mb += mb.n;
                st->n_mt += mt.n;
                if (mb.n > st->max_mb_per_middle) st->max_mb_per_middle = mb.n;
                if (mt.n > st->max_mt_per_middle) st->max_mt_per_middle = mt.n;
            }
            if (mt.n == 0) continue;
            if (filt || dump) {
                /* bottoms first; a middle left without bottoms has no seeds
                 * and its tops are not scored */
                int reach = 0;
                score_role(filt, 0, spM, m, sps, &mb, dump, dump_cap, n_dump,
                           &st->n_scored_mb, &st->n_pruned_mb, &reach);
                if (mb.n == 0) continue;
                score_role(filt, 1, spM, m, sps, &mt, dump, dump_cap, n_dump,
                           &st->n_scored_mt, &st->n_pruned_mt, &reach);
                if (filt && filt->prune_top == 2u && !reach &&
                    (filt->gate_max_tops == 0u || mt.n <= filt->gate_max_tops)) {
                    /* gated middle: no seed, its middle-top doublets pruned */
                    st->n_pruned_mt += mt.n;
                    continue;
                }
                if (mt.n == 0) continue;
            }
            if (st) {
                st->n_middles_both++;
                st->n_triplet_tests += (uint64_t)mb.n * mt.n;
            }
            tr.n = 0;
            const dbl_t* MB = (const dbl_t*)mb.p;
            const dbl_t* MT = (const dbl_t*)mt.p;
            for (size_t k = 0; k < mb.n && rc == 0; ++k) {
                const float* lb = MB[k].lc;
                /* triplet_finding.hpp:82-88 */
                const float iSinTheta2 = 1.f + lb[1] * lb[1];
                float scatteringInRegion2 = fc->maxScatteringAngle2 * iSinTheta2;
                scatteringInRegion2 *= fc->sigmaScattering * fc->sigmaScattering;
                size_t first = tr.n;
                for (size_t t = 0; t < mt.n; ++t) {
                    float curvature, impact;
                    if (!or_triplet_compatible(m, lb, MT[t].lc, fc, iSinTheta2,
                                               scatteringInRegion2, &curvature,
                                               &impact))
                        continue;
                    trip_t tp;
                    tp.spB = MB[k].sp;
                    tp.spT = MT[t].sp;
                    tp.order = (uint32_t)tr.n;
                    tp.curvature = curvature;
                    tp.weight = -impact * flt->impactWeightFactor;
                    tp.z_vertex = lb[0];
                    if (vec_push(&tr, &tp)) { rc = -2; break; }
                    if (tdump && n_tdump) {
                        if (*n_tdump < tdump_cap) {
                            or_triplet_rec* r = &tdump[*n_tdump];
                            r->middle = spM;
                            r->bottom = MB[k].sp;
                            r->top = MT[t].sp;
                            r->event = 0;
                        }
                        ++*n_tdump;
                    }
                }
                /* compatible-seed weights, triplet_finding.hpp:107-179 */
                trip_t* T = (trip_t*)tr.p;
                size_t nk = tr.n - first;
                if (st && nk > st->max_triplets_per_mb) st->max_triplets_per_mb = nk;
                for (size_t i = first; i < tr.n; ++i) {
                    float tv[6];
                    load_sp(sps, T[i].spT, tv);
                    const float currentTop_r = tv[3];
                    cr.n = 0;
                    float lowerLimitCurv = T[i].curvature - flt->deltaInvHelixDiameter;
                    float upperLimitCurv = T[i].curvature + flt->deltaInvHelixDiameter;
                    for (size_t j2 = first; j2 < tr.n; ++j2) {
                        if (i == j2) continue;
                        float ov[6];
                        load_sp(sps, T[j2].spT, ov);
                        const float otherTop_r = ov[3];
                        const float deltaR = currentTop_r - otherTop_r;
                        if (fabsf(deltaR) < flt->deltaRMin) continue;
                        if (T[j2].curvature < lowerLimitCurv) continue;
                        if (T[j2].curvature > upperLimitCurv) continue;
                        int newCompSeed = 1;
                        const float* prev = (const float*)cr.p;
                        for (size_t q = 0; q < cr.n; ++q) {
                            if (fabsf(prev[q] - otherTop_r) < flt->deltaRMin) {
                                newCompSeed = 0;
                                break;
                            }
                        }
                        if (newCompSeed) {
                            if (vec_push(&cr, &otherTop_r)) { rc = -2; break; }
                            T[i].weight += flt->compatSeedWeight;
                        }
                        if (cr.n >= flt->compatSeedLimit) break;
                    }
                }
            }
            if (rc) break;
            if (st) {
                st->n_triplets += tr.n;
                if (tr.n > st->max_triplets_per_middle)
                    st->max_triplets_per_middle = tr.n;
            }
            /* seed_filtering::operator(), seed_filtering.cpp:34-122 */
            trip_t* T = (trip_t*)tr.p;
            sel.n = 0;
            for (size_t i = 0; i < tr.n; ++i) {
                float bv[6], tv[6];
                load_sp(sps, T[i].spB, bv);
                load_sp(sps, T[i].spT, tv);
                /* seed_selecting_helper::seed_weight, :27-43 */
                float weight = 0;
                if (bv[3] > flt->good_spB_min_radius)
                    weight = flt->good_spB_weight_increase;
                if (tv[3] < flt->good_spT_max_radius)
                    weight = flt->good_spT_weight_increase;
                T[i].weight += weight;
                /* single_seed_cut, :54-62 */
                if (bv[3] > flt->good_spB_min_radius &&
                    T[i].weight < flt->good_spB_min_weight)
                    continue;
                uint32_t ii = (uint32_t)i;
                if (vec_push(&sel, &ii)) { rc = -2; break; }
            }
            if (rc) break;
            if (st) st->n_triplets_after_cut += sel.n;
            if (sel.n == 0) continue;
            while (tmp.cap < sel.n) {
                uint32_t z = 0;
                if (vec_push(&tmp, &z)) { rc = -2; break; }
            }
            if (rc) break;
            merge_sort((uint32_t*)sel.p, (uint32_t*)tmp.p, sel.n, T, sps);
            const uint32_t* S = (const uint32_t*)sel.p;
            uint32_t acc[64];
            uint32_t nacc = 0;
            acc[nacc++] = S[0];
            size_t itLength = sel.n < fc->maxSeedsPerSpM ? sel.n : fc->maxSeedsPerSpM;
            for (size_t i = 1; i < itLength; ++i) {
                float bv[6];
                load_sp(sps, T[S[i]].spB, bv);
                /* cut_per_middle_sp, seed_selecting_helper.hpp:73-79 */
                if (T[S[i]].weight > flt->seed_min_weight ||
                    bv[3] > flt->spB_min_radius) {
                    if (nacc < 64) acc[nacc++] = S[i];
                }
            }
            for (uint32_t i = 0; i < nacc && i < fc->maxSeedsPerSpM; ++i) {
                if (n_seeds < cap && out) {
                    out[n_seeds].bottom = T[acc[i]].spB;
                    out[n_seeds].middle = spM;
                    out[n_seeds].top = T[acc[i]].spT;
                    out[n_seeds].quality = (float)T[acc[i]].weight;
                }
                n_seeds++;
            }
        }
    }
    if (st) {
        st->n_seeds += n_seeds;
        st->near_doublet_cuts += g_near_doublet;
        st->near_triplet_cuts += g_near_triplet;
        st->n_window_pairs += g_window_pass;
        st->ops_doublet_tests += g_ops_doublet;
        st->ops_triplet_tests += g_ops_triplet;
    }
    free(mb.p); free(mt.p); free(tr.p); free(sel.p); free(tmp.p); free(cr.p);
    free(bin_off); free(bin_sps);
    *n_out = n_seeds;
    if (rc) return rc;
    return n_seeds > cap ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* Track parameter estimation                                                */
/* ------------------------------------------------------------------------ */

static void v3_cross(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}
static float v3_norm(const float a[3]) {
    return sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
}
static void v3_normalize(const float a[3], float o[3]) {
    float n = v3_norm(a);
    o[0] = a[0] / n;
    o[1] = a[1] / n;
    o[2] = a[2] / n;
}
static float perp2(float a, float b) { return sqrtf(a * a + b * b); }

/* seed_to_bound_param_vector, core/include/traccc/seeding/
 * track_params_estimation_helper.hpp:48-129, with the covariance of
 * core/src/seeding/track_params_estimation.cpp:59-86.  The frame algebra
 * (detray transform3) is restated with standard definitions:
 * point_to_local(p) = R^T (p - t), rotate(v) = R v, R = [x y z] columns. */
int or_track_params(const or_tp_config* c, const or_measurements* meas,
                    const or_spacepoints* sps, const or_seed* seeds,
                    uint32_t n_seeds, const float bfield[3],
                    or_bound_params* out) {
    for (uint32_t i = 0; i < n_seeds; ++i) {
        or_bound_params* p = &out[i];
        memset(p, 0, sizeof(*p));
        const uint32_t ib = seeds[i].bottom, im = seeds[i].middle,
                       it = seeds[i].top;
        const float* gB = &sps->global[3 * ib];
        const float* gM = &sps->global[3 * im];
        const float* gT = &sps->global[3 * it];
        float relVec[3] = {gM[0] - gB[0], gM[1] - gB[1], gM[2] - gB[2]};
        float newZ[3], tmp[3], newY[3], newX[3];
        v3_normalize(bfield, newZ);
        v3_cross(newZ, relVec, tmp);
        v3_normalize(tmp, newY);
        v3_cross(newY, newZ, newX);
        float d1[3] = {gM[0] - gB[0], gM[1] - gB[1], gM[2] - gB[2]};
        float d2[3] = {gT[0] - gB[0], gT[1] - gB[1], gT[2] - gB[2]};
        float l1[3] = {newX[0] * d1[0] + newX[1] * d1[1] + newX[2] * d1[2],
                       newY[0] * d1[0] + newY[1] * d1[1] + newY[2] * d1[2],
                       newZ[0] * d1[0] + newZ[1] * d1[1] + newZ[2] * d1[2]};
        float l2[3] = {newX[0] * d2[0] + newX[1] * d2[1] + newX[2] * d2[2],
                       newY[0] * d2[0] + newY[1] * d2[1] + newY[2] * d2[2],
                       newZ[0] * d2[0] + newZ[1] * d2[1] + newZ[2] * d2[2]};
        /* uv_transform, track_params_estimation_helper.hpp:29-36 */
        float den1 = l1[0] * l1[0] + l1[1] * l1[1];
        float u1 = l1[0] / den1, v1 = l1[1] / den1;
        float den2 = l2[0] * l2[0] + l2[1] * l2[1];
        float u2 = l2[0] / den2, v2 = l2[1] / den2;
        float A = (v2 - v1) / (u2 - u1);
        float B = v2 - A * u2;
        float R = -perp2(1.f, A) / (2.f * B);
        float invTanTheta =
            l2[2] / (2.f * R * asinf(perp2(l2[0], l2[1]) / (2.f * R)));
        float td[3] = {1.f, A, perp2(1.f, A) * invTanTheta};
        float tdn[3];
        v3_normalize(td, tdn);
        float dir[3] = {newX[0] * tdn[0] + newY[0] * tdn[1] + newZ[0] * tdn[2],
                        newX[1] * tdn[0] + newY[1] * tdn[1] + newZ[1] * tdn[2],
                        newX[2] * tdn[0] + newY[2] * tdn[1] + newZ[2] * tdn[2]};
        float phi = atan2f(dir[1], dir[0]);
        float theta = atan2f(perp2(dir[0], dir[1]), dir[2]);
        uint32_t mi = sps->measurement_index_1[ib];
        if (mi >= meas->size) return -4;
        p->surface_link = meas->surface_link[mi];
        p->params[0] = meas->local_position[2 * mi];
        p->params[1] = meas->local_position[2 * mi + 1];
        p->params[2] = phi;
        p->params[3] = theta;
        float qOverPt = 1.f / (R * v3_norm(bfield));
        p->params[4] = qOverPt / perp2(1.f, invTanTheta);
        p->params[5] = 0.f;
        /* covariance, track_params_estimation.cpp:64-86 */
        for (int j = 0; j < 6; ++j) {
            float var = c->initial_sigma[j] * c->initial_sigma[j];
            if (j == 4) {
                float var_theta = p->cov[3 * 6 + 3];
                var += powf(c->initial_sigma_qopt * sinf(p->params[3]), 2.f);
                var += powf(c->initial_sigma_pt_rel * p->params[4], 2.f);
                var += var_theta *
                       powf(p->params[4] / tanf(p->params[3]), 2.f);
            }
            var *= c->initial_inflation[j];
            p->cov[j * 6 + j] = var;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Spacepoint formation                                                      */
/* ------------------------------------------------------------------------ */

/* silicon_pixel_spacepoint_formation.hpp:31-60 with fill_pixel_spacepoint
 * (spacepoint_formation.ipp:27-47): valid = 2-dimensional measurement. */
uint32_t or_form_spacepoints(const or_surface* surfaces, uint32_t n_surfaces,
                             const or_measurements* meas, const uint8_t* dims,
                             uint32_t* mi1, uint32_t* mi2, float* global,
                             float* zvar, float* rvar) {
    uint32_t k = 0;
    for (uint32_t i = 0; i < meas->size; ++i) {
        if (dims && dims[i] != 2u) continue;
        if (meas->surface_link[i] >= n_surfaces) continue;
        const or_surface* S = &surfaces[meas->surface_link[i]];
        const float l0 = meas->local_position[2 * i];
        const float l1 = meas->local_position[2 * i + 1];
        float a, b, c;
        if (S->type == 1u) {
            const double phi = (double)l0 / (double)S->radius;
            a = S->radius * (float)cos(phi);
            b = S->radius * (float)sin(phi);
            c = l1;
        } else {
            a = l0;
            b = l1;
            c = 0.f;
        }
        for (int r = 0; r < 3; ++r) {
            float v = S->rotation[3 * r] * a + S->rotation[3 * r + 1] * b;
            v = v + S->rotation[3 * r + 2] * c;
            global[3 * k + r] = v + S->translation[r];
        }
        mi1[k] = i;
        mi2[k] = 0xFFFFFFFFu;
        zvar[k] = 0.f;
        rvar[k] = 0.f;
        ++k;
    }
    return k;
}
