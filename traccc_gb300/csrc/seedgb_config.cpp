// Host-side configuration logic of the seeding library: the reference's config
// defaults, seedfinder_config::setup() and get_axes(), evaluated on the host
// in float exactly as the reference does (no FMA contraction: this file is
// built with -ffp-contract=off).  The derived values are passed to the kernels
// by value, so the device uses bit-identical constants.
#include <cmath>
#include <cstring>

#include "seedgb.h"

namespace {
// detray units used by traccc (core/include/traccc/definitions/common.hpp:
// 18-25): mm = 1, GeV = 1, MeV = 1e-3, T = 0.000299792458 GeV/(e mm),
// degree = pi/180, ns = 299.792458 mm (time in mm of light travel).
constexpr float kMM = 1.f;
constexpr float kMeV = 1e-3f;
constexpr float kGeV = 1.f;
constexpr float kT = 0.000299792458f;
constexpr float kDegree = 0.017453292519943295f;
constexpr float kNs = 299.792458f;
constexpr float kE = 1.f;
}  // namespace

extern "C" {

// seedfinder_config::setup(), core/include/traccc/seeding/detail/
// seeding_config.hpp:120-138 (the pT2perRadius unit slip is kept as written).
void seedgb_seedfinder_config_setup(seedgb_seedfinder_config* c) {
    c->highland = 13.6f * kMeV * std::sqrt(c->radLengthPerSeed) *
                  (1.f + 0.038f * std::log(c->radLengthPerSeed));
    const float maxScatteringAngle = c->highland / c->minPt;
    c->maxScatteringAngle2 = maxScatteringAngle * maxScatteringAngle;
    c->pTPerHelixRadius = c->bFieldInZ;
    c->minHelixDiameter2 = std::pow(c->minPt * 2.f / c->pTPerHelixRadius, 2.f);
    c->minHelixRadius = std::sqrt(c->minHelixDiameter2) / 2.f;
    c->pT2perRadius = std::pow(c->highland / c->pTPerHelixRadius, 2.f);
}

// seedfinder_config member initialisers, seeding_config.hpp:19-118.
void seedgb_seedfinder_config_default(seedgb_seedfinder_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->zMin = -2000.f * kMM;
    c->zMax = 2000.f * kMM;
    c->rMax = 200.f * kMM;
    c->rMin = 33.f * kMM;
    c->collisionRegionMin = -250 * kMM;
    c->collisionRegionMax = +250 * kMM;
    c->phiMin = static_cast<float>(-M_PI);
    c->phiMax = static_cast<float>(M_PI);
    c->minPt = 500.f * kMeV;
    c->cotThetaMax = 27.2845f;
    c->deltaRMin = 20 * kMM;
    c->deltaRMax = 80 * kMM;
    c->deltaZMax = 450 * kMM;
    c->impactMax = 10.f * kMM;
    c->sigmaScattering = 3.0f;
    c->maxPtScattering = 10.f * kGeV;
    c->maxSeedsPerSpM = 5;
    c->bFieldInZ = 1.99724f * kT;
    c->beamPos[0] = -.0f * kMM;
    c->beamPos[1] = -.0f * kMM;
    c->radLengthPerSeed = 0.05f;
    c->zAlign = 0 * kMM;
    c->rAlign = 0 * kMM;
    c->sigmaError = 5;
    c->phiBinDeflectionCoverage = 1;
    c->neighbor_scope[0] = 1;
    c->neighbor_scope[1] = 1;
    seedgb_seedfinder_config_setup(c);
}

// spacepoint_grid_config(const seedfinder_config&), seeding_config.hpp:146-157.
void seedgb_spacepoint_grid_config_from_finder(
    seedgb_spacepoint_grid_config* g, const seedgb_seedfinder_config* f) {
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

// seedfilter_config member initialisers, seeding_config.hpp:191-219.
void seedgb_seedfilter_config_default(seedgb_seedfilter_config* c) {
    c->deltaInvHelixDiameter = 0.00003f / kMM;
    c->impactWeightFactor = 1.f;
    c->compatSeedWeight = 200.f;
    c->deltaRMin = 5.f * kMM;
    c->compatSeedLimit = 2;
    c->good_spB_min_radius = 150.f * kMM;
    c->good_spB_weight_increase = 400.f;
    c->good_spT_max_radius = 150.f * kMM;
    c->good_spT_weight_increase = 200.f;
    c->good_spB_min_weight = 380.f;
    c->seed_min_weight = 200.f;
    c->spB_min_radius = 43.f * kMM;
}

// track_params_estimation_config, track_params_estimation_config.hpp:18-33.
void seedgb_track_params_estimation_config_default(
    seedgb_track_params_estimation_config* c) {
    c->initial_sigma[0] = 1.f * kMM;
    c->initial_sigma[1] = 1.f * kMM;
    c->initial_sigma[2] = 1.f * kDegree;
    c->initial_sigma[3] = 1.f * kDegree;
    c->initial_sigma[4] = 0.f * kE / kGeV;
    c->initial_sigma[5] = 1.f * kNs;
    c->initial_sigma_qopt = 0.1f * kE / kGeV;
    c->initial_sigma_pt_rel = 0.1f;
    for (int i = 0; i < 6; ++i) c->initial_inflation[i] = 1.f;
    c->initial_inflation[5] = 100.f;
}

// get_axes, core/include/traccc/seeding/spacepoint_binning_helper.hpp:22-110.
// The two std::domain_error conditions become SEEDGB_BAD_CONFIG.
seedgb_status seedgb_get_axes(const seedgb_spacepoint_grid_config* g,
                              seedgb_grid_axes* out) {
    if (!g || !out) return SEEDGB_INVALID_ARGUMENT;
    unsigned int phiBins;
    if (g->bFieldInZ == 0) {
        phiBins = 100;
    } else {
        const float minHelixRadius = g->minPt / g->bFieldInZ;
        if (minHelixRadius < g->rMax / 2) return SEEDGB_BAD_CONFIG;
        const float maxR2 = g->rMax * g->rMax;
        const float xOuter = maxR2 / (2 * minHelixRadius);
        const float yOuter = std::sqrt(maxR2 - xOuter * xOuter);
        const float outerAngle = std::atan(xOuter / yOuter);
        float innerAngle = 0;
        float rMin = g->rMax;
        if (g->rMax > g->deltaRMax) {
            rMin = g->rMax - g->deltaRMax;
            const float innerCircleR2 =
                (g->rMax - g->deltaRMax) * (g->rMax - g->deltaRMax);
            const float xInner = innerCircleR2 / (2 * minHelixRadius);
            const float yInner = std::sqrt(innerCircleR2 - xInner * xInner);
            innerAngle = std::atan(xInner / yInner);
        }
        const float deltaAngleWithMaxD0 =
            std::fabs(std::asin(g->impactMax / (rMin)) -
                      std::asin(g->impactMax / g->rMax));
        const float deltaPhi = (outerAngle - innerAngle + deltaAngleWithMaxD0) /
                               static_cast<float>(g->phiBinDeflectionCoverage);
        if (!(deltaPhi > 0.)) return SEEDGB_BAD_CONFIG;
        phiBins = static_cast<unsigned int>(std::llround(2 * M_PI / deltaPhi + 0.5));
    }
    const float zBinSize = g->cotThetaMax * g->deltaRMax;
    const unsigned int zb = static_cast<unsigned int>(
        std::floor((g->zMax - g->zMin) / zBinSize));
    out->phi_bins = phiBins;
    out->phi_min = g->phiMin;
    out->phi_max = g->phiMax;
    out->z_bins = zb > 1u ? zb : 1u;
    out->z_min = g->zMin;
    out->z_max = g->zMax;
    return SEEDGB_OK;
}

uint32_t seedgb_abi_version(void) { return SEEDGB_ABI_VERSION; }

const char* seedgb_status_string(seedgb_status s) {
    switch (s) {
        case SEEDGB_OK: return "ok";
        case SEEDGB_EMPTY: return "empty input";
        case SEEDGB_BAD_CONFIG: return "bad configuration";
        case SEEDGB_CUDA_ERROR: return "CUDA error";
        case SEEDGB_CAPACITY_OVERFLOW: return "device buffer capacity exceeded";
        case SEEDGB_TIMEOUT: return "device wait timed out";
        case SEEDGB_INVALID_ARGUMENT: return "invalid argument";
        case SEEDGB_UNSUPPORTED: return "unsupported configuration";
        case SEEDGB_SIZE_LIMIT: return "input larger than the fixed capacity of this entry point";
    }
    return "unknown status";
}

}  // extern "C"
