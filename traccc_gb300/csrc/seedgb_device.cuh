// Device helpers shared by the seeding kernels (seedgb_kernels.cu) and the
// allocation-free binning entry point (seedgb_noalloc.cu): spacepoint
// validity and the (phi, z) grid bin with the reference's float semantics.
// Each translation unit gets its own copy (internal linkage).
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "seedgb_internal.h"

namespace seedgb {
namespace {

__device__ __forceinline__ void raise_status(unsigned long long* ctr,
                                             seedgb_status s) {
    atomicOr(&ctr[kStatus], 1ull << static_cast<int>(s));
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------------------
// Axes (core/include/traccc/seeding/grids/axis.hpp)
// ---------------------------------------------------------------------------

// circular::bin, axis.hpp:277-289
__device__ __forceinline__ uint32_t circular_bin(uint32_t n, float mn, float mx,
                                                 float v) {
    const int ibin = static_cast<int>((v - mn) / (mx - mn) * static_cast<float>(n));
    if (ibin >= 0 && ibin < static_cast<int>(n)) return static_cast<uint32_t>(ibin);
    if (ibin < 0) return n + static_cast<uint32_t>(ibin);
    return static_cast<uint32_t>(ibin) - n;
}

// regular::bin, axis.hpp:87-100 (closed axis)
__device__ __forceinline__ uint32_t regular_bin(uint32_t n, float mn, float mx,
                                                float v) {
    const int ibin = static_cast<int>((v - mn) / (mx - mn) * static_cast<float>(n));
    if (ibin >= 0 && ibin < static_cast<int>(n)) return static_cast<uint32_t>(ibin);
    return ibin < 0 ? 0u : n - 1u;
}

// ---------------------------------------------------------------------------
// Spacepoint classification (core/src/seeding/spacepoint_binning.cpp:39-51,
// spacepoint_binning_helper.hpp:112-127, spacepoint_collection.ipp:52-63)
// ---------------------------------------------------------------------------

// Returns the grid bin of a spacepoint or -1 if is_valid_sp rejects it.  phi is
// the correctly rounded float atan2(y, x): CUDA's atan2f decides it unless the
// value lies within a few ulp of a bin edge or of the phi range limits, where
// the double-precision atan2 rounded to float takes over.  Non-finite
// coordinates are rejected (the reference's size_t / int casts of NaN are
// undefined behaviour).
__device__ int32_t classify(const DevConfig& c, float x, float y, float z,
                            unsigned long long* ctr) {
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) return -1;
    if (z > c.zMax || z < c.zMin) return -1;
    float phi = atan2f(y, x);
    const float v = (phi - c.phi_min) / (c.phi_max - c.phi_min) *
                    static_cast<float>(c.phi_bins);
    const float fr = v - floorf(v);
    const float margin = 4e-6f * static_cast<float>(c.phi_bins) + 1e-5f;
    const float pm = 4e-6f * (1.f + fabsf(phi));
    if (fr < margin || fr > 1.f - margin || fabsf(phi - c.phiMin) <= pm ||
        fabsf(phi - c.phiMax) <= pm) {
        const double r = atan2(static_cast<double>(y), static_cast<double>(x));
        phi = static_cast<float>(r);
        if (r != 0.0) {
            const double f = static_cast<double>(phi);
            const double lo = static_cast<double>(nextafterf(phi, -FLT_MAX * 2.f));
            const double hi = static_cast<double>(nextafterf(phi, FLT_MAX * 2.f));
            const double tol = fabs(r) * 0x1p-44;
            if (fabs(r - 0.5 * (f + lo)) <= tol || fabs(r - 0.5 * (f + hi)) <= tol)
                atomicAdd(&ctr[kPhiUndecided], 1ull);
        }
    }
    if (phi > c.phiMax || phi < c.phiMin) return -1;
    const float bx = x - c.beam0, by = y - c.beam1;
    const float perp = sqrtf(bx * bx + by * by);
    if (!(perp < 1.8e19f)) return -1;
    if (static_cast<unsigned long long>(perp) >= c.nrbins) return -1;
    const uint32_t pb = circular_bin(c.phi_bins, c.phi_min, c.phi_max, phi);
    const uint32_t zb = regular_bin(c.z_bins, c.z_min, c.z_max, z);
    // a grid phi range narrower than the finder's accepts phi values the
    // circular axis cannot wrap; the reference indexes out of its grid there
    if (pb >= c.phi_bins || zb >= c.z_bins) {
        raise_status(ctr, SEEDGB_BAD_CONFIG);
        return -1;
    }
    return static_cast<int32_t>(pb + c.phi_bins * zb);
}

}  // namespace
}  // namespace seedgb
