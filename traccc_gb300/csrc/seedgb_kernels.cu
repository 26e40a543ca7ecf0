// GB300 (sm_103a) kernels of the triplet seeding path.
//
// Pipeline for a batch of events (one launch each, all asynchronous):
//   k_bin_count    validity + (phi, z) bin per spacepoint, per-warp histograms
//   k_bin_scan     per event: stable offsets, bin ranges, work items
//   k_bin_scatter  stable counting-sort scatter into the binned SoA grid
//   k_seed_fast    per work item (event, bin, chunk of middles): stage the
//                  bin's neighbourhood in shared memory; one warp per middle
//                  runs doublet finding (ballot compaction), triplet finding
//                  (cot-sorted middle-top doublets, exact reference cuts),
//                  compatible-seed weights and seed selection
//   k_seed_slow    the same per-middle routine with large capacities, reading
//                  the neighbourhood from global memory, for the few middles
//                  that overflow the fast kernel's shared-memory buffers
//   k_seed_compact per event: seeds in host order into the output buffer
//
// Floating-point semantics follow the reference host code: the file is built
// with -fmad=false --prec-div=true --prec-sqrt=true --ftz=false, and every
// cut is evaluated in the reference's operation order, so decisions are
// bit-identical to the reference's host seeding.
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

// circular::remap, axis.hpp:394-404
__device__ __forceinline__ uint32_t circular_remap(uint32_t n, uint32_t ibin,
                                                   int shood) {
    const int opt = static_cast<int>(ibin) + shood;
    if (opt >= 0 && opt < static_cast<int>(n)) return static_cast<uint32_t>(opt);
    if (opt < 0) return static_cast<uint32_t>(static_cast<int>(n) + opt);
    return static_cast<uint32_t>(opt) - n;
}

// circular::zone_t for a binned neighbourhood, axis.hpp:333-358, including
// its wrap-around order.  Returns the zone length.
__device__ uint32_t phi_zone(const DevConfig& c, uint32_t pbin, uint32_t* out,
                             uint32_t cap) {
    const uint32_t n = c.phi_bins;
    const uint32_t lo = circular_remap(n, pbin, -static_cast<int>(c.scope0));
    const uint32_t hi = circular_remap(n, pbin, static_cast<int>(c.scope1));
    if (lo < hi) {
        const uint32_t len = hi - lo + 1u;
        for (uint32_t i = 0; i < len && i < cap; ++i) out[i] = lo + i;
        return len;
    }
    const uint32_t vl = n - lo + hi + 1u;
    uint32_t mi = 0, mo = 0;
    for (uint32_t i = 0; i < vl; ++i) {
        uint32_t b = lo + mi++;
        if (b > n - 1u) b = mo++;
        if (i < cap) out[i] = b;
    }
    return vl;
}

// regular::range for a binned neighbourhood (axis.hpp:110-123), evaluated at
// the raw (unclamped) bin index of z.
__device__ __forceinline__ void z_range(const DevConfig& c, float z,
                                        uint32_t& lo, uint32_t& hi) {
    const int ibin = static_cast<int>((z - c.z_min) / (c.z_max - c.z_min) *
                                      static_cast<float>(c.z_bins));
    const int imin = ibin - static_cast<int>(c.scope0);
    const int imax = ibin + static_cast<int>(c.scope1);
    lo = imin >= 0 ? static_cast<uint32_t>(imin) : 0u;
    hi = imax < static_cast<int>(c.z_bins) ? static_cast<uint32_t>(imax)
                                           : c.z_bins - 1u;
}

// Neighbourhood segments of (phi bin, z range): phi outer, z inner, in-bin
// order (core/src/seeding/doublet_finding.hpp:74-106).  seg_pos is a prefix
// array of positions, seg_g the first grid position of each segment.
__device__ uint32_t build_segments(const DevConfig& c, const uint32_t* bs,
                                   uint32_t pbin, uint32_t zlo, uint32_t zhi,
                                   uint32_t* seg_pos, uint32_t* seg_g,
                                   uint32_t* nseg_out) {
    uint32_t phis[kMaxSegments];
    const uint32_t np = phi_zone(c, pbin, phis, kMaxSegments);
    const uint32_t nzz = zhi + 1u - zlo;  // zone length (may be 0)
    uint32_t ns = 0, pos = 0;
    for (uint32_t ip = 0; ip < np && ip < kMaxSegments; ++ip) {
        for (uint32_t iz = 0; iz < nzz; ++iz) {
            if (ns >= kMaxSegments) break;
            const uint32_t bin = phis[ip] + (zlo + iz) * c.phi_bins;
            seg_pos[ns] = pos;
            seg_g[ns] = bs[bin];
            pos += bs[bin + 1] - bs[bin];
            ++ns;
        }
    }
    seg_pos[ns] = pos;
    *nseg_out = ns;
    return pos;
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

__device__ __forceinline__ uint32_t event_of_chunk(const Arena& a, uint32_t chunk) {
    uint32_t lo = 0, hi = a.n_events;  // last event with chunk_base <= chunk
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a.events[mid].chunk_base <= chunk) lo = mid; else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Binning
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kBinWarps * 32)
k_bin_count(DevConfig c, Arena a) {
    extern __shared__ uint32_t hist[];  // [kBinWarps][nbins]
    const uint32_t chunk = blockIdx.x;
    if (chunk >= a.total_chunks) return;
    const uint32_t e = event_of_chunk(a, chunk);
    const EventDesc ev = a.events[e];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t i = threadIdx.x; i < kBinWarps * c.nbins; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    uint32_t* h = hist + warp * c.nbins;
    const uint32_t base = (chunk - ev.chunk_base) * kBinChunk + warp * (kBinRounds * 32);
    bool anyvar = false;
#pragma unroll 2
    for (int r = 0; r < kBinRounds; ++r) {
        const uint32_t i = base + r * 32 + lane;
        if (i < ev.n_sp) {
            const float x = ev.global[3 * i], y = ev.global[3 * i + 1],
                        z = ev.global[3 * i + 2];
            const int32_t bin = classify(c, x, y, z, a.counters);
            a.sp_bin[ev.sp_base + i] = bin;
            if (bin >= 0) atomicAdd(&h[bin], 1u);
            anyvar |= (ev.zvar && ev.zvar[i] != 0.f) || (ev.rvar && ev.rvar[i] != 0.f);
        }
    }
    if (__any_sync(0xffffffffu, anyvar) && lane == 0)
        atomicOr(&a.counters[kAnyVariance], 1ull);
    __syncthreads();
    uint32_t* out = a.whist + static_cast<size_t>(chunk) * kBinWarps * c.nbins;
    for (uint32_t i = threadIdx.x; i < kBinWarps * c.nbins; i += blockDim.x) out[i] = hist[i];
}

// Block-wide exclusive scan of n values in shared memory (n <= 64k).
__device__ uint32_t block_exclusive_scan(uint32_t* data, uint32_t n, uint32_t* tmp) {
    const uint32_t nt = blockDim.x, t = threadIdx.x;
    const uint32_t per = (n + nt - 1) / nt;
    const uint32_t b0 = min(n, t * per), b1 = min(n, b0 + per);
    uint32_t s = 0;
    for (uint32_t i = b0; i < b1; ++i) s += data[i];
    // warp scan of per-thread sums
    const uint32_t lane = t & 31, warp = t >> 5;
    uint32_t incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += v;
    }
    if (lane == 31) tmp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t nw = (nt + 31) / 32;
        uint32_t w = lane < nw ? tmp[lane] : 0u;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= static_cast<uint32_t>(o)) wi += v;
        }
        if (lane < nw) tmp[lane] = wi - w;
        if (lane == 31) tmp[32] = wi;
    }
    __syncthreads();
    uint32_t run = tmp[warp] + incl - s;
    for (uint32_t i = b0; i < b1; ++i) {
        const uint32_t v = data[i];
        data[i] = run;
        run += v;
    }
    const uint32_t total = tmp[32];
    __syncthreads();
    return total;
}

// One CTA per event: turns the per-(chunk, warp) histograms into absolute
// grid positions (bin-major, then spacepoint order), the bin ranges, the
// number of valid spacepoints and the event's work items.
__global__ void __launch_bounds__(1024) k_bin_scan(DevConfig c, Arena a, uint32_t mpi) {
    extern __shared__ uint32_t sh[];
    const uint32_t e = blockIdx.x;
    if (e >= a.n_events) return;
    const EventDesc ev = a.events[e];
    const uint32_t nb = c.nbins;
    const uint32_t nslots = ev.n_chunks * kBinWarps;
    const uint32_t G = max(1u, min(blockDim.x / nb, max(1u, nslots)));
    const uint32_t per = (nslots + G - 1) / G;
    uint32_t* gs = sh;                 // [G][nb] group sums -> group offsets
    uint32_t* tot = gs + G * nb;       // [nb] bin totals -> bin starts
    uint32_t* items = tot + nb;        // [nb] items per bin -> item prefix
    uint32_t* tmp = items + nb;        // [33]
    uint32_t* whist = a.whist + static_cast<size_t>(ev.chunk_base) * kBinWarps * nb;
    for (uint32_t idx = threadIdx.x; idx < G * nb; idx += blockDim.x) {
        const uint32_t b = idx % nb, g = idx / nb;
        uint32_t s = 0;
        const uint32_t s0 = g * per, s1 = min(nslots, s0 + per);
        for (uint32_t k = s0; k < s1; ++k) s += whist[static_cast<size_t>(k) * nb + b];
        gs[g * nb + b] = s;
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        uint32_t run = 0;
        for (uint32_t g = 0; g < G; ++g) {
            const uint32_t v = gs[g * nb + b];
            gs[g * nb + b] = run;
            run += v;
        }
        tot[b] = run;
        items[b] = (run + mpi - 1) / mpi;
    }
    __syncthreads();
    const uint32_t n_valid = block_exclusive_scan(tot, nb, tmp);
    const uint32_t n_items = block_exclusive_scan(items, nb, tmp);
    uint32_t* bs = a.bin_start + static_cast<size_t>(e) * (nb + 1);
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) bs[b] = ev.sp_base + tot[b];
    if (threadIdx.x == 0) {
        bs[nb] = ev.sp_base + n_valid;
        a.n_valid[e] = n_valid;
        atomicAdd(&a.counters[kNumValid], static_cast<unsigned long long>(n_valid));
        tmp[0] = static_cast<uint32_t>(
            atomicAdd(&a.counters[kItemTotal], static_cast<unsigned long long>(n_items)));
    }
    __syncthreads();
    const uint32_t item_base = tmp[0];
    // absolute positions for every (chunk, warp, bin)
    for (uint32_t idx = threadIdx.x; idx < G * nb; idx += blockDim.x) {
        const uint32_t b = idx % nb, g = idx / nb;
        uint32_t run = ev.sp_base + tot[b] + gs[g * nb + b];
        const uint32_t s0 = g * per, s1 = min(nslots, s0 + per);
        for (uint32_t k = s0; k < s1; ++k) {
            uint32_t* p = &whist[static_cast<size_t>(k) * nb + b];
            const uint32_t v = *p;
            *p = run;
            run += v;
        }
    }
    // work items: (event, bin | chunk << 16)
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        const uint32_t i0 = items[b];
        const uint32_t i1 = (b + 1 < nb) ? items[b + 1] : n_items;
        for (uint32_t k = i0; k < i1 && item_base + k < a.max_items; ++k)
            a.items[item_base + k] = make_uint2(e, b | ((k - i0) << 16));
    }
    if (threadIdx.x == 0 && item_base + n_items > a.max_items)
        raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
}

__global__ void __launch_bounds__(kBinWarps * 32) k_bin_scatter(DevConfig c, Arena a) {
    extern __shared__ uint32_t base[];  // [kBinWarps][nbins]
    const uint32_t chunk = blockIdx.x;
    if (chunk >= a.total_chunks) return;
    const uint32_t e = event_of_chunk(a, chunk);
    const EventDesc ev = a.events[e];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t* src = a.whist + static_cast<size_t>(chunk) * kBinWarps * c.nbins;
    for (uint32_t i = threadIdx.x; i < kBinWarps * c.nbins; i += blockDim.x) base[i] = src[i];
    __syncthreads();
    uint32_t* wb = base + warp * c.nbins;
    const uint32_t b0 = (chunk - ev.chunk_base) * kBinChunk + warp * (kBinRounds * 32);
    const uint32_t lt = lanemask_lt();
    for (int r = 0; r < kBinRounds; ++r) {
        const uint32_t i = b0 + r * 32 + lane;
        const int32_t bin = (i < ev.n_sp) ? a.sp_bin[ev.sp_base + i] : -1;
        const uint32_t peers = __match_any_sync(0xffffffffu, bin);
        const uint32_t rank = __popc(peers & lt);
        if (bin >= 0) {
            const uint32_t pos = wb[bin] + rank;
            const float x = ev.global[3 * i], y = ev.global[3 * i + 1],
                        z = ev.global[3 * i + 2];
            // spacepoint::radius, spacepoint_collection.ipp:52-57
            a.g_xyzr[pos] = make_float4(x, y, z, sqrtf(x * x + y * y));
            a.g_var[pos] = make_float2(ev.zvar ? ev.zvar[i] : 0.f, ev.rvar ? ev.rvar[i] : 0.f);
            a.g_idx[pos] = i;
        }
        __syncwarp();
        if (bin >= 0 && rank == 0) wb[bin] += __popc(peers);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Doublet and triplet cuts (exact reference arithmetic)
// ---------------------------------------------------------------------------

struct LinCircle {
    float Zo, cot, idr, er, u, v;
};

// First part of doublet_finding_helper::isCompatible<bottom>
// (doublet_finding_helper.hpp:59-82): r, z windows and the z-origin window.
__device__ __forceinline__ bool window_bottom(const DevConfig& c, const float4 m,
                                              const float4 o) {
    const float deltaR = m.w - o.w;
    const float cotTheta = m.z - o.z;
    const float zOrigin = m.z * deltaR - m.w * cotTheta;
    return !((deltaR >= c.deltaRMax) || (deltaR <= c.deltaRMin) ||
             (fabsf(cotTheta) >= c.cotThetaMax * deltaR) ||
             (zOrigin <= c.collisionRegionMin * deltaR) ||
             (zOrigin >= c.collisionRegionMax * deltaR) ||
             fabsf(cotTheta) >= c.deltaZMax);
}

// Same for isCompatible<top> (doublet_finding_helper.hpp:67-74).
__device__ __forceinline__ bool window_top(const DevConfig& c, const float4 m,
                                           const float4 o) {
    const float deltaR = o.w - m.w;
    const float cotTheta = (o.z - m.z);
    const float zOrigin = m.z * deltaR - m.w * cotTheta;
    return !((deltaR >= c.deltaRMax) || (deltaR <= c.deltaRMin) ||
             (fabsf(cotTheta) >= c.cotThetaMax * deltaR) ||
             (zOrigin <= c.collisionRegionMin * deltaR) ||
             (zOrigin >= c.collisionRegionMax * deltaR) ||
             fabsf(cotTheta) >= c.deltaZMax);
}

// Second part of isCompatible: the minimum-helix-radius circle test
// (doublet_finding_helper.hpp:84-213).  std::min keeps (b < a) ? b : a.
__device__ __forceinline__ bool helix_ok(const DevConfig& c, const float4 m,
                                         const float4 o) {
    const float midX = 0.5f * (m.x + o.x);
    const float midY = 0.5f * (m.y + o.y);
    const float slope = (o.y - m.y) / (o.x - m.x);
    const float deltaX = o.x - m.x;
    const float deltaY = o.y - m.y;
    const float deltaXY2 = deltaX * deltaX + deltaY * deltaY;
    const float sagittaLength =
        sqrtf(c.minHelixRadius * c.minHelixRadius - deltaXY2 / 4.f);
    const float denom = sqrtf((slope * slope + 1) / (slope * slope));
    const float cosCentralAngle = 1.f / denom;
    const float sinCentralAngle = -1.f / (slope * denom);
    const float mpDeltaX = sagittaLength * cosCentralAngle;
    const float mpDeltaY = sagittaLength * sinCentralAngle;
    const float mp1X = midX + mpDeltaX;
    const float mp2X = midX - mpDeltaX;
    const float mp1Y = midY + mpDeltaY;
    const float mp2Y = midY - mpDeltaY;
    const float mp1R2 = mp1X * mp1X + mp1Y * mp1Y;
    const float mp2R2 = mp2X * mp2X + mp2Y * mp2Y;
    const float mn = (mp2R2 < mp1R2) ? mp2R2 : mp1R2;
    return !(mn <= ((c.minHelixRadius - c.impactMax) *
                    (c.minHelixRadius - c.impactMax)));
}

// doublet_finding_helper::transform_coordinates, doublet_finding_helper.hpp:
// 218-272.  vm/vo = (z_variance, radius_variance).
__device__ __forceinline__ LinCircle lin_circle(bool top, const float4 m,
                                                const float2 vm, const float4 o,
                                                const float2 vo) {
    const float cosPhiM = m.x / m.w;
    const float sinPhiM = m.y / m.w;
    const float deltaX = o.x - m.x;
    const float deltaY = o.y - m.y;
    const float deltaZ = o.z - m.z;
    const float x = deltaX * cosPhiM + deltaY * sinPhiM;
    const float y = deltaY * cosPhiM - deltaX * sinPhiM;
    const float iDeltaR2 = 1.f / (deltaX * deltaX + deltaY * deltaY);
    const float iDeltaR = sqrtf(iDeltaR2);
    float cot_theta = deltaZ * iDeltaR;
    if (!top) cot_theta = -cot_theta;
    LinCircle l;
    l.cot = cot_theta;
    l.Zo = m.z - m.w * cot_theta;
    l.idr = iDeltaR;
    l.u = x * iDeltaR2;
    l.v = y * iDeltaR2;
    l.er = ((vm.x + vo.x) + (cot_theta * cot_theta) * (vm.y + vo.y)) * iDeltaR2;
    return l;
}

// triplet_finding_helper::isCompatible, triplet_finding_helper.hpp:42-133.
__device__ __forceinline__ bool triplet_ok(const DevConfig& c, const float rM,
                                           const float2 vm, const LinCircle& lb,
                                           const float ltCot, const float ltIdr,
                                           const float ltEr, const float ltU,
                                           const float ltV, const float iSinTheta2,
                                           const float scatteringInRegion2,
                                           float& curvature, float& impact) {
    const float error2 =
        ltEr + lb.er + 2.f * (lb.cot * ltCot * vm.y + vm.x) * lb.idr * ltIdr;
    float deltaCotTheta = lb.cot - ltCot;
    const float deltaCotTheta2 = deltaCotTheta * deltaCotTheta;
    float error = 0.f;
    float dCotThetaMinusError2 = 0.f;
    if (deltaCotTheta2 - error2 > 0) {
        deltaCotTheta = fabsf(deltaCotTheta);
        error = sqrtf(error2);
        dCotThetaMinusError2 =
            deltaCotTheta2 + error2 - 2.f * deltaCotTheta * error;
        if (dCotThetaMinusError2 > scatteringInRegion2) return false;
    }
    const float dU = ltU - lb.u;
    if (dU == 0.f) return false;
    const float A = (ltV - lb.v) / dU;
    const float S2 = 1.f + A * A;
    const float B = lb.v - A * lb.u;
    const float B2 = B * B;
    if (S2 < B2 * c.minHelixDiameter2) return false;
    const float iHelixDiameter2 = B2 / S2;
    float pT2scatter = 4.f * iHelixDiameter2 * c.pT2perRadius;
    const float pT = c.pTPerHelixRadius * sqrtf(S2 / B2) / 2.f;
    if (pT > c.maxPtScattering) {
        const float pTscatter = c.highland / c.maxPtScattering;
        pT2scatter = pTscatter * pTscatter;
    }
    const float p2scatter = pT2scatter * iSinTheta2;
    if ((deltaCotTheta2 - error2 > 0.f) &&
        (dCotThetaMinusError2 >
         p2scatter * c.sigmaScattering * c.sigmaScattering))
        return false;
    curvature = B / sqrtf(S2);
    impact = fabsf((A - B * rM) * rM);
    if (impact > c.impactMax) return false;
    return true;
}

// triplet_sorter (core/include/traccc/seeding/detail/triplet_sorter.hpp:39-71):
// weight descending, then sum y^2+z^2 of bottom and top descending; exact ties
// keep the host triplet order (middle-bottom index, then middle-top index).
__device__ __forceinline__ bool better(float wa, float sa, uint32_t ka, float wb,
                                       float sb, uint32_t kb) {
    if (wa != wb) return wa > wb;
    if (sa != sb) return sa > sb;
    return ka < kb;
}

// ---------------------------------------------------------------------------
// Per-middle seeding routine
// ---------------------------------------------------------------------------

// Neighbourhood of a middle spacepoint: a concatenation of grid bins, either
// staged in shared memory or read from the binned grid in global memory.
struct NbView {
    const float4* staged;    // nullptr: read from g_xyzr
    const float4* g_xyzr;
    const uint32_t* seg_pos; // [nseg + 1]
    const uint32_t* seg_g;   // [nseg]
    uint32_t nseg;
    uint32_t size;

    __device__ __forceinline__ uint32_t gpos(uint32_t p) const {
        uint32_t s = 0;
        while (s + 1 < nseg && seg_pos[s + 1] <= p) ++s;
        return seg_g[s] + (p - seg_pos[s]);
    }
    __device__ __forceinline__ float4 get(uint32_t p) const {
        return staged ? staged[p] : g_xyzr[gpos(p)];
    }
};

template <int CAPB, int CAPT, int CAPLC>
struct WarpScratch {
    float key[CAPLC];  // cot theta of the middle-top doublets, sorted
    float idr[CAPLC], er[CAPLC], u[CAPLC], v[CAPLC];  // in list order
    uint16_t perm[CAPLC];                              // sorted -> list index
    uint16_t qb[CAPB];  // middle-bottom doublets (neighbourhood positions)
    uint16_t qt[CAPT];  // middle-top doublets
};

using FastScratch = WarpScratch<1024, 512, 256>;
constexpr int kFastTcap = 8;
using SlowScratch = WarpScratch<8192, 8192, 4096>;
constexpr int kSlowTcap = 64;

// Keep the positions that pass `pred` (in order) in q[0..n).
template <bool TOP>
__device__ __forceinline__ uint32_t helix_compact(const DevConfig& c, const NbView& nb,
                                                  const float4 m, uint16_t* q,
                                                  uint32_t n, uint32_t lane,
                                                  uint32_t lt) {
    uint32_t w = 0;
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i = base + lane;
        bool ok = false;
        uint16_t p = 0;
        if (i < n) {
            p = q[i];
            ok = helix_ok(c, m, nb.get(p));
        }
        __syncwarp();
        const uint32_t mask = __ballot_sync(0xffffffffu, ok);
        if (ok) q[w + __popc(mask & lt)] = p;
        w += __popc(mask);
        __syncwarp();
    }
    return w;
}

struct MiddleResult {
    uint32_t n_mb, n_mt, n_trip;
    int status;  // 0 done, 1 needs the large-capacity path
};

// Seeds of one middle spacepoint, following host seed_finding::operator()
// (core/src/seeding/seed_finding.cpp:69-118) with triplet_finding
// (triplet_finding.hpp:60-183) and seed_filtering (seed_filtering.cpp:28-123).
// Executed by one full warp.
template <int CAPB, int CAPT, int CAPLC, int TCAP>
__device__ MiddleResult process_middle(const DevConfig& c, const Arena& a,
                                       const NbView& nb, const uint32_t gm,
                                       const bool any_var, const bool check_r,
                                       const float nb_minr, const float nb_maxr,
                                       WarpScratch<CAPB, CAPT, CAPLC>& ws) {
    constexpr int kUnroll = TCAP <= 8 ? TCAP : 1;
    MiddleResult res{0, 0, 0, 0};
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt = lanemask_lt();
    const float4 M = a.g_xyzr[gm];
    const float2 vM = any_var ? a.g_var[gm] : make_float2(0.f, 0.f);

    if (check_r) {
        // fl(rM - r) is non-increasing in r: if the smallest radius of the
        // neighbourhood cannot make deltaR > deltaRMin, no bottom passes;
        // likewise for tops with the largest radius.
        const float db = M.w - nb_minr, dt = nb_maxr - M.w;
        const float db2 = M.w - nb_maxr, dt2 = nb_minr - M.w;
        if (!(db > c.deltaRMin) || !(dt > c.deltaRMin) || (db2 >= c.deltaRMax) ||
            (dt2 >= c.deltaRMax)) {
            if (lane == 0) a.seed_cnt[gm] = 0;
            return res;
        }
    }

    // -- doublets: window cuts with ballot compaction, in neighbourhood order
    uint32_t nqb = 0, nqt = 0;
    for (uint32_t base = 0; base < nb.size; base += 32) {
        const uint32_t p = base + lane;
        bool pb = false, pt = false;
        if (p < nb.size) {
            const float4 o = nb.get(p);
            pb = window_bottom(c, M, o);
            pt = window_top(c, M, o);
        }
        const uint32_t mb = __ballot_sync(0xffffffffu, pb);
        const uint32_t mt = __ballot_sync(0xffffffffu, pt);
        if (pb) {
            const uint32_t k = nqb + __popc(mb & lt);
            if (k < CAPB) ws.qb[k] = static_cast<uint16_t>(p);
        }
        if (pt) {
            const uint32_t k = nqt + __popc(mt & lt);
            if (k < CAPT) ws.qt[k] = static_cast<uint16_t>(p);
        }
        nqb += __popc(mb);
        nqt += __popc(mt);
    }
    if (nqb > CAPB || nqt > CAPT) { res.status = 1; return res; }
    __syncwarp();
    const uint32_t n_mb = nqb ? helix_compact<false>(c, nb, M, ws.qb, nqb, lane, lt) : 0u;
    const uint32_t n_mt =
        (n_mb && nqt) ? helix_compact<true>(c, nb, M, ws.qt, nqt, lane, lt) : 0u;
    res.n_mb = n_mb;
    res.n_mt = n_mt;
    if (n_mb == 0 || n_mt == 0) {
        if (lane == 0) a.seed_cnt[gm] = 0;
        return res;
    }
    if (n_mt > CAPLC) { res.status = 1; return res; }

    // -- middle-top lin_circles, sorted by cot(theta)
    float maxEr = 0.f, minEr = 0.f, maxCot = 0.f, maxIdr = 0.f;
    for (uint32_t i = lane; i < n_mt; i += 32) {
        const uint32_t p = ws.qt[i];
        const float2 vo = any_var ? a.g_var[nb.gpos(p)] : make_float2(0.f, 0.f);
        const LinCircle l = lin_circle(true, M, vM, nb.get(p), vo);
        ws.key[i] = l.cot;
        ws.idr[i] = l.idr;
        ws.er[i] = l.er;
        ws.u[i] = l.u;
        ws.v[i] = l.v;
        ws.perm[i] = static_cast<uint16_t>(i);
        maxEr = fmaxf(maxEr, l.er);
        minEr = fminf(minEr, l.er);
        maxCot = fmaxf(maxCot, fabsf(l.cot));
        maxIdr = fmaxf(maxIdr, l.idr);
        if (!(l.er == l.er)) minEr = -1.f;  // NaN error term: no window
    }
    uint32_t P = 1;
    while (P < n_mt) P <<= 1;
    for (uint32_t i = n_mt + lane; i < P; i += 32) {
        ws.key[i] = __int_as_float(0x7f800000);
        ws.perm[i] = 0xffff;
    }
    __syncwarp();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = lane; t < P / 2; t += 32) {
                const uint32_t i = 2 * t - (t & (j - 1));
                const uint32_t l = i + j;
                const bool up = (i & k) == 0;
                const float ki = ws.key[i], kl = ws.key[l];
                if (up ? (ki > kl) : (ki < kl)) {
                    ws.key[i] = kl;
                    ws.key[l] = ki;
                    const uint16_t pi = ws.perm[i];
                    ws.perm[i] = ws.perm[l];
                    ws.perm[l] = pi;
                }
            }
            __syncwarp();
        }
    }
    if (any_var) {
        for (int o = 16; o > 0; o >>= 1) {
            maxEr = fmaxf(maxEr, __shfl_xor_sync(0xffffffffu, maxEr, o));
            minEr = fminf(minEr, __shfl_xor_sync(0xffffffffu, minEr, o));
            maxCot = fmaxf(maxCot, __shfl_xor_sync(0xffffffffu, maxCot, o));
            maxIdr = fmaxf(maxIdr, __shfl_xor_sync(0xffffffffu, maxIdr, o));
        }
    }

    // -- triplets per middle-bottom doublet, weights, lane-local best seeds
    const uint32_t K = min(c.maxSeedsPerSpM, static_cast<uint32_t>(kMaxSeedsPerMiddle));
    float bw[kMaxSeedsPerMiddle], bs[kMaxSeedsPerMiddle];
    uint32_t bk[kMaxSeedsPerMiddle], bp[kMaxSeedsPerMiddle];
#pragma unroll
    for (int k = 0; k < kMaxSeedsPerMiddle; ++k) {
        bw[k] = -__int_as_float(0x7f800000);
        bs[k] = 0.f;
        bk[k] = 0xffffffffu;
        bp[k] = 0;
    }
    uint32_t bn = 0;
    bool lane_ovf = false;
    uint32_t n_trip = 0;
    const float sig2 = c.sigmaScattering * c.sigmaScattering;

    for (uint32_t ib = lane; ib < n_mb && !lane_ovf; ib += 32) {
        const uint32_t pB = ws.qb[ib];
        const float4 B = nb.get(pB);
        const float2 vB = any_var ? a.g_var[nb.gpos(pB)] : make_float2(0.f, 0.f);
        const LinCircle lb = lin_circle(false, M, vM, B, vB);
        // triplet_finding.hpp:82-88
        const float iSinTheta2 = 1.f + lb.cot * lb.cot;
        float scatteringInRegion2 = c.maxScatteringAngle2 * iSinTheta2;
        scatteringInRegion2 *= sig2;

        // Window in cot(theta): a middle-top doublet outside it fails the
        // reference's first scattering test for any rounding (1 % relative
        // and 1e-5 absolute margins), so only doublets inside are tested.
        float W;
        if (c.brute_force_triplets) {
            W = __int_as_float(0x7f800000);
        } else if (!any_var) {
            W = sqrtf(scatteringInRegion2) * 1.01f + 1e-5f * (1.f + fabsf(lb.cot));
        } else {
            const float e2 = (maxEr + lb.er +
                              2.f * (fabsf(lb.cot) * maxCot * fabsf(vM.y) + fabsf(vM.x)) *
                                  lb.idr * maxIdr) * 1.001f;
            const bool ok = (minEr >= 0.f) && (lb.er >= 0.f) && (vM.x >= 0.f) &&
                            (vM.y >= 0.f) && (e2 >= 0.f) && (e2 < 3.0e38f);
            W = ok ? (sqrtf(scatteringInRegion2) + sqrtf(e2)) * 1.01f +
                         1e-5f * (1.f + fabsf(lb.cot))
                   : __int_as_float(0x7f800000);
        }
        const float klo = lb.cot - W, khi = lb.cot + W;
        uint32_t lo = 0, hi = n_mt;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (ws.key[mid] < klo) lo = mid + 1; else hi = mid;
        }
        // candidate triplets of this middle-bottom doublet (list order later)
        uint32_t tt[TCAP];
        float tcv[TCAP], twt[TCAP];
        uint32_t nt = 0;
        for (uint32_t s = lo; s < n_mt && ws.key[s] <= khi; ++s) {
            const uint32_t tp = ws.perm[s];
            float curvature, impact;
            if (!triplet_ok(c, M.w, vM, lb, ws.key[s], ws.idr[tp], ws.er[tp],
                            ws.u[tp], ws.v[tp], iSinTheta2, scatteringInRegion2,
                            curvature, impact))
                continue;
            if (nt == TCAP) { lane_ovf = true; break; }
#pragma unroll kUnroll
            for (int k = 0; k < TCAP; ++k) {
                if (k == static_cast<int>(nt)) {
                    tt[k] = tp;
                    tcv[k] = curvature;
                    twt[k] = -impact * c.impactWeightFactor;
                }
            }
            ++nt;
        }
        if (lane_ovf || nt == 0) continue;
        n_trip += nt;
        // host order of the triplets of this doublet: middle-top list order
        if (nt > 1) {
#pragma unroll kUnroll
            for (int pass = 0; pass < TCAP - 1; ++pass) {
#pragma unroll kUnroll
                for (int k = 0; k + 1 < TCAP; ++k) {
                    if (k + 1 < static_cast<int>(nt) && tt[k] > tt[k + 1]) {
                        const uint32_t a0 = tt[k]; tt[k] = tt[k + 1]; tt[k + 1] = a0;
                        const float c0 = tcv[k]; tcv[k] = tcv[k + 1]; tcv[k + 1] = c0;
                        const float w0 = twt[k]; twt[k] = twt[k + 1]; twt[k + 1] = w0;
                    }
                }
            }
        }
        float trT[TCAP];
#pragma unroll kUnroll
        for (int k = 0; k < TCAP; ++k)
            trT[k] = (k < static_cast<int>(nt)) ? nb.get(ws.qt[tt[k]]).w : 0.f;
        // compatible-seed weights, triplet_finding.hpp:107-179
        if (nt > 1) {
#pragma unroll kUnroll
            for (int i = 0; i < TCAP; ++i) {
                if (i >= static_cast<int>(nt)) break;
                const float currentTop_r = trT[i];
                const float lowerLimitCurv = tcv[i] - c.deltaInvHelixDiameter;
                const float upperLimitCurv = tcv[i] + c.deltaInvHelixDiameter;
                float compR[8];
                uint32_t ncr = 0;
                float w = twt[i];
                for (int j = 0; j < TCAP; ++j) {
                    if (j >= static_cast<int>(nt)) break;
                    if (i == j) continue;
                    const float otherTop_r = trT[j];
                    const float deltaR = currentTop_r - otherTop_r;
                    if (fabsf(deltaR) < c.filterDeltaRMin) continue;
                    if (tcv[j] < lowerLimitCurv) continue;
                    if (tcv[j] > upperLimitCurv) continue;
                    bool newCompSeed = true;
                    for (uint32_t q = 0; q < ncr; ++q) {
                        if (fabsf(compR[q] - otherTop_r) < c.filterDeltaRMin) {
                            newCompSeed = false;
                            break;
                        }
                    }
                    if (newCompSeed) {
                        if (ncr < 8) compR[ncr] = otherTop_r;
                        ++ncr;
                        w += c.compatSeedWeight;
                    }
                    if (ncr >= c.compatSeedLimit) break;
                }
                twt[i] = w;
            }
        }
        // seed_selecting_helper::seed_weight / single_seed_cut
        // (seed_selecting_helper.hpp:27-62), then the per-lane best list
#pragma unroll kUnroll
        for (int i = 0; i < TCAP; ++i) {
            if (i >= static_cast<int>(nt)) break;
            float weight = 0;
            if (B.w > c.good_spB_min_radius) weight = c.good_spB_weight_increase;
            if (trT[i] < c.good_spT_max_radius) weight = c.good_spT_weight_increase;
            const float w = twt[i] + weight;
            if (B.w > c.good_spB_min_radius && w < c.good_spB_min_weight) continue;
            const float4 T = nb.get(ws.qt[tt[i]]);
            const float s = B.y * B.y + B.z * B.z + T.y * T.y + T.z * T.z;
            const uint32_t key = (ib << 16) | tt[i];
            // insertion into the sorted best-K list
            uint32_t pos = 0;
#pragma unroll
            for (int k = 0; k < kMaxSeedsPerMiddle; ++k)
                if (k < static_cast<int>(bn) && better(bw[k], bs[k], bk[k], w, s, key)) ++pos;
            if (pos < K) {
#pragma unroll
                for (int k = kMaxSeedsPerMiddle - 1; k > 0; --k) {
                    if (k > static_cast<int>(pos)) {
                        bw[k] = bw[k - 1]; bs[k] = bs[k - 1];
                        bk[k] = bk[k - 1]; bp[k] = bp[k - 1];
                    }
                }
#pragma unroll
                for (int k = 0; k < kMaxSeedsPerMiddle; ++k) {
                    if (k == static_cast<int>(pos)) {
                        bw[k] = w; bs[k] = s; bk[k] = key;
                        bp[k] = (static_cast<uint32_t>(pB) << 16) | ws.qt[tt[i]];
                    }
                }
                bn = min(bn + 1, K);
            }
        }
    }
    if (__any_sync(0xffffffffu, lane_ovf)) { res.status = 1; return res; }

    // -- warp merge of the lane-local lists: the global best K in order
    float my_w = 0.f;
    uint32_t my_p = 0;
    uint32_t n_sel = 0;
    for (uint32_t r = 0; r < K; ++r) {
        float cw = bn > 0 ? bw[0] : -__int_as_float(0x7f800000);
        float cs = bn > 0 ? bs[0] : 0.f;
        uint32_t ck = bn > 0 ? bk[0] : 0xffffffffu;
        uint32_t cl = lane;
        for (int o = 16; o > 0; o >>= 1) {
            const float ow = __shfl_xor_sync(0xffffffffu, cw, o);
            const float os = __shfl_xor_sync(0xffffffffu, cs, o);
            const uint32_t ok = __shfl_xor_sync(0xffffffffu, ck, o);
            const uint32_t ol = __shfl_xor_sync(0xffffffffu, cl, o);
            if (better(ow, os, ok, cw, cs, ck)) { cw = ow; cs = os; ck = ok; cl = ol; }
        }
        if (ck == 0xffffffffu) break;
        const uint32_t wp = __shfl_sync(0xffffffffu, bp[0], cl);
        if (lane == cl) {
#pragma unroll
            for (int k = 0; k + 1 < kMaxSeedsPerMiddle; ++k) {
                bw[k] = bw[k + 1]; bs[k] = bs[k + 1]; bk[k] = bk[k + 1]; bp[k] = bp[k + 1];
            }
            --bn;
        }
        if (lane == r) { my_w = cw; my_p = wp; }
        ++n_sel;
    }
    // -- final selection (seed_filtering.cpp:87-122): the first is always
    //    accepted, the next ones if cut_per_middle_sp holds
    bool acc = false;
    float4 Bsel = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < n_sel) {
        Bsel = nb.get(my_p >> 16);
        acc = (lane == 0) || (my_w > c.seed_min_weight) || (Bsel.w > c.spB_min_radius);
    }
    const uint32_t amask = __ballot_sync(0xffffffffu, acc);
    if (acc) {
        const uint32_t k = __popc(amask & lt);
        SeedSlot s;
        s.b = a.g_idx[nb.gpos(my_p >> 16)];
        s.m = a.g_idx[gm];
        s.t = a.g_idx[nb.gpos(my_p & 0xffffu)];
        s.q = my_w;
        a.seed_slot[static_cast<size_t>(gm) * kMaxSeedsPerMiddle + k] = s;
    }
    if (lane == 0) a.seed_cnt[gm] = static_cast<uint8_t>(__popc(amask));
    uint32_t tsum = n_trip;
    for (int o = 16; o > 0; o >>= 1) tsum += __shfl_xor_sync(0xffffffffu, tsum, o);
    res.n_trip = tsum;
    return res;
}

__device__ __forceinline__ void push_overflow(const Arena& a, uint32_t gm) {
    const unsigned long long k = atomicAdd(&a.counters[kOvfCount], 1ull);
    if (k < a.total_sp) a.ovf[k] = gm;
    a.seed_cnt[gm] = 0;
}

__device__ __forceinline__ void count_middle(const Arena& a, const MiddleResult& r) {
    if (r.n_mb) atomicAdd(&a.counters[kNumMB], static_cast<unsigned long long>(r.n_mb));
    if (r.n_mt) atomicAdd(&a.counters[kNumMT], static_cast<unsigned long long>(r.n_mt));
    if (r.n_trip) atomicAdd(&a.counters[kNumTriplets], static_cast<unsigned long long>(r.n_trip));
}

// Persistent kernel over work items (event, bin, chunk of middles).
__global__ void __launch_bounds__(256) k_seed_fast(DevConfig c, Arena a, uint32_t mpi,
                                                    uint32_t nb_cap) {
    extern __shared__ __align__(16) uint8_t smem[];
    float4* nb_xyzr = reinterpret_cast<float4*>(smem);
    uint32_t* seg_pos = reinterpret_cast<uint32_t*>(nb_xyzr + nb_cap);  // [kMaxSegments+1]
    uint32_t* seg_g = seg_pos + kMaxSegments + 1;                        // [kMaxSegments]
    uint32_t* misc = seg_g + kMaxSegments;                               // [16]
    FastScratch* wsb = reinterpret_cast<FastScratch*>(
        reinterpret_cast<uint8_t*>(misc) + 16 * sizeof(uint32_t));
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nwarps = blockDim.x >> 5;
    FastScratch& ws = wsb[warp];
    const bool any_var = a.counters[kAnyVariance] != 0;
    const uint32_t total_items =
        static_cast<uint32_t>(min(a.counters[kItemTotal], static_cast<unsigned long long>(a.max_items)));

    for (;;) {
        if (threadIdx.x == 0) {
            misc[0] = static_cast<uint32_t>(atomicAdd(&a.counters[kItemFetch], 1ull));
            misc[3] = 0x7f800000u;  // min r (as bits, r >= 0)
            misc[4] = 0u;           // max r
        }
        __syncthreads();
        const uint32_t item = misc[0];
        if (item >= total_items) break;
        const uint2 it = a.items[item];
        const uint32_t e = it.x, bin = it.y & 0xffffu, ch = it.y >> 16;
        const uint32_t* bs = a.bin_start + static_cast<size_t>(e) * (c.nbins + 1);
        const uint32_t pbin = bin % c.phi_bins, zbin = bin / c.phi_bins;
        uint32_t zlo, zhi;
        {
            const int imin = static_cast<int>(zbin) - static_cast<int>(c.scope0);
            const int imax = static_cast<int>(zbin) + static_cast<int>(c.scope1);
            zlo = imin >= 0 ? static_cast<uint32_t>(imin) : 0u;
            zhi = imax < static_cast<int>(c.z_bins) ? static_cast<uint32_t>(imax) : c.z_bins - 1u;
        }
        if (threadIdx.x == 0) {
            uint32_t ns;
            misc[2] = build_segments(c, bs, pbin, zlo, zhi, seg_pos, seg_g, &ns);
            misc[1] = ns;
        }
        __syncthreads();
        const uint32_t nseg = misc[1], size = misc[2];
        const bool staged = size <= nb_cap && size <= 65535u;
        if (staged) {
            float lmin = __int_as_float(0x7f800000), lmax = 0.f;
            for (uint32_t s = 0; s < nseg; ++s) {
                const uint32_t p0 = seg_pos[s], len = seg_pos[s + 1] - p0, g0 = seg_g[s];
                for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) {
                    const float4 v = a.g_xyzr[g0 + k];
                    nb_xyzr[p0 + k] = v;
                    lmin = fminf(lmin, v.w);
                    lmax = fmaxf(lmax, v.w);
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
                lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            }
            if (lane == 0) {
                atomicMin(&misc[3], __float_as_uint(lmin));
                atomicMax(&misc[4], __float_as_uint(lmax));
            }
        }
        __syncthreads();
        const float nb_minr = __uint_as_float(misc[3]), nb_maxr = __uint_as_float(misc[4]);
        NbView nb{staged ? nb_xyzr : nullptr, a.g_xyzr, seg_pos, seg_g, nseg, size};
        const uint32_t m0 = bs[bin] + ch * mpi;
        const uint32_t m1 = min(m0 + mpi, bs[bin + 1]);
        for (uint32_t gm = m0 + warp; gm < m1; gm += nwarps) {
            bool standard = staged;
            if (standard && c.z_bins > 1) {
                uint32_t l2, h2;
                z_range(c, a.g_xyzr[gm].z, l2, h2);
                standard = (l2 == zlo && h2 == zhi);
            }
            if (!standard) {
                if (lane == 0) push_overflow(a, gm);
                continue;
            }
            const MiddleResult r = process_middle<1024, 512, 256, kFastTcap>(
                c, a, nb, gm, any_var, true, nb_minr, nb_maxr, ws);
            if (lane == 0) {
                if (r.status) push_overflow(a, gm);
                else count_middle(a, r);
            }
        }
        __syncthreads();
    }
}

// Large-capacity path: one warp per CTA, neighbourhood read from global
// memory, per-middle z neighbourhood.
__global__ void __launch_bounds__(32) k_seed_slow(DevConfig c, Arena a) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t* seg_pos = reinterpret_cast<uint32_t*>(smem);     // [kMaxSegments+1]
    uint32_t* seg_g = seg_pos + kMaxSegments + 1;              // [kMaxSegments]
    SlowScratch& ws = *reinterpret_cast<SlowScratch*>(smem + 1024);
    const uint32_t lane = threadIdx.x & 31;
    const bool any_var = a.counters[kAnyVariance] != 0;
    const uint32_t n = static_cast<uint32_t>(
        min(a.counters[kOvfCount], static_cast<unsigned long long>(a.total_sp)));
    for (;;) {
        uint32_t idx = 0;
        if (lane == 0) idx = static_cast<uint32_t>(atomicAdd(&a.counters[kOvfFetch], 1ull));
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= n) break;
        const uint32_t gm = a.ovf[idx];
        // event: last with sp_base <= gm
        uint32_t lo = 0, hi = a.n_events;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (a.events[mid].sp_base <= gm) lo = mid; else hi = mid;
        }
        const uint32_t e = lo;
        const uint32_t* bs = a.bin_start + static_cast<size_t>(e) * (c.nbins + 1);
        uint32_t b0 = 0, b1 = c.nbins;  // last bin with bs[b] <= gm
        while (b1 - b0 > 1) {
            const uint32_t mid = (b0 + b1) >> 1;
            if (bs[mid] <= gm) b0 = mid; else b1 = mid;
        }
        const uint32_t bin = b0;
        uint32_t zlo, zhi;
        z_range(c, a.g_xyzr[gm].z, zlo, zhi);
        if (lane == 0) {
            uint32_t ns;
            seg_g[kMaxSegments - 1] = 0;
            const uint32_t size = build_segments(c, bs, bin % c.phi_bins, zlo, zhi,
                                                 seg_pos, seg_g, &ns);
            seg_pos[kMaxSegments] = size;
            ws.qb[0] = 0;
            reinterpret_cast<uint32_t*>(smem)[2 * kMaxSegments + 1] = ns;
        }
        __syncwarp();
        const uint32_t nseg = reinterpret_cast<uint32_t*>(smem)[2 * kMaxSegments + 1];
        const uint32_t size = seg_pos[nseg];
        MiddleResult r{0, 0, 0, 1};
        if (size <= 65535u) {
            NbView nb{nullptr, a.g_xyzr, seg_pos, seg_g, nseg, size};
            r = process_middle<8192, 8192, 4096, kSlowTcap>(c, a, nb, gm, any_var, false,
                                                            0.f, 0.f, ws);
        }
        if (lane == 0) {
            if (r.status) {
                raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
                a.seed_cnt[gm] = 0;
            } else {
                count_middle(a, r);
            }
        }
        __syncwarp();
    }
}

// Seeds of one event in host order (bin, middle, rank) into its buffer.
__global__ void __launch_bounds__(1024) k_seed_compact(Arena a) {
    __shared__ uint32_t tmp[33];
    const uint32_t e = blockIdx.x;
    if (e >= a.n_events) return;
    const EventDesc ev = a.events[e];
    const uint32_t nv = a.n_valid[e];
    const uint32_t t = threadIdx.x, nt = blockDim.x;
    const uint32_t per = (nv + nt - 1) / nt;
    const uint32_t i0 = ev.sp_base + min(nv, t * per), i1 = ev.sp_base + min(nv, (t + 1) * per);
    uint32_t s = 0;
    for (uint32_t i = i0; i < i1; ++i) s += a.seed_cnt[i];
    const uint32_t lane = t & 31, warp = t >> 5;
    uint32_t incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += v;
    }
    if (lane == 31) tmp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t nw = nt / 32;
        const uint32_t w = lane < nw ? tmp[lane] : 0u;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= static_cast<uint32_t>(o)) wi += v;
        }
        if (lane < nw) tmp[lane] = wi - w;
        if (lane == 31) tmp[32] = wi;
    }
    __syncthreads();
    uint32_t o = tmp[warp] + incl - s;
    const uint32_t total = tmp[32];
    for (uint32_t i = i0; i < i1; ++i) {
        const uint32_t cnt = a.seed_cnt[i];
        for (uint32_t k = 0; k < cnt; ++k, ++o) {
            if (o < ev.out_cap) {
                const SeedSlot sl = a.seed_slot[static_cast<size_t>(i) * kMaxSeedsPerMiddle + k];
                ev.out_b[o] = sl.b;
                ev.out_m[o] = sl.m;
                ev.out_t[o] = sl.t;
                ev.out_q[o] = sl.q;
            }
        }
    }
    if (t == 0) {
        *ev.out_size = min(total, ev.out_cap);
        atomicAdd(&a.counters[kNumSeeds], static_cast<unsigned long long>(total));
        if (total > ev.out_cap) raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
    }
}

// ---------------------------------------------------------------------------
// Track parameter estimation
// ---------------------------------------------------------------------------

__device__ __forceinline__ float perp2(float a, float b) { return sqrtf(a * a + b * b); }

// seed_to_bound_param_vector (core/include/traccc/seeding/
// track_params_estimation_helper.hpp:48-129) and the covariance of
// core/src/seeding/track_params_estimation.cpp:59-86.  Frame algebra with
// point_to_local(p) = R^T (p - t), rotate(v) = R v, R = [x y z] columns.
__global__ void __launch_bounds__(128)
k_params(ParamsConfig c, float bx, float by, float bz, seedgb_measurement_view meas,
         seedgb_spacepoint_view sps, seedgb_seed_buffer seeds, seedgb_params_buffer out) {
    const uint32_t n = min(*seeds.size, seeds.capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (i >= out.capacity) break;
        const uint32_t ib = seeds.bottom_index[i], im = seeds.middle_index[i],
                       it = seeds.top_index[i];
        if (ib >= sps.size || im >= sps.size || it >= sps.size) continue;
        const float gB[3] = {sps.global[3 * ib], sps.global[3 * ib + 1], sps.global[3 * ib + 2]};
        const float gM[3] = {sps.global[3 * im], sps.global[3 * im + 1], sps.global[3 * im + 2]};
        const float gT[3] = {sps.global[3 * it], sps.global[3 * it + 1], sps.global[3 * it + 2]};
        const float relVec[3] = {gM[0] - gB[0], gM[1] - gB[1], gM[2] - gB[2]};
        const float bn = sqrtf(bx * bx + by * by + bz * bz);
        const float newZ[3] = {bx / bn, by / bn, bz / bn};
        const float cz[3] = {newZ[1] * relVec[2] - relVec[1] * newZ[2],
                             newZ[2] * relVec[0] - relVec[2] * newZ[0],
                             newZ[0] * relVec[1] - relVec[0] * newZ[1]};
        const float cn = sqrtf(cz[0] * cz[0] + cz[1] * cz[1] + cz[2] * cz[2]);
        const float newY[3] = {cz[0] / cn, cz[1] / cn, cz[2] / cn};
        const float newX[3] = {newY[1] * newZ[2] - newZ[1] * newY[2],
                               newY[2] * newZ[0] - newZ[2] * newY[0],
                               newY[0] * newZ[1] - newZ[0] * newY[1]};
        const float d1[3] = {gM[0] - gB[0], gM[1] - gB[1], gM[2] - gB[2]};
        const float d2[3] = {gT[0] - gB[0], gT[1] - gB[1], gT[2] - gB[2]};
        const float l1[3] = {newX[0] * d1[0] + newX[1] * d1[1] + newX[2] * d1[2],
                             newY[0] * d1[0] + newY[1] * d1[1] + newY[2] * d1[2],
                             newZ[0] * d1[0] + newZ[1] * d1[1] + newZ[2] * d1[2]};
        const float l2[3] = {newX[0] * d2[0] + newX[1] * d2[1] + newX[2] * d2[2],
                             newY[0] * d2[0] + newY[1] * d2[1] + newY[2] * d2[2],
                             newZ[0] * d2[0] + newZ[1] * d2[1] + newZ[2] * d2[2]};
        // uv_transform, track_params_estimation_helper.hpp:29-36
        const float den1 = l1[0] * l1[0] + l1[1] * l1[1];
        const float u1 = l1[0] / den1, v1 = l1[1] / den1;
        const float den2 = l2[0] * l2[0] + l2[1] * l2[1];
        const float u2 = l2[0] / den2, v2 = l2[1] / den2;
        const float A = (v2 - v1) / (u2 - u1);
        const float B = v2 - A * u2;
        const float R = -perp2(1.f, A) / (2.f * B);
        const float invTanTheta =
            l2[2] / (2.f * R * asinf(perp2(l2[0], l2[1]) / (2.f * R)));
        const float td[3] = {1.f, A, perp2(1.f, A) * invTanTheta};
        const float tn = sqrtf(td[0] * td[0] + td[1] * td[1] + td[2] * td[2]);
        const float tdn[3] = {td[0] / tn, td[1] / tn, td[2] / tn};
        const float dir[3] = {newX[0] * tdn[0] + newY[0] * tdn[1] + newZ[0] * tdn[2],
                              newX[1] * tdn[0] + newY[1] * tdn[1] + newZ[1] * tdn[2],
                              newX[2] * tdn[0] + newY[2] * tdn[1] + newZ[2] * tdn[2]};
        seedgb_bound_track_parameters p;
        const float phi = atan2f(dir[1], dir[0]);
        const float theta = atan2f(perp2(dir[0], dir[1]), dir[2]);
        const uint32_t mi = sps.measurement_index_1[ib];
        const bool mok = mi < meas.size;
        p.surface_link = mok ? meas.surface_link[mi] : ~0ull;
        p.params[0] = mok ? meas.local_position[2 * mi] : 0.f;
        p.params[1] = mok ? meas.local_position[2 * mi + 1] : 0.f;
        p.params[2] = phi;
        p.params[3] = theta;
        const float qOverPt = 1.f / (R * bn);
        p.params[4] = qOverPt / perp2(1.f, invTanTheta);
        p.params[5] = 0.f;
#pragma unroll
        for (int k = 0; k < 36; ++k) p.cov[k] = 0.f;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            float var = c.initial_sigma[j] * c.initial_sigma[j];
            if (j == 4) {
                const float var_theta = p.cov[3 * 6 + 3];
                var += powf(c.initial_sigma_qopt * sinf(p.params[3]), 2.f);
                var += powf(c.initial_sigma_pt_rel * p.params[4], 2.f);
                var += var_theta * powf(p.params[4] / tanf(p.params[3]), 2.f);
            }
            var *= c.initial_inflation[j];
            p.cov[j * 6 + j] = var;
        }
        out.data[i] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *out.size = min(n, out.capacity);
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

size_t fast_kernel_smem(const TuneParams& tp) {
    return static_cast<size_t>(tp.nb_cap) * sizeof(float4) +
           (2 * kMaxSegments + 1 + 16) * sizeof(uint32_t) +
           static_cast<size_t>(tp.fast_warps) * sizeof(FastScratch) + 16;
}

static size_t slow_kernel_smem() { return 1024 + sizeof(SlowScratch); }

cudaError_t launch_seeding(const DevConfig& cfg, const Arena& a, const TuneParams& tp,
                           int num_sms, cudaStream_t stream) {
    static bool attrs_set = false;
    const size_t fsm = fast_kernel_smem(tp);
    const size_t ssm = slow_kernel_smem();
    if (!attrs_set) {
        cudaError_t err = cudaFuncSetAttribute(
            k_seed_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (err != cudaSuccess) return err;
        err = cudaFuncSetAttribute(k_seed_slow, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(ssm));
        if (err != cudaSuccess) return err;
        attrs_set = true;
    }
    const size_t hsm = static_cast<size_t>(kBinWarps) * cfg.nbins * sizeof(uint32_t);
    if (a.total_chunks > 0) {
        k_bin_count<<<a.total_chunks, kBinWarps * 32, hsm, stream>>>(cfg, a);
    }
    {
        const uint32_t nb = cfg.nbins;
        const uint32_t G = std::max(1u, 1024u / nb);
        const size_t ssz = (static_cast<size_t>(G) * nb + 2 * nb + 40) * sizeof(uint32_t);
        k_bin_scan<<<a.n_events, 1024, ssz, stream>>>(cfg, a,
                                                      static_cast<uint32_t>(tp.middles_per_item));
    }
    if (a.total_chunks > 0) {
        k_bin_scatter<<<a.total_chunks, kBinWarps * 32, hsm, stream>>>(cfg, a);
    }
    k_seed_fast<<<num_sms * tp.ctas_per_sm, tp.fast_warps * 32, fsm, stream>>>(
        cfg, a, static_cast<uint32_t>(tp.middles_per_item), static_cast<uint32_t>(tp.nb_cap));
    k_seed_slow<<<num_sms, 32, ssm, stream>>>(cfg, a);
    k_seed_compact<<<a.n_events, 1024, 0, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_params(const ParamsConfig& cfg, const float bfield[3],
                          const seedgb_measurement_view& meas,
                          const seedgb_spacepoint_view& sps,
                          const seedgb_seed_buffer& seeds, const seedgb_params_buffer& out,
                          int num_sms, cudaStream_t stream) {
    k_params<<<num_sms * 4, 128, 0, stream>>>(cfg, bfield[0], bfield[1], bfield[2], meas, sps,
                                               seeds, out);
    return cudaGetLastError();
}

}  // namespace seedgb
