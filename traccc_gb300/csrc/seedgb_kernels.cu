// GB300 (sm_103a) kernels of the triplet seeding path.
//
// Pipeline for a batch of events (one launch each, all asynchronous):
//   k_bin_count    validity + (phi, z) bin per spacepoint, per-warp histograms
//   k_bin_scan     per event: stable offsets, bin ranges, work items
//   k_item_order   work items in longest-processing-time order
//   k_bin_scatter  stable counting-sort scatter into the binned SoA grid
//   k_seed_fast    per work item (event, bin, chunk of middles): stage the
//                  bin's neighbourhood in shared memory; one warp per middle
//                  runs doublet finding (ballot compaction), triplet finding
//                  (cot-sorted middle-top doublets, exact reference cuts),
//                  compatible-seed weights and seed selection
//   k_seed_mid     the same per-middle routine on the middles the fast kernel
//                  hands over (neighbourhood too large to stage, per-middle z
//                  neighbourhood, lists beyond its buffers), reading the
//                  neighbourhood from global memory, many warps per SM
//   k_seed_slow    the same with large capacities, one warp per SM, for the
//                  few middles whose lists overflow k_seed_mid's buffers
//   k_seed_count   seeds per chunk of middles
//   k_seed_compact per chunk of middles: seeds in host order into the output
//                  buffers
//
// Floating-point semantics follow the reference host code: the file is built
// with -fmad=false --prec-div=true --prec-sqrt=true --ftz=false, and every
// cut is evaluated in the reference's operation order, so decisions are
// bit-identical to the reference's host seeding.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "seedgb_device.cuh"
#include "seedgb_internal.h"
#include "seedgb_mlp.cuh"

namespace seedgb {
namespace {

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
                                   uint32_t* nseg_out, uint32_t* seg_bin) {
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
            if (seg_bin) seg_bin[ns] = bin;
            pos += bs[bin + 1] - bs[bin];
            ++ns;
        }
    }
    seg_pos[ns] = pos;
    *nseg_out = ns;
    return pos;
}

__device__ __forceinline__ uint32_t event_of_chunk(const Arena& a, uint32_t n_events,
                                                   uint32_t chunk) {
    uint32_t lo = 0, hi = n_events;  // last event with chunk_base <= chunk
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
    const BatchHeader hb = *a.hdr;
    if (chunk >= hb.total_chunks) return;
    const uint32_t e = event_of_chunk(a, hb.n_events, chunk);
    const EventDesc ev = a.events[e];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t i = threadIdx.x; i < kBinWarps * c.nbins; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    uint32_t* h = hist + warp * c.nbins;
    const uint32_t base = (chunk - ev.chunk_base) * kBinChunk + warp * (kBinRounds * 32);
    // all rounds' loads first: one memory latency per warp instead of one
    // per round (the kernel waits on its loads)
    float px[kBinRounds], py[kBinRounds], pz[kBinRounds];
    bool anyvar = false;
#pragma unroll
    for (int r = 0; r < kBinRounds; ++r) {
        const uint32_t i = base + r * 32 + lane;
        px[r] = py[r] = pz[r] = 0.f;
        if (i < ev.n_sp) {
            px[r] = ev.global[3 * i];
            py[r] = ev.global[3 * i + 1];
            pz[r] = ev.global[3 * i + 2];
            anyvar |= (ev.zvar && ev.zvar[i] != 0.f) || (ev.rvar && ev.rvar[i] != 0.f);
        }
    }
#pragma unroll
    for (int r = 0; r < kBinRounds; ++r) {
        const uint32_t i = base + r * 32 + lane;
        if (i < ev.n_sp) {
            const int32_t bin = classify(c, px[r], py[r], pz[r], a.counters);
            a.sp_bin[ev.sp_base + i] = bin;
            if (bin >= 0) atomicAdd(&h[bin], 1u);
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
// Log-scale bucket of a work item's estimated cost (8 buckets per power of
// two, largest last).
__device__ __forceinline__ uint32_t cost_bucket(unsigned long long cost) {
    if (cost == 0) return 0;
    const uint32_t e = 63u - static_cast<uint32_t>(__clzll(cost));  // floor(log2)
    const uint32_t f = static_cast<uint32_t>(e >= 3 ? (cost >> (e - 3)) : (cost << (3 - e))) & 7u;
    return min(8u * e + f, kOrderBuckets - 1u);
}

__global__ void __launch_bounds__(1024) k_bin_scan(DevConfig c, Arena a, uint32_t mpi) {
    extern __shared__ uint32_t sh[];
    const uint32_t e = blockIdx.x;
    if (e >= a.hdr->n_events) return;
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
    // work items: (event, bin | chunk << 16), with the bucket of their cost
    // (middles x spacepoints of the bin's neighbourhood) for k_item_order
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        const uint32_t i0 = items[b];
        const uint32_t i1 = (b + 1 < nb) ? items[b + 1] : n_items;
        const uint32_t size = ((b + 1 < nb) ? tot[b + 1] : n_valid) - tot[b];
        uint32_t nbsize = 0;
        {
            uint32_t phis[kMaxSegments];
            const uint32_t np = phi_zone(c, b % c.phi_bins, phis, kMaxSegments);
            const uint32_t zb = b / c.phi_bins;
            const uint32_t zlo = zb >= c.scope0 ? zb - c.scope0 : 0u;
            const uint32_t zhi = min(zb + c.scope1, c.z_bins - 1u);
            for (uint32_t ip = 0; ip < np; ++ip)
                for (uint32_t z = zlo; z <= zhi; ++z) {
                    const uint32_t nbin = phis[ip] + z * c.phi_bins;
                    nbsize += ((nbin + 1 < nb) ? tot[nbin + 1] : n_valid) - tot[nbin];
                }
        }
        for (uint32_t k = i0; k < i1 && item_base + k < a.max_items; ++k) {
            a.items[item_base + k] = make_uint2(e, b | ((k - i0) << 16));
            const uint32_t m = min(mpi, size - (k - i0) * mpi);
            const uint32_t q = cost_bucket(static_cast<unsigned long long>(m) * nbsize);
            a.item_key[item_base + k] = static_cast<uint8_t>(q);
            atomicAdd(&a.order_hist[q], 1u);
        }
    }
    if (threadIdx.x == 0 && item_base + n_items > a.max_items)
        raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
}

// Work items in longest-processing-time order: the persistent seeding
// kernel then ends on its cheapest items instead of whichever items the last
// event appended, which leaves fewer SMs idle at its end.  A counting sort
// over the cost buckets k_bin_scan recorded; the order inside a bucket is
// arbitrary.  Results do not depend on the order of the items.
__global__ void __launch_bounds__(1024) k_item_order(Arena a) {
    __shared__ uint32_t start[kOrderBuckets];
    const uint32_t n = static_cast<uint32_t>(
        min(a.counters[kItemTotal], static_cast<unsigned long long>(a.max_items)));
    if (blockIdx.x * blockDim.x >= n) return;
    if (threadIdx.x < 32) {
        // exclusive prefix over the buckets, most costly first
        constexpr uint32_t kPer = kOrderBuckets / 32;
        const uint32_t lane = threadIdx.x;
        uint32_t v[kPer], sum = 0;
#pragma unroll
        for (uint32_t j = 0; j < kPer; ++j) {
            v[j] = a.order_hist[kOrderBuckets - 1 - (kPer * lane + j)];
            sum += v[j];
        }
        uint32_t incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += t;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (uint32_t j = 0; j < kPer; ++j) {
            start[kOrderBuckets - 1 - (kPer * lane + j)] = run;
            run += v[j];
        }
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t q = a.item_key[i];
        const uint32_t k = start[q] + atomicAdd(&a.order_hist[kOrderBuckets + q], 1u);
        if (k < n) a.items_ord[k] = a.items[i];
    }
}

__global__ void __launch_bounds__(kBinWarps * 32) k_bin_scatter(DevConfig c, Arena a) {
    extern __shared__ uint32_t base[];  // [kBinWarps][nbins]
    const uint32_t chunk = blockIdx.x;
    const BatchHeader hb = *a.hdr;
    if (chunk >= hb.total_chunks) return;
    const uint32_t e = event_of_chunk(a, hb.n_events, chunk);
    const EventDesc ev = a.events[e];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t* src = a.whist + static_cast<size_t>(chunk) * kBinWarps * c.nbins;
    for (uint32_t i = threadIdx.x; i < kBinWarps * c.nbins; i += blockDim.x) base[i] = src[i];
    __syncthreads();
    uint32_t* wb = base + warp * c.nbins;
    const uint32_t b0 = (chunk - ev.chunk_base) * kBinChunk + warp * (kBinRounds * 32);
    const uint32_t lt = lanemask_lt();
    // all rounds' bins and coordinates first: one memory latency per warp
    // instead of two per round (the kernel waits on its loads)
    int32_t pbin[kBinRounds];
    float px[kBinRounds], py[kBinRounds], pz[kBinRounds];
#pragma unroll
    for (int r = 0; r < kBinRounds; ++r) {
        const uint32_t i = b0 + r * 32 + lane;
        pbin[r] = -1;
        px[r] = py[r] = pz[r] = 0.f;
        if (i < ev.n_sp) {
            pbin[r] = a.sp_bin[ev.sp_base + i];
            px[r] = ev.global[3 * i];
            py[r] = ev.global[3 * i + 1];
            pz[r] = ev.global[3 * i + 2];
        }
    }
#pragma unroll
    for (int r = 0; r < kBinRounds; ++r) {
        const uint32_t i = b0 + r * 32 + lane;
        const int32_t bin = pbin[r];
        const uint32_t peers = __match_any_sync(0xffffffffu, bin);
        const uint32_t rank = __popc(peers & lt);
        if (bin >= 0) {
            const uint32_t pos = wb[bin] + rank;
            const float x = px[r], y = py[r], z = pz[r];
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
    float s;  // y * iDeltaR: sine of the doublet's angle to the radial direction
};

// First part of doublet_finding_helper::isCompatible<bottom>
// (doublet_finding_helper.hpp:59-82): r, z windows and the z-origin window.
__device__ __forceinline__ bool window_bottom(const DevConfig& c, const float4 m,
                                              const float4 o) {
    const float deltaR = m.w - o.w;
    const float cotTheta = m.z - o.z;
    const float zOrigin = m.z * deltaR - m.w * cotTheta;
    // the reference's short-circuit || over side-effect-free comparisons,
    // evaluated without branches
    return !((deltaR >= c.deltaRMax) | (deltaR <= c.deltaRMin) |
             (fabsf(cotTheta) >= c.cotThetaMax * deltaR) |
             (zOrigin <= c.collisionRegionMin * deltaR) |
             (zOrigin >= c.collisionRegionMax * deltaR) |
             (fabsf(cotTheta) >= c.deltaZMax));
}

// Same for isCompatible<top> (doublet_finding_helper.hpp:67-74).
__device__ __forceinline__ bool window_top(const DevConfig& c, const float4 m,
                                           const float4 o) {
    const float deltaR = o.w - m.w;
    const float cotTheta = (o.z - m.z);
    const float zOrigin = m.z * deltaR - m.w * cotTheta;
    // the reference's short-circuit || over side-effect-free comparisons,
    // evaluated without branches
    return !((deltaR >= c.deltaRMax) | (deltaR <= c.deltaRMin) |
             (fabsf(cotTheta) >= c.cotThetaMax * deltaR) |
             (zOrigin <= c.collisionRegionMin * deltaR) |
             (zOrigin >= c.collisionRegionMax * deltaR) |
             (fabsf(cotTheta) >= c.deltaZMax));
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

// Fast evaluation of the same test.  The two circle centres are
// mid +- sagitta * n with n = (|dy|, -sign(dy) dx) / |d| (the reference's
// (cosCentralAngle, sinCentralAngle) written without the slope), so the
// squared distances are evaluated with approximate reciprocal square roots.
// Returns 1 (passes) or 0 (rejected) when the smaller squared distance is more
// than 2e-4 relative away from the cut -- more than ten times the combined
// rounding error of either evaluation (about 15 operations of 2^-22 relative
// error each, amplified at most 2 (|mid| + R)^2 / (R - impactMax)^2 < 8 while
// the chord midpoint lies inside the helix circle) -- and -1 when only the
// exact evaluation can decide: near the cut, for a chord midpoint outside the
// helix radius, and for degenerate chords (dx or dy zero or negligible,
// sagitta undefined), where the reference's own arithmetic produces inf/NaN.
__device__ __forceinline__ int helix_fast(const DevConfig& c, const float4 m,
                                          const float4 o) {
    const float dX = o.x - m.x, dY = o.y - m.y;
    const float aX = fabsf(dX), aY = fabsf(dY);
    const float d2 = dX * dX + dY * dY;
    const float R2 = c.minHelixRadius * c.minHelixRadius;
    const float s2 = R2 - 0.25f * d2;
    if (!(aX > 1e-6f * aY) || !(aY > 1e-6f * aX) || !(s2 > 1e-3f * R2) ||
        !(d2 > 1e-20f) || !(d2 < 1e30f))
        return -1;
    const float inv = rsqrtf(d2);
    const float sag = s2 * rsqrtf(s2);
    const float nX = aY * inv;
    const float nY = (dY > 0.f ? -dX : dX) * inv;
    const float midX = 0.5f * (m.x + o.x), midY = 0.5f * (m.y + o.y);
    if (!(midX * midX + midY * midY < R2)) return -1;
    const float p1X = midX + sag * nX, p1Y = midY + sag * nY;
    const float p2X = midX - sag * nX, p2Y = midY - sag * nY;
    const float mn = fminf(p1X * p1X + p1Y * p1Y, p2X * p2X + p2Y * p2Y);
    const float lim = (c.minHelixRadius - c.impactMax) * (c.minHelixRadius - c.impactMax);
    if (mn > lim * 1.0002f) return 1;
    if (mn < lim * 0.9998f) return 0;
    return -1;
}

// doublet_finding_helper::transform_coordinates, doublet_finding_helper.hpp:
// 218-272, with the middle's cos/sin(phi) (x/r, y/r) computed once per middle
// spacepoint.  vm/vo = (z_variance, radius_variance).
__device__ __forceinline__ LinCircle lin_circle_cs(bool top, const float4 m,
                                                   const float cosPhiM, const float sinPhiM,
                                                   const float2 vm, const float4 o,
                                                   const float2 vo) {
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
    l.s = y * iDeltaR;
    return l;
}

// triplet_finding_helper::isCompatible (triplet_finding_helper.hpp:42-133),
// split in two exact stages, so that the candidates the
// minimum-helix-diameter cut rejects (most of them) are dropped before the
// costly remainder.  Stage 1 runs triplet_finding_helper.hpp:42-90 and returns
// A and B; stage 2 runs the rest (:92-130) from A and B.  Together they make
// the same decisions and produce the same curvature and impact parameter.
__device__ __forceinline__ float triplet_error2(const float2 vm, const LinCircle& lb,
                                                const float ltCot, const float ltIdr,
                                                const float ltEr) {
    return ltEr + lb.er + 2.f * (lb.cot * ltCot * vm.y + vm.x) * lb.idr * ltIdr;
}

__device__ __forceinline__ bool triplet_stage1(const DevConfig& c, const float2 vm,
                                               const LinCircle& lb, const float ltCot,
                                               const float ltIdr, const float ltEr,
                                               const float ltU, const float ltV,
                                               const float scatteringInRegion2,
                                               float& A_out, float& B_out) {
    const float error2 = triplet_error2(vm, lb, ltCot, ltIdr, ltEr);
    const float deltaCotTheta = lb.cot - ltCot;
    const float deltaCotTheta2 = deltaCotTheta * deltaCotTheta;
    if (deltaCotTheta2 - error2 > 0) {
        const float adct = fabsf(deltaCotTheta);
        // sqrtf(+-0) = +-0: skip the square root of a zero error term
        const float error = (error2 == 0.f) ? error2 : sqrtf(error2);
        const float d = deltaCotTheta2 + error2 - 2.f * adct * error;
        if (d > scatteringInRegion2) return false;
    }
    const float dU = ltU - lb.u;
    if (dU == 0.f) return false;
    const float A = (ltV - lb.v) / dU;
    const float S2 = 1.f + A * A;
    const float B = lb.v - A * lb.u;
    const float B2 = B * B;
    if (S2 < B2 * c.minHelixDiameter2) return false;
    A_out = A;
    B_out = B;
    return true;
}

__device__ __forceinline__ bool triplet_stage2(const DevConfig& c, const float rM,
                                               const float2 vm, const LinCircle& lb,
                                               const float ltCot, const float ltIdr,
                                               const float ltEr, const float iSinTheta2,
                                               const float A, const float B,
                                               float& curvature, float& impact) {
    const float S2 = 1.f + A * A;
    const float B2 = B * B;
    const float iHelixDiameter2 = B2 / S2;
    float pT2scatter = 4.f * iHelixDiameter2 * c.pT2perRadius;
    const float pT = c.pTPerHelixRadius * sqrtf(S2 / B2) / 2.f;
    if (pT > c.maxPtScattering) {
        const float pTscatter = c.highland / c.maxPtScattering;
        pT2scatter = pTscatter * pTscatter;
    }
    const float p2scatter = pT2scatter * iSinTheta2;
    const float error2 = triplet_error2(vm, lb, ltCot, ltIdr, ltEr);
    const float deltaCotTheta = lb.cot - ltCot;
    const float deltaCotTheta2 = deltaCotTheta * deltaCotTheta;
    if (deltaCotTheta2 - error2 > 0.f) {
        const float adct = fabsf(deltaCotTheta);
        const float error = (error2 == 0.f) ? error2 : sqrtf(error2);
        const float d = deltaCotTheta2 + error2 - 2.f * adct * error;
        if (d > p2scatter * c.sigmaScattering * c.sigmaScattering) return false;
    }
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

// An unsigned key in the order of the float values, +0 and -0 equal (as they
// compare in better); the values are never NaN (finite coordinates give
// finite weights and tie sums).
__device__ __forceinline__ uint32_t order_key(float x) {
    const uint32_t u = __float_as_uint(x + 0.0f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// The best untaken triplet (weight not -inf) among k = lane, lane + 32, ...
// in the order of better; ck = 0xffffffff when there is none.
__device__ __forceinline__ void lane_best(const float* wf, const float* ts, uint32_t n,
                                          uint32_t lane, float& cw, float& cs, uint32_t& ck) {
    ck = 0xffffffffu;
    for (uint32_t k = lane; k < n; k += 32) {
        const float wk = wf[k];
        if (wk == -__int_as_float(0x7f800000)) continue;
        if (ck == 0xffffffffu || better(wk, ts[k], k, cw, cs, ck)) {
            cw = wk;
            cs = ts[k];
            ck = k;
        }
    }
}

// ---------------------------------------------------------------------------
// Radius-sorted copy of every grid bin
// ---------------------------------------------------------------------------

constexpr int kSortCap = 4096;  // largest bin sorted in shared memory

// One CTA per (event, bin): the bin's spacepoints sorted by radius (ties by
// grid position), with the grid position of each.  One 64-bit key per
// spacepoint, radius bits above the grid position: a bitonic network over
// single keys (radii are non-negative, so their bits order as the values).  A bin larger than kSortCap is
// flagged; middles whose neighbourhood holds such a bin take the
// large-capacity path, which scans in host order.
__global__ void __launch_bounds__(256) k_bin_rsort(DevConfig c, Arena a) {
    __shared__ unsigned long long key[kSortCap];
    const uint32_t e = blockIdx.x / c.nbins, b = blockIdx.x % c.nbins;
    if (e >= a.hdr->n_events) return;
    const uint32_t* bs = a.bin_start + static_cast<size_t>(e) * (c.nbins + 1);
    const uint32_t g0 = bs[b], n = bs[b + 1] - g0;
    if (threadIdx.x == 0) a.bin_unsorted[static_cast<size_t>(e) * c.nbins + b] = n > kSortCap;
    if (n == 0 || n > kSortCap) return;
    uint32_t P = 1;
    while (P < n) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x)
        key[i] = i < n ? (static_cast<unsigned long long>(__float_as_uint(a.g_xyzr[g0 + i].w))
                          << 32) | (g0 + i)
                       : ~0ull;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = threadIdx.x; t < P / 2; t += blockDim.x) {
                const uint32_t i = 2 * t - (t & (j - 1));
                const uint32_t l = i + j;
                const bool up = (i & k) == 0;
                const unsigned long long ki = key[i], kl = key[l];
                if (up ? (ki > kl) : (ki < kl)) {
                    key[i] = kl;
                    key[l] = ki;
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t gp = static_cast<uint32_t>(key[i]);
        a.g_rs[g0 + i] = a.g_xyzr[gp];
        a.g_rs_gp[g0 + i] = gp;
    }
}

// ---------------------------------------------------------------------------
// Per-middle seeding routine
// ---------------------------------------------------------------------------

constexpr uint32_t kFastSegs = 16;  // neighbourhood bins on the fast path

// Neighbourhood of a middle spacepoint: the concatenation of its grid bins in
// host order (phi zone outer, z zone inner).  "Host position" = position in
// that concatenation.  Three ways to read it (a template parameter, so that
// the fused kernel carries no per-access branch on it: measured 9 % faster
// than a runtime test):
//   kNbShared    every bin staged as a radius-sorted run in shared memory
//                (staged / staged_hp give the spacepoint and its host
//                position): the fast kernel;
//   kNbGlobalRs  the bins are consecutive in the grid, so their radius-sorted
//                copies (g_rs) form one array in host order of the bins:
//                staged = g_rs from the first bin on, the host position is
//                the grid position (staged_gp) minus the first one (base);
//   kNbHost      the grid itself in host order (any neighbourhood).
// The first two give radius-sorted runs (the exact radial windows).
enum NbMode : int { kNbHost = 0, kNbShared = 1, kNbGlobalRs = 2 };

template <int MODE>
struct NbViewT {
    static constexpr bool kRSorted = MODE != kNbHost;
    const float4* staged;       // radius-sorted runs (kNbShared, kNbGlobalRs)
    const uint16_t* staged_hp;  // kNbShared: host position of each staged spacepoint
    const uint32_t* staged_gp;  // kNbGlobalRs: grid position of each run element
    uint32_t base;              // kNbGlobalRs: grid position of host position 0
    const float4* g_xyzr;
    const uint32_t* seg_pos;    // [nseg + 1] host-position prefix
    const uint32_t* seg_g;      // [nseg] first grid position of each bin
    uint32_t nseg;
    uint32_t size;

    // host position -> grid position
    __device__ __forceinline__ uint32_t gpos(uint32_t hp) const {
        if constexpr (MODE == kNbGlobalRs) {
            return base + hp;
        } else {
            uint32_t s = 0;
            while (s + 1 < nseg && seg_pos[s + 1] <= hp) ++s;
            return seg_g[s] + (hp - seg_pos[s]);
        }
    }
    __device__ __forceinline__ float4 get(uint32_t p) const {
        if constexpr (MODE != kNbHost) return staged[p];
        else return g_xyzr[gpos(p)];
    }
    __device__ __forceinline__ uint32_t hpos(uint32_t p) const {
        if constexpr (MODE == kNbShared) return staged_hp[p];
        else if constexpr (MODE == kNbGlobalRs) return staged_gp[p] - base;
        else return p;
    }
};

constexpr int kBuckets = 160;  // cot(theta) buckets of the middle-top doublets

// A triplet of the middle spacepoint (before the compatible-seed weights).
struct TripCand {
    uint16_t tp;  // middle-top list index
    uint16_t ib;  // middle-bottom list index
    float curv;   // curvature
    float w;      // weight: -impact * impactWeightFactor
};

// A candidate inside its doublet's cot window, with the doublet's lin_circle.
struct Stage0Cand {
    uint16_t tp, ib;  // middle-top / middle-bottom list indices
    float cot, idr, er, u, v;
};

// A triplet candidate that passed stage 1, with what stage 2 needs of its
// middle-bottom doublet.
struct Stage1Cand {
    uint16_t tp, ib;
    float A, B;
    float cot, idr, er, is2;  // lin_circle of the doublet, 1 + cot^2
};

template <int CAPB, int CAPT, int CAPLC, int CAPCT>
struct WarpScratch {
    // the host-order sort pads the triplets to the next power of two
    static_assert((CAPCT & (CAPCT - 1)) == 0, "triplet capacity must be a power of two");
    // the bucket prefix gives kBuckets / 32 buckets to each lane, and the
    // learned filter uses bstart as 160 words of scratch
    static_assert(kBuckets % 32 == 0 && kBuckets + 1 >= 160, "cot buckets");
    static_assert(CAPB <= 65536 && CAPT <= 65536 && CAPLC <= 65536, "16-bit positions");
    union {
        // middle-top doublets in list order: {cot(theta), iDeltaR, U, V}
        float4 mtd[CAPLC];
        struct {  // the doublet scans' radius windows and candidate prefixes (before mtd)
            uint32_t bnd[4 * kFastSegs];        // radius windows per bin
            uint32_t pre[2 * (kFastSegs + 1)];  // candidate prefix per bin
        };
    };
    float er[CAPLC];
    uint16_t hpt[CAPLC];  // host position of the top
    uint16_t ppt[CAPLC];  // neighbourhood position of the top
    uint16_t perm[CAPLC]; // bucket-sorted slot -> list index
    uint32_t bstart[kBuckets + 1];
    uint16_t qb[CAPB];  // middle-bottom doublets (neighbourhood positions)
    union {
        uint16_t qt[CAPT];        // middle-top doublets, until their lin_circles exist
        uint32_t bcur[kBuckets];  // counting-sort cursors, after the lin_circles
        struct {
            Stage0Cand q0[64];  // in-window candidates awaiting stage 1 (< 32 + 32)
            Stage1Cand q1[64];  // stage-1 survivors awaiting stage 2 (< 32 + 32)
        } q;                    // during the triplet search
        struct {                // after the triplet search
            uint32_t skey[CAPCT]; // host-order sort key of the triplets
            uint16_t sidx[CAPCT]; // sorted -> ct index
            float wf[CAPCT];      // final weight in sorted order, -inf when cut
            float ts[CAPCT];      // tie sum of the sort, sorted order
        };
    };
    TripCand ct[CAPCT];   // triplets of the middle
};
// Shared memory per warp: fast 11.9 KiB, middle tier 22.1 KiB, last tier
// 173 KiB.  The fast capacities sit at the measured list sizes so that 16
// warps fit beside a 2048-spacepoint neighbourhood (smaller scratch means more
// warps per SM, which is what hides this kernel's latency): 512 middle-bottom
// and 1024 middle-top candidates (largest lists on a batch of
// 5k-114k-spacepoint events: 497 and 383), 216 middle-top doublets and 128
// triplets (at most 208 and 101 on 100k-spacepoint events; a few per cent of
// the batch's middles exceed them).  A middle beyond a fast capacity goes to
// the general path's middle tier, whose capacities are above every list
// measured; the last tier takes what exceeds those.
using FastScratch = WarpScratch<512, 1024, 216, 128>;
using MidScratch = WarpScratch<1024, 1024, 512, 256>;
using SlowScratch = WarpScratch<8192, 8192, 4096, 2048>;

// Keep the positions whose doublet passes the minimum-helix-radius test, in
// order, in q[0..n).  One doublet per lane per iteration (two measured 1.3 %
// slower over the whole kernel).
// Out of line: one copy serves both roles (instruction-cache pressure of the
// fused kernel; measured faster than two inlined copies).
template <int MODE>
__device__ __noinline__ uint32_t helix_compact(const DevConfig& c, const NbViewT<MODE>& nb,
                                                  const float4 m, uint16_t* q,
                                                  uint32_t n, uint32_t lane,
                                                  uint32_t lt) {
    const bool exact = c.brute_force_triplets != 0;
    uint32_t w = 0;
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i0 = base + lane;
        bool ok0 = false;
        uint16_t p0 = 0;
        if (i0 < n) {
            p0 = q[i0];
            const float4 o0 = nb.get(p0);
            const int f0 = exact ? -1 : helix_fast(c, m, o0);
            ok0 = f0 == 1;
            if (f0 < 0) ok0 = helix_ok(c, m, o0);
        }
        __syncwarp();
        const uint32_t m0 = __ballot_sync(0xffffffffu, ok0);
        if (ok0) q[w + __popc(m0 & lt)] = p0;
        w += __popc(m0);
        __syncwarp();
    }
    return w;
}

struct MiddleResult {
    uint32_t n_mb, n_mt, n_trip;
    int status;  // 0 done, 1 needs the large-capacity path
};

// Append the positions passing the window cuts of one role to q (in order of
// the flattened per-bin ranges).  One candidate per lane per iteration: two
// or four in flight per lane measured 8 % and 25 % slower over the whole
// seeding kernel (code size and registers of the fused routine).
template <bool TOP, int MODE>
__device__ __forceinline__ uint32_t scan_runs(const DevConfig& c, const NbViewT<MODE>& nb,
                                              const float4 M, const uint32_t* bnd,
                                              const uint32_t* pre, uint32_t ns,
                                              uint16_t* q, uint32_t cap, uint32_t lane,
                                              uint32_t lt) {
    const uint32_t total = pre[ns];
    uint32_t nq = 0;
    // a lane's flat indices only rise: its run, the flat index where that
    // run ends and the run's position offset stay in registers and advance
    // at run boundaries only
    uint32_t run = 0u, end = pre[1], off = bnd[TOP ? 2 : 0];  // pre[0] == 0
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t f = base + lane;
        bool ok = false;
        uint32_t p = 0;
        if (f < total) {
            while (f >= end) {
                const uint32_t s = ++run;
                end = pre[s + 1];
                off = bnd[4 * s + (TOP ? 2 : 0)] - pre[s];
            }
            p = off + f;
            const float4 o = nb.staged[p];
            ok = TOP ? window_top(c, M, o) : window_bottom(c, M, o);
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            const uint32_t k = nq + __popc(mask & lt);
            if (k < cap) q[k] = static_cast<uint16_t>(p);
        }
        nq += __popc(mask);
    }
    return nq;
}

__device__ __forceinline__ uint32_t cot_bucket(float x, float cmin, float scale) {
    const int b = static_cast<int>((x - cmin) * scale);
    return static_cast<uint32_t>(b < 0 ? 0 : (b >= kBuckets ? kBuckets - 1 : b));
}

// One scored doublet as the dump records it (48 bytes).
struct DoubletRec {
    uint32_t middle, other, role;  // role: 1 = middle-top, | event << 1
    float feat[kMlpIn];
    float logit;
};
static_assert(sizeof(DoubletRec) == 48, "doublet record layout");

// Scores one chunk of up to 32 doublets (lane i: doublet i, valid when
// `valid`): the features x go to the warp scratch xs as packed bf16 inputs,
// the network runs on the tensor cores (two 16-doublet tiles), and each
// lane gets its doublet's logit back through lg.  Records the doublets when
// a dump buffer is set.  xs: 128 words of warp scratch, lg: 32 floats.
// The learned filter's threshold of a role and band for event `ev`: its
// size class when classes are set, else the filter-wide values.
__device__ __forceinline__ uint32_t filter_class(const DevConfig& c, const Arena& a, uint32_t ev) {
    const uint32_t n_sp = a.events[ev].n_sp;
    uint32_t k = 0;
    while (k + 1 < c.mlp_n_classes && n_sp > c.mlp_class_max[k]) ++k;
    return k;
}
__device__ __forceinline__ float filter_threshold(const DevConfig& c, const Arena& a, uint32_t ev,
                                                  int role) {
    return c.mlp_n_classes ? c.mlp_class_thr[filter_class(c, a, ev)][role] : c.mlp_thr[role];
}

// Records one chunk of scored doublets (cold path, kept out of line).
__device__ __noinline__ void dump_chunk(unsigned long long* count, DoubletRec* dump,
                                        unsigned long long cap, bool valid, uint32_t mid_idx,
                                        uint32_t oth_idx, uint32_t role, const float (&x)[kMlpIn],
                                        float logit) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t vm = __ballot_sync(0xffffffffu, valid);
    unsigned long long b = 0;
    if (lane == 0) b = atomicAdd(count, static_cast<unsigned long long>(__popc(vm)));
    __syncwarp();
    b = __shfl_sync(0xffffffffu, b, 0) + __popc(vm & lanemask_lt());
    if (valid && b < cap) {
        uint4* r = reinterpret_cast<uint4*>(dump + b);
        r[0] = make_uint4(mid_idx, oth_idx, role, __float_as_uint(x[0]));
        r[1] = make_uint4(__float_as_uint(x[1]), __float_as_uint(x[2]), __float_as_uint(x[3]),
                          __float_as_uint(x[4]));
        r[2] = make_uint4(__float_as_uint(x[5]), __float_as_uint(x[6]), __float_as_uint(x[7]),
                          __float_as_uint(logit));
    }
    __syncwarp();
}

template <bool TOP>
__device__ __forceinline__ float score_chunk(const DevConfig& c, const Arena& a,
                                             const MlpRegs& R, const float (&x)[kMlpIn],
                                             bool valid, uint32_t* xs, float* lg,
                                             uint32_t ev, uint32_t mid_idx, uint32_t oth_idx,
                                             uint32_t lane, uint32_t lt) {
    uint32_t pk[4] = {0u, 0u, 0u, 0u};
    if (valid) mlp_pack_inputs(c.mlp_mu, c.mlp_isd, x, pk);
    *reinterpret_cast<uint4*>(xs + 4 * lane) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    __syncwarp();
    // one copy of the tile code for both 16-doublet tiles (instruction cache)
#pragma unroll 1
    for (uint32_t tt = 0; tt < 2; ++tt) {
        float lo, hi;
        mlp_tile16_regs(R, xs + 64 * tt, lane, lo, hi);
        if ((lane & 3) == 0) {
            const uint32_t g = lane >> 2;
            lg[16 * tt + g] = lo;
            lg[16 * tt + g + 8] = hi;
        }
    }
    __syncwarp();
    const float logit = lg[lane];
    if (a.dump) dump_chunk(a.counters + kDumpCount, static_cast<DoubletRec*>(a.dump), a.dump_cap,
                           valid, mid_idx, oth_idx, (TOP ? 1u : 0u) | (ev << 1), x, logit);
    __syncwarp();
    return logit;
}

// Learned doublet filter on the middle-bottom doublets q[0..n) of middle M:
// in-order compaction of those with logit >= threshold when the filter
// prunes bottoms (otherwise scoring only, for the dump).  Adds the scored /
// pruned counts to the event's filter counters.
template <int MODE>
__device__ __noinline__ uint32_t filter_bottoms(const DevConfig& c, const Arena& a,
                                                const NbViewT<MODE>& nb, const float4 M, uint16_t* q,
                                                uint32_t n, uint32_t* xs, float* lg,
                                                uint32_t ev, uint32_t gm, uint32_t lane,
                                                uint32_t lt) {
    MlpRegs R;
    mlp_load_regs(*c.mlp, lane, R);
    const bool prune = c.mlp_prune_bottom != 0;
    const float cosPhiM = M.x / M.w, sinPhiM = M.y / M.w;
    const float thr = filter_threshold(c, a, ev, 0);
    const float2 zero2 = make_float2(0.f, 0.f);
    const uint32_t mid_idx = a.dump ? a.g_idx[gm] : 0u;
    uint32_t w = 0;
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i = base + lane;
        const bool valid = i < n;
        uint16_t p = 0;
        float x[kMlpIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        uint32_t oth = 0;
        if (valid) {
            p = q[i];
            const float4 o = nb.get(p);
            const LinCircle l = lin_circle_cs(false, M, cosPhiM, sinPhiM, zero2, o, zero2);
            mlp_features(c.mlp_edges, c.mlp_n_edges, M, o, l.cot, l.s, l.Zo, x);
            if (a.dump) oth = a.g_idx[nb.gpos(nb.hpos(p))];
        }
        const float logit =
            score_chunk<false>(c, a, R, x, valid, xs, lg, ev, mid_idx, oth, lane, lt);
        const bool keep = valid && (!prune || logit >= thr);
        const uint32_t mask = __ballot_sync(0xffffffffu, keep);
        if (keep) q[w + __popc(mask & lt)] = p;
        w += __popc(mask);
        __syncwarp();
    }
    if (lane == 0) {
        atomicAdd(&a.ev_filter[4 * ev + 0], n);
        atomicAdd(&a.ev_filter[4 * ev + 1], n - w);
    }
    return w;
}

// The middle gate inside the plain seeding routine: true when one of the
// middle's middle-top doublets (neighbourhood positions q[0..n)) has a logit
// >= its event's threshold.  Features and network as in the scoring
// instantiation (the lin_circle's cot, s and Zo do not depend on the
// variances; the network's fragments are read from memory rather than held in
// registers, with the same operands and mma order, so the same logits).
// Doublets are scored 16 at a time (one network tile, lanes 0-15 computing
// the features), stopping at the first tile that decides.  Out of line and
// with rolled loops, so that the routine's hot loops keep their registers and
// the instruction cache its footprint.  xs: 64 words, lg: 16 floats of warp
// scratch.
template <int MODE>
__device__ __noinline__ bool gate_keeps_middle(const DevConfig& c, const Arena& a,
                                               const NbViewT<MODE>& nb, const float4 M,
                                               const uint16_t* q, uint32_t n_mt,
                                               uint32_t* xs, float* lg, uint32_t ev,
                                               uint32_t lane) {
    const float thr = filter_threshold(c, a, ev, 1);
    const float cosPhiM = M.x / M.w, sinPhiM = M.y / M.w;
    const float2 zero2 = make_float2(0.f, 0.f);
    uint32_t bm = 0;  // band of the middle spacepoint
#pragma unroll 1
    for (uint32_t e = 0; e < c.mlp_n_edges; ++e) bm += c.mlp_edges[e] <= M.w ? 1u : 0u;
#pragma unroll 1
    for (uint32_t base = 0; base < n_mt; base += 16) {
        const uint32_t i = base + lane;
        const bool valid = lane < 16 && i < n_mt;
        if (lane < 16) {
            uint32_t pk[4] = {0u, 0u, 0u, 0u};
            if (valid) {
                const float4 o = nb.get(q[i]);
                const LinCircle l = lin_circle_cs(true, M, cosPhiM, sinPhiM, zero2, o, zero2);
                uint32_t bo = 0;
#pragma unroll 1
                for (uint32_t e = 0; e < c.mlp_n_edges; ++e) bo += c.mlp_edges[e] <= o.w ? 1u : 0u;
                const float x[kMlpIn] = {M.w, M.z, o.w - M.w, o.z - M.z, l.cot, l.s, l.Zo,
                                         static_cast<float>(bm * (c.mlp_n_edges + 1) + bo)};
                mlp_pack_inputs(c.mlp_mu, c.mlp_isd, x, pk);
            }
            *reinterpret_cast<uint4*>(xs + 4 * lane) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
        __syncwarp();
        float lo, hi;
        mlp_tile16_lean(*c.mlp, xs, lane, lo, hi);
        if ((lane & 3) == 0) {
            const uint32_t g = lane >> 2;
            lg[g] = lo;
            lg[g + 8] = hi;
        }
        __syncwarp();
        const bool reach = valid && lg[lane & 15] >= thr;
        __syncwarp();
        if (__any_sync(0xffffffffu, reach)) return true;
    }
    return false;
}

// Seeds of one middle spacepoint, following host seed_finding::operator()
// (core/src/seeding/seed_finding.cpp:69-118) with triplet_finding
// (triplet_finding.hpp:60-183) and seed_filtering (seed_filtering.cpp:28-123).
// Executed by one full warp.  The order-dependent steps (compatible-seed
// weights, ties of the final sort) use host positions, so the result does not
// depend on the order in which doublets are found.
// VAR: read the spacepoint variances.  With VAR false every variance term is
// zero (valid when no spacepoint of the batch has a variance); the results
// are the same as with VAR true on such a batch, without the variance loads.
template <int MODE, bool SCORE, bool VAR, int CAPB, int CAPT, int CAPLC, int CAPCT,
          bool GATE = false>
__device__ MiddleResult process_middle(const DevConfig& c, const Arena& a,
                                       const NbViewT<MODE>& nb, const uint32_t gm,
                                       const bool check_r,
                                       const float nb_minr, const float nb_maxr,
                                       const uint32_t ev,
                                       WarpScratch<CAPB, CAPT, CAPLC, CAPCT>& ws) {
    MiddleResult res{0, 0, 0, 0};
    constexpr bool RSORTED = NbViewT<MODE>::kRSorted;
    constexpr bool any_var = VAR;
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

    // -- doublets: window cuts with ballot compaction
    uint32_t nqb = 0, nqt = 0;
    if constexpr (RSORTED) {
        // Exact radial windows per radius-sorted bin: deltaR = fl(rM - r)
        // (bottom) is non-increasing and fl(r - rM) (top) non-decreasing in r,
        // so the spacepoints with deltaRMin < deltaR < deltaRMax form one
        // contiguous range of each run, found by binary search on the same
        // float expressions the cut evaluates.
        const uint32_t ns = nb.nseg;
        for (uint32_t i = lane; i < 4 * ns; i += 32) {
            const uint32_t s = i >> 2, k = i & 3;
            uint32_t lo = nb.seg_pos[s], hi = nb.seg_pos[s + 1];
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                const float r = nb.staged[mid].w;
                const float d = (k < 2) ? (M.w - r) : (r - M.w);
                const bool pr = (k == 0) ? (d < c.deltaRMax)
                              : (k == 1) ? (d <= c.deltaRMin)
                              : (k == 2) ? (d > c.deltaRMin)
                                         : (d >= c.deltaRMax);
                if (pr) hi = mid; else lo = mid + 1;
            }
            ws.bnd[i] = lo;
        }
        __syncwarp();
        if (lane == 0) {
            uint32_t ab = 0, at = 0;
            for (uint32_t s = 0; s < ns; ++s) {
                ws.pre[s] = ab;
                ws.pre[kFastSegs + 1 + s] = at;
                const uint32_t b0 = ws.bnd[4 * s], b1 = ws.bnd[4 * s + 1];
                const uint32_t t0 = ws.bnd[4 * s + 2], t1 = ws.bnd[4 * s + 3];
                ab += b1 > b0 ? b1 - b0 : 0u;
                at += t1 > t0 ? t1 - t0 : 0u;
            }
            ws.pre[ns] = ab;
            ws.pre[kFastSegs + 1 + ns] = at;
        }
        __syncwarp();
        if (ws.pre[ns] == 0 || ws.pre[kFastSegs + 1 + ns] == 0) {
            if (lane == 0) a.seed_cnt[gm] = 0;
            return res;
        }
        nqb = scan_runs<false, MODE>(c, nb, M, ws.bnd, ws.pre, ns, ws.qb, CAPB, lane, lt);
        nqt = scan_runs<true, MODE>(c, nb, M, ws.bnd, ws.pre + kFastSegs + 1, ns, ws.qt, CAPT,
                                    lane, lt);
    } else {
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
    }
    if (nqb > CAPB || nqt > CAPT) { res.status = 1; return res; }
    __syncwarp();
    uint32_t n_mb = nqb ? helix_compact(c, nb, M, ws.qb, nqb, lane, lt) : 0u;
    uint32_t n_mt = (n_mb && nqt) ? helix_compact(c, nb, M, ws.qt, nqt, lane, lt) : 0u;
    res.n_mb = n_mb;
    res.n_mt = n_mt;
    if (n_mb == 0 || n_mt == 0) {
        if (lane == 0) a.seed_cnt[gm] = 0;
        return res;
    }
    if constexpr (SCORE) {
        // learned doublet filter on the middle-bottom doublets (when it prunes
        // them, or to record them); the cot-bucket tables are free until the
        // middle-top doublets are sorted below
        if (c.mlp_prune_bottom || a.dump) {
            uint32_t* xs = ws.bstart;
            float* lg = reinterpret_cast<float*>(ws.bstart + 128);
            n_mb = filter_bottoms(c, a, nb, M, ws.qb, n_mb, xs, lg, ev, gm, lane, lt);
            if (n_mb == 0) {
                if (lane == 0) a.seed_cnt[gm] = 0;
                return res;
            }
        }
    }
    if (n_mt > CAPLC) { res.status = 1; return res; }
    if constexpr (!SCORE && GATE) {
        // learned middle gate, the scoring instantiation's decision, before
        // any middle-top work (the cot-bucket tables are free scratch here);
        // middles above the gate's size limit are kept unscored
        const bool keep =
            (c.mlp_gate_max_tops != 0 && n_mt > c.mlp_gate_max_tops) ||
            gate_keeps_middle(c, a, nb, M, ws.qt, n_mt, ws.bstart,
                              reinterpret_cast<float*>(ws.bstart + 128), ev, lane);
        if (lane == 0) {
            atomicAdd(&a.ev_filter[4 * ev + 2], n_mt);
            if (!keep) atomicAdd(&a.ev_filter[4 * ev + 3], n_mt);
        }
        __syncwarp();
        if (!keep) {
            res.n_mt = 0;
            if (lane == 0) a.seed_cnt[gm] = 0;
            return res;
        }
    }

    // -- middle-top lin_circles (list order) and a counting sort by cot(theta)
    const float cosPhiM = M.x / M.w, sinPhiM = M.y / M.w;
    float maxEr = 0.f, minEr = 0.f, maxCot = 0.f, maxIdr = 0.f;
    float cmin = __int_as_float(0x7f800000), cmax = -__int_as_float(0x7f800000);
    if constexpr (SCORE) {
        // learned doublet filter on the middle-top doublets, fused into their
        // lin_circle set-up: the survivors are written in order
        MlpRegs R;
        mlp_load_regs(*c.mlp, lane, R);
        uint32_t* xs = ws.bstart;
        float* lg = reinterpret_cast<float*>(ws.bstart + 128);
        // mlp_prune_top: 1 drops the doublets below the threshold; 2 gates
        // the whole middle (it yields no seed unless one of its middle-top
        // doublets reaches the threshold, and then runs unpruned)
        const bool prune = c.mlp_prune_top == SEEDGB_FILTER_PRUNE_DOUBLETS;
        const bool gate = c.mlp_prune_top == SEEDGB_FILTER_GATE_MIDDLE;
        const float thr = filter_threshold(c, a, ev, 1);
        const uint32_t mid_idx = a.dump ? a.g_idx[gm] : 0u;
        uint32_t w = 0;
        bool reach = false;
        // gate: once a doublet of the middle reaches the threshold the middle
        // is kept whatever the rest score, so the remaining chunks are not
        // scored (unless every score is recorded); warp-uniform
        bool decided = false;
        for (uint32_t base = 0; base < n_mt; base += 32) {
            const uint32_t i = base + lane;
            const bool valid = i < n_mt;
            const bool score = !(gate && decided && !a.dump);
            uint32_t p = 0, hp = 0, oth = 0;
            LinCircle l{};
            float x[kMlpIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (valid) {
                p = ws.qt[i];
                hp = nb.hpos(p);
                const float2 vo = any_var ? a.g_var[nb.gpos(hp)] : make_float2(0.f, 0.f);
                const float4 o = nb.get(p);
                l = lin_circle_cs(true, M, cosPhiM, sinPhiM, vM, o, vo);
                if (score) mlp_features(c.mlp_edges, c.mlp_n_edges, M, o, l.cot, l.s, l.Zo, x);
                if (a.dump) oth = a.g_idx[nb.gpos(hp)];
            }
            const float logit =
                score ? score_chunk<true>(c, a, R, x, valid, xs, lg, ev, mid_idx, oth, lane, lt)
                      : thr;
            const bool keep = valid && (!prune || logit >= thr);
            reach |= valid && logit >= thr;
            if (gate) decided = __any_sync(0xffffffffu, reach);
            const uint32_t mask = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const uint32_t k = w + __popc(mask & lt);
                ws.mtd[k] = make_float4(l.cot, l.idr, l.u, l.v);
                ws.er[k] = l.er;
                ws.hpt[k] = static_cast<uint16_t>(hp);
                ws.ppt[k] = static_cast<uint16_t>(p);
                maxEr = fmaxf(maxEr, l.er);
                minEr = fminf(minEr, l.er);
                maxCot = fmaxf(maxCot, fabsf(l.cot));
                maxIdr = fmaxf(maxIdr, l.idr);
                cmin = fminf(cmin, l.cot);
                cmax = fmaxf(cmax, l.cot);
                if (!(l.er == l.er)) minEr = -1.f;
            }
            w += __popc(mask);
            __syncwarp();
        }
        // gated (no seed) unless the middle is too large to be gated
        if (gate && (c.mlp_gate_max_tops == 0 || n_mt <= c.mlp_gate_max_tops) &&
            !__any_sync(0xffffffffu, reach))
            w = 0;
        if (lane == 0) {
            atomicAdd(&a.ev_filter[4 * ev + 2], n_mt);
            atomicAdd(&a.ev_filter[4 * ev + 3], n_mt - w);
        }
        __syncwarp();
        n_mt = w;
        res.n_mt = w;
        if (n_mt == 0) {
            if (lane == 0) a.seed_cnt[gm] = 0;
            return res;
        }
    } else {
        for (uint32_t i = lane; i < n_mt; i += 32) {
            const uint32_t p = ws.qt[i];
            const uint32_t hp = nb.hpos(p);
            const float2 vo = any_var ? a.g_var[nb.gpos(hp)] : make_float2(0.f, 0.f);
            const LinCircle l = lin_circle_cs(true, M, cosPhiM, sinPhiM, vM, nb.get(p), vo);
            ws.mtd[i] = make_float4(l.cot, l.idr, l.u, l.v);
            ws.er[i] = l.er;
            ws.hpt[i] = static_cast<uint16_t>(hp);
            ws.ppt[i] = static_cast<uint16_t>(p);
            maxEr = fmaxf(maxEr, l.er);
            minEr = fminf(minEr, l.er);
            maxCot = fmaxf(maxCot, fabsf(l.cot));
            maxIdr = fmaxf(maxIdr, l.idr);
            cmin = fminf(cmin, l.cot);
            cmax = fmaxf(cmax, l.cot);
            if (!(l.er == l.er)) minEr = -1.f;  // NaN error term: no window
        }
    }
    for (uint32_t b = lane; b <= kBuckets; b += 32) ws.bstart[b] = 0;
    for (int o = 16; o > 0; o >>= 1) {
        cmin = fminf(cmin, __shfl_xor_sync(0xffffffffu, cmin, o));
        cmax = fmaxf(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
        if (any_var) {
            maxEr = fmaxf(maxEr, __shfl_xor_sync(0xffffffffu, maxEr, o));
            minEr = fminf(minEr, __shfl_xor_sync(0xffffffffu, minEr, o));
            maxCot = fmaxf(maxCot, __shfl_xor_sync(0xffffffffu, maxCot, o));
            maxIdr = fmaxf(maxIdr, __shfl_xor_sync(0xffffffffu, maxIdr, o));
        }
    }
    const float scale = (cmax > cmin) ? static_cast<float>(kBuckets) / (cmax - cmin) : 0.f;
    __syncwarp();
    for (uint32_t i = lane; i < n_mt; i += 32)
        atomicAdd(&ws.bstart[cot_bucket(ws.mtd[i].x, cmin, scale) + 1], 1u);
    __syncwarp();
    {
        // exclusive prefix over the buckets, kBuckets / 32 per lane
        constexpr int kPer = kBuckets / 32;
        uint32_t v[kPer], sum = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) { v[j] = ws.bstart[kPer * lane + j + 1]; sum += v[j]; }
        uint32_t incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += t;
        }
        __syncwarp();
        uint32_t run = incl - sum;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            ws.bcur[kPer * lane + j] = run;
            run += v[j];
            ws.bstart[kPer * lane + j + 1] = run;
        }
    }
    __syncwarp();
    for (uint32_t i = lane; i < n_mt; i += 32) {
        const float kt = ws.mtd[i].x;
        const uint32_t slot = atomicAdd(&ws.bcur[cot_bucket(kt, cmin, scale)], 1u);
        ws.perm[slot] = static_cast<uint16_t>(i);
        // without variances the error terms are never read again: er holds
        // the tops' cot(theta) in bucket order, so the window walk below reads
        // it beside perm instead of through it
        if constexpr (!any_var) ws.er[slot] = kt;
    }
    __syncwarp();

    // -- triplets.  The middle-bottom doublets are set up 32 at a time (one
    //    per lane); each lane walks the middle-top doublets of its cot
    //    buckets and queues those inside its exact cot window (q0, with the
    //    doublet's lin_circle), one entry per lane per step; stage 1 runs on
    //    32 queued candidates at a time, stage 2 on 32 stage-1 survivors at a
    //    time, so both run with full lanes across doublets and chunks.  Both
    //    queues are rings of 64 entries (heads h0 / h1, counts n0 / n1, at
    //    most 63 held), so what a stage leaves stays in place.
    const float sig2 = c.sigmaScattering * c.sigmaScattering;
    uint32_t n_ct = 0, n0 = 0, n1 = 0, h1 = 0, h0 = 0;
    uint32_t c0 = 0, it = 0, maxc = 0;
    bool have_chunk = false;
    LinCircle lbm;
    lbm.Zo = 0.f;
    float klo = 0.f, khi = 0.f;
    uint32_t lo = 0, cnt = 0;
    for (;;) {
        __syncwarp();
        if (!have_chunk && c0 < n_mb) {
            const uint32_t ib = c0 + lane;
            cnt = 0;
            if (ib < n_mb) {
                const uint32_t pB = ws.qb[ib];
                const float4 B = nb.get(pB);
                const float2 vB =
                    any_var ? a.g_var[nb.gpos(nb.hpos(pB))] : make_float2(0.f, 0.f);
                lbm = lin_circle_cs(false, M, cosPhiM, sinPhiM, vM, B, vB);
                // triplet_finding.hpp:82-88
                const float iSinTheta2 = 1.f + lbm.cot * lbm.cot;
                float scatteringInRegion2 = c.maxScatteringAngle2 * iSinTheta2;
                scatteringInRegion2 *= sig2;
                // Window in cot(theta): a middle-top doublet outside it fails
                // the reference's first scattering test for any rounding (1 %
                // relative and 1e-5 absolute margins), so only doublets inside
                // are tested.
                float W;
                if (c.brute_force_triplets) {
                    W = __int_as_float(0x7f800000);
                } else if (!any_var) {
                    // approximate square root: its ~1e-6 relative error is far
                    // inside the 1 % margin
                    const float sq = scatteringInRegion2 > 1e-30f
                                         ? scatteringInRegion2 * rsqrtf(scatteringInRegion2)
                                         : sqrtf(scatteringInRegion2);
                    W = sq * 1.01f + 1e-5f * (1.f + fabsf(lbm.cot));
                } else {
                    const float e2 =
                        (maxEr + lbm.er +
                         2.f * (fabsf(lbm.cot) * maxCot * fabsf(vM.y) + fabsf(vM.x)) *
                             lbm.idr * maxIdr) * 1.001f;
                    const bool ok = (minEr >= 0.f) && (lbm.er >= 0.f) && (vM.x >= 0.f) &&
                                    (vM.y >= 0.f) && (e2 >= 0.f) && (e2 < 3.0e38f);
                    W = ok ? (sqrtf(scatteringInRegion2) + sqrtf(e2)) * 1.01f +
                                 1e-5f * (1.f + fabsf(lbm.cot))
                           : __int_as_float(0x7f800000);
                }
                klo = lbm.cot - W;
                khi = lbm.cot + W;
                lo = ws.bstart[cot_bucket(klo, cmin, scale)];
                cnt = ws.bstart[cot_bucket(khi, cmin, scale) + 1] - lo;
            }
            maxc = cnt;
            for (int o = 16; o > 0; o >>= 1) maxc = max(maxc, __shfl_xor_sync(0xffffffffu, maxc, o));
            it = 0;
            have_chunk = true;
        }
        if (have_chunk) {
            while (it < maxc && n0 < 32) {
                {
                    const uint32_t j = it;
                    bool ok = false;
                    uint32_t tp = 0;
                    if (j < cnt) {
                        tp = ws.perm[lo + j];
                        const float kt = any_var ? ws.mtd[tp].x : ws.er[lo + j];
                        ok = kt >= klo && kt <= khi;
                    }
                    const uint32_t mask = __ballot_sync(0xffffffffu, ok);
                    if (ok) {
                        Stage0Cand e;
                        e.tp = static_cast<uint16_t>(tp);
                        e.ib = static_cast<uint16_t>(c0 + lane);
                        e.cot = lbm.cot;
                        e.idr = lbm.idr;
                        e.er = lbm.er;
                        e.u = lbm.u;
                        e.v = lbm.v;
                        ws.q.q0[(h0 + n0 + __popc(mask & lt)) & 63u] = e;
                    }
                    n0 += __popc(mask);
                }
                ++it;
            }
            if (it >= maxc) {
                have_chunk = false;
                c0 += 32;
            }
        }
        __syncwarp();
        const bool more = have_chunk || c0 < n_mb;
        if (n0 >= 32 || (!more && n0 > 0)) {
            // stage 1 on q0[0..k), survivors to q1
            const uint32_t k1 = min(n0, 32u);
            {
                const uint32_t i = lane;
                bool ok = false;
                Stage1Cand s1;
                if (i < k1) {
                    const Stage0Cand e = ws.q.q0[(h0 + i) & 63u];
                    LinCircle lb;
                    lb.cot = e.cot;
                    lb.idr = e.idr;
                    lb.er = e.er;
                    lb.u = e.u;
                    lb.v = e.v;
                    lb.Zo = 0.f;
                    const float iSinTheta2 = 1.f + lb.cot * lb.cot;
                    float scatteringInRegion2 = c.maxScatteringAngle2 * iSinTheta2;
                    scatteringInRegion2 *= sig2;
                    const float4 mt = ws.mtd[e.tp];
                    // with no variance anywhere every Er is +0 (transform_
                    // coordinates multiplies (0 + 0) + cot^2 (0 + 0) by iDeltaR2)
                    const float ter = any_var ? ws.er[e.tp] : 0.f;
                    ok = triplet_stage1(c, vM, lb, mt.x, mt.y, ter, mt.z, mt.w,
                                        scatteringInRegion2, s1.A, s1.B);
                    s1.tp = e.tp;
                    s1.ib = e.ib;
                    s1.cot = e.cot;
                    s1.idr = e.idr;
                    s1.er = e.er;
                    s1.is2 = iSinTheta2;
                }
                const uint32_t mask = __ballot_sync(0xffffffffu, ok);
                if (ok) ws.q.q1[(h1 + n1 + __popc(mask & lt)) & 63u] = s1;
                n1 += __popc(mask);
            }
            h0 = (h0 + k1) & 63u;
            n0 -= k1;
            __syncwarp();
        }
        while (n1 >= 32 || (!more && n0 == 0 && n1 > 0)) {
            // stage 2 on q1[0..k), triplets to ct
            const uint32_t k2 = min(n1, 32u);
            bool ok = false;
            TripCand t;
            if (lane < k2) {
                const Stage1Cand e = ws.q.q1[(h1 + lane) & 63u];
                LinCircle lb;
                lb.cot = e.cot;
                lb.idr = e.idr;
                lb.er = e.er;
                lb.u = lb.v = lb.Zo = 0.f;
                float curv = 0.f, imp = 0.f;
                const float4 mt = ws.mtd[e.tp];
                const float ter = any_var ? ws.er[e.tp] : 0.f;
                ok = triplet_stage2(c, M.w, vM, lb, mt.x, mt.y, ter, e.is2, e.A, e.B, curv,
                                    imp);
                t.tp = e.tp;
                t.ib = e.ib;
                t.curv = curv;
                t.w = -imp * c.impactWeightFactor;
            }
            const uint32_t mask = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                const uint32_t k = n_ct + __popc(mask & lt);
                if (k < CAPCT) ws.ct[k] = t;
            }
            n_ct += __popc(mask);
            h1 = (h1 + k2) & 63u;
            n1 -= k2;
            __syncwarp();
        }
        if (!more && n0 == 0 && n1 == 0) break;
    }
    if (n_ct > CAPCT) { res.status = 1; return res; }
    res.n_trip = n_ct;
    if constexpr (SCORE) {
        if (a.tdump && n_ct) {
            // record the middle's triplets (labels of the filter's training data)
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(&a.counters[kTripDumpCount], static_cast<unsigned long long>(n_ct));
            __syncwarp();
            b = __shfl_sync(0xffffffffu, b, 0);
            const uint32_t mid_idx = a.g_idx[gm];
            for (uint32_t i = lane; i < n_ct; i += 32) {
                if (b + i < a.tdump_cap) {
                    const TripCand T = ws.ct[i];
                    a.tdump[b + i] = make_uint4(mid_idx, a.g_idx[nb.gpos(nb.hpos(ws.qb[T.ib]))],
                                                a.g_idx[nb.gpos(ws.hpt[T.tp])], ev);
                }
            }
            __syncwarp();
        }
    }

    // -- the middle's triplets in host order: (bottom host position, top
    //    host position) ascending, so the triplets of one middle-bottom
    //    doublet form a run ordered as triplet_finding.hpp:109-179 visits them,
    //    and the position in this order breaks exact ties of the final sort
    //    as the reference's triplet list order does
    {
        uint32_t P = 1;
        while (P < n_ct) P <<= 1;
        for (uint32_t i = lane; i < P; i += 32) {
            // host order: the bottom's host position (the middle-bottom list
            // itself is in radius order), then the top's
            ws.skey[i] = i < n_ct ? ((nb.hpos(ws.qb[ws.ct[i].ib]) << 16) |
                                     ws.hpt[ws.ct[i].tp])
                                  : 0xffffffffu;
            ws.sidx[i] = static_cast<uint16_t>(i);
        }
        __syncwarp();
        for (uint32_t k = 2; k <= P; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t t = lane; t < P / 2; t += 32) {
                    const uint32_t i = 2 * t - (t & (j - 1));
                    const uint32_t l = i + j;
                    const bool up = (i & k) == 0;
                    const uint32_t ki = ws.skey[i], kl = ws.skey[l];
                    if (up ? (ki > kl) : (ki < kl)) {
                        ws.skey[i] = kl;
                        ws.skey[l] = ki;
                        const uint16_t x = ws.sidx[i];
                        ws.sidx[i] = ws.sidx[l];
                        ws.sidx[l] = x;
                    }
                }
                __syncwarp();
            }
        }
    }

    // the lane's best untaken triplet (cw, cs, ck), kept as the weights are
    // written (the order of better; ck = 0xffffffff: none)
    float cw = 0.f, cs = 0.f;
    uint32_t ck = 0xffffffffu;
    // -- weights, one lane per triplet: compatible-seed weights over its
    //    doublet's run (triplet_finding.hpp:107-179), seed_weight and
    //    single_seed_cut (seed_selecting_helper.hpp:27-62)
    for (uint32_t k = lane; k < n_ct; k += 32) {
        const TripCand T = ws.ct[ws.sidx[k]];
        const uint32_t hB = ws.skey[k] >> 16;
        uint32_t b = k, e = k + 1;
        while (b > 0 && (ws.skey[b - 1] >> 16) == hB) --b;
        while (e < n_ct && (ws.skey[e] >> 16) == hB) ++e;
        const float4 Tp = nb.get(ws.ppt[T.tp]);
        float w = T.w;
        if (e - b > 1) {
            const float currentTop_r = Tp.w;
            const float lowerLimitCurv = T.curv - c.deltaInvHelixDiameter;
            const float upperLimitCurv = T.curv + c.deltaInvHelixDiameter;
            float compR[8];
            uint32_t ncr = 0;
            for (uint32_t j = b; j < e; ++j) {
                if (j == k) continue;
                const TripCand Tj = ws.ct[ws.sidx[j]];
                const float otherTop_r = nb.get(ws.ppt[Tj.tp]).w;
                const float deltaR = currentTop_r - otherTop_r;
                if (fabsf(deltaR) < c.filterDeltaRMin) continue;
                if (Tj.curv < lowerLimitCurv) continue;
                if (Tj.curv > upperLimitCurv) continue;
                bool newCompSeed = true;
                for (uint32_t q = 0; q < ncr && q < 8; ++q) {
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
        }
        const float4 B = nb.get(ws.qb[T.ib]);
        float weight = 0;
        if (B.w > c.good_spB_min_radius) weight = c.good_spB_weight_increase;
        if (Tp.w < c.good_spT_max_radius) weight = c.good_spT_weight_increase;
        w += weight;
        const bool cut = B.w > c.good_spB_min_radius && w < c.good_spB_min_weight;
        const float wk = cut ? -__int_as_float(0x7f800000) : w;
        const float tk = B.y * B.y + B.z * B.z + Tp.y * Tp.y + Tp.z * Tp.z;
        ws.wf[k] = wk;
        ws.ts[k] = tk;
        if (wk != -__int_as_float(0x7f800000) &&
            (ck == 0xffffffffu || better(wk, tk, k, cw, cs, ck))) {
            cw = wk;
            cs = tk;
            ck = k;
        }
    }
    __syncwarp();

    // -- the best K triplets in triplet_sorter order (K warp argmax rounds),
    //    then the final selection (seed_filtering.cpp:87-122).  Index k of
    //    the sorted triplets is their host order (the tie-break).
    const uint32_t K = min(c.maxSeedsPerSpM, static_cast<uint32_t>(kMaxSeedsPerMiddle));
    // Each lane holds its best untaken triplet among k = lane, lane + 32, ...
    // A round takes the warp's best by three warp reductions over order-
    // preserving keys (weight, then tie sum, then host order); only the lane
    // that held it looks for its next best.
    float my_w = 0.f;
    uint32_t my_k = 0, n_sel = 0;
    for (uint32_t r = 0; r < K; ++r) {
        const bool has = ck != 0xffffffffu;
        if (!__any_sync(0xffffffffu, has)) break;
        const uint32_t kw = has ? order_key(cw) : 0u;
        const uint32_t mw = __reduce_max_sync(0xffffffffu, kw);
        const bool c1 = has && kw == mw;
        const uint32_t ks = c1 ? order_key(cs) : 0u;
        const uint32_t ms = __reduce_max_sync(0xffffffffu, ks);
        const uint32_t mk = __reduce_min_sync(0xffffffffu, (c1 && ks == ms) ? ck : 0xffffffffu);
        const uint32_t owner = mk & 31u;
        const float w_sel = __shfl_sync(0xffffffffu, cw, owner);
        if (lane == r) {
            my_w = w_sel;
            my_k = mk;
        }
        if (lane == owner) {
            ws.wf[mk] = -__int_as_float(0x7f800000);  // taken
            lane_best(ws.wf, ws.ts, n_ct, lane, cw, cs, ck);
        }
        ++n_sel;
    }
    bool acc = false;
    uint32_t my_p = 0;
    if (lane < n_sel) {
        const TripCand T = ws.ct[ws.sidx[my_k]];
        my_p = (static_cast<uint32_t>(ws.qb[T.ib]) << 16) | ws.ppt[T.tp];
        const float4 Bsel = nb.get(my_p >> 16);
        acc = (lane == 0) || (my_w > c.seed_min_weight) || (Bsel.w > c.spB_min_radius);
    }
    const uint32_t amask = __ballot_sync(0xffffffffu, acc);
    if (acc) {
        const uint32_t k = __popc(amask & lt);
        SeedSlot s;
        s.b = a.g_idx[nb.gpos(nb.hpos(my_p >> 16))];
        s.m = a.g_idx[gm];
        s.t = a.g_idx[nb.gpos(nb.hpos(my_p & 0xffffu))];
        s.q = my_w;
        a.seed_slot[static_cast<size_t>(gm) * kMaxSeedsPerMiddle + k] = s;
    }
    if (lane == 0) a.seed_cnt[gm] = static_cast<uint8_t>(__popc(amask));
    return res;
}

__device__ __forceinline__ void push_overflow(const Arena& a, uint32_t gm) {
    const unsigned long long k = atomicAdd(&a.counters[kOvfCount], 1ull);
    if (k < 2ull * a.cap_sp) a.ovf[k] = gm;
    else raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
    a.seed_cnt[gm] = 0;
}

__device__ __forceinline__ void count_middle(const Arena& a, const MiddleResult& r) {
    if (r.n_mb) atomicAdd(&a.counters[kNumMB], static_cast<unsigned long long>(r.n_mb));
    if (r.n_mt) atomicAdd(&a.counters[kNumMT], static_cast<unsigned long long>(r.n_mt));
    if (r.n_trip) atomicAdd(&a.counters[kNumTriplets], static_cast<unsigned long long>(r.n_trip));
}

// Shared-memory layout of k_seed_fast: the staged neighbourhood (float4 and
// host position), the segment tables, then one scratch per warp at a
// 128-byte boundary (the scratch holds float4 arrays).
static_assert(alignof(FastScratch) <= 128, "scratch alignment");
static_assert(sizeof(FastScratch) % 16 == 0, "scratch size");
__host__ __device__ constexpr size_t fast_seg_offset(uint32_t nb_cap) {
    return (static_cast<size_t>(nb_cap) * (sizeof(float4) + sizeof(uint16_t)) + 15) &
           ~static_cast<size_t>(15);
}
__host__ __device__ constexpr size_t fast_scratch_offset(uint32_t nb_cap) {
    return (fast_seg_offset(nb_cap) + (3 * kMaxSegments + 1 + 16) * sizeof(uint32_t) + 127) &
           ~static_cast<size_t>(127);
}

// Persistent loop over work items (event, bin, chunk of middles).  The CTA
// stages the bin's neighbourhood (radius-sorted runs) once per item; its warps
// then take middles of the item one at a time.
// pass 0: every event (with the learned filter when one is installed);
// pass 1: only the events marked for the fallback, without the filter.
// SCORE: run the learned doublet filter (pass 0 with a filter installed).
// The scoring variant holds the network in registers: at most
// kScoreWarps warps per CTA, so that each thread keeps 168 registers (14
// warps would force 128 and spill: 11 % slower than 12).
constexpr int kScoreWarps = 12;
template <bool SCORE, bool VAR, bool GATE = false>
__device__ __forceinline__ void seed_fast_items(const DevConfig& c, const Arena& a, uint32_t mpi,
                                                uint32_t nb_cap, uint32_t pass) {
    extern __shared__ __align__(128) uint8_t smem[];
    float4* nb_xyzr = reinterpret_cast<float4*>(smem);
    uint16_t* nb_hp = reinterpret_cast<uint16_t*>(nb_xyzr + nb_cap);      // [nb_cap]
    uint32_t* seg_pos = reinterpret_cast<uint32_t*>(smem + fast_seg_offset(nb_cap));
    uint32_t* seg_g = seg_pos + kMaxSegments + 1;                          // [kMaxSegments]
    uint32_t* seg_bin = seg_g + kMaxSegments;                              // [kMaxSegments]
    uint32_t* misc = seg_bin + kMaxSegments;                               // [16]
    FastScratch* wsb = reinterpret_cast<FastScratch*>(smem + fast_scratch_offset(nb_cap));
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    FastScratch& ws = wsb[warp];
    const uint32_t total_items = static_cast<uint32_t>(
        min(a.counters[kItemTotal], static_cast<unsigned long long>(a.max_items)));
    unsigned long long* fetch = &a.counters[pass ? kItemFetch2 : kItemFetch];
    // lane 0: this warp's doublet and triplet counts, added to the batch's
    // counters once per item instead of once per middle
    uint32_t agg_mb = 0, agg_mt = 0, agg_trip = 0;

    for (;;) {
        if (threadIdx.x == 0) {
            misc[0] = static_cast<uint32_t>(atomicAdd(fetch, 1ull));
            misc[3] = 0x7f800000u;  // min r (as bits, r >= 0)
            misc[4] = 0u;           // max r
            misc[5] = 0u;           // next middle of the item
            misc[6] = 0u;           // any unsorted bin
        }
        __syncthreads();
        const uint32_t item = misc[0];
        if (item >= total_items) break;
        const uint2 it = a.items_ord[item];
        const uint32_t e = it.x, bin = it.y & 0xffffu, ch = it.y >> 16;
        if (pass && !a.ev_mode[e]) {
            __syncthreads();  // misc[0] is rewritten by the next fetch
            continue;
        }
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
            misc[2] = build_segments(c, bs, pbin, zlo, zhi, seg_pos, seg_g, &ns, seg_bin);
            misc[1] = ns;
        }
        __syncthreads();
        const uint32_t nseg = misc[1], size = misc[2];
        if (threadIdx.x < nseg &&
            a.bin_unsorted[static_cast<size_t>(e) * c.nbins + seg_bin[threadIdx.x]])
            misc[6] = 1u;
        __syncthreads();
        const bool staged = size <= nb_cap && size <= 65535u && nseg <= kFastSegs && !misc[6];
        if (staged) {
            float lmin = __int_as_float(0x7f800000), lmax = 0.f;
            for (uint32_t s = 0; s < nseg; ++s) {
                const uint32_t p0 = seg_pos[s], len = seg_pos[s + 1] - p0, g0 = seg_g[s];
                for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) {
                    const float4 v = a.g_rs[g0 + k];
                    nb_xyzr[p0 + k] = v;
                    nb_hp[p0 + k] = static_cast<uint16_t>(p0 + (a.g_rs_gp[g0 + k] - g0));
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
        // only staged neighbourhoods reach process_middle here (the others go
        // to the large-capacity kernel)
        NbViewT<kNbShared> nb{nb_xyzr, nb_hp, nullptr, 0u, a.g_xyzr, seg_pos, seg_g, nseg, size};
        const uint32_t m0 = bs[bin] + ch * mpi;
        const uint32_t m1 = min(m0 + mpi, bs[bin + 1]);
        for (;;) {
            uint32_t k = 0;
            if (lane == 0) k = atomicAdd(&misc[5], 1u);
            k = __shfl_sync(0xffffffffu, k, 0);
            const uint32_t gm = m0 + k;
            if (gm >= m1) break;
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
            const MiddleResult r = process_middle<kNbShared, SCORE, VAR, 512, 1024, 216, 128, GATE>(
                c, a, nb, gm, true, nb_minr, nb_maxr, e, ws);
            if (lane == 0) {
                if (r.status) {
                    push_overflow(a, gm);
                } else {
                    agg_mb += r.n_mb;
                    agg_mt += r.n_mt;
                    agg_trip += r.n_trip;
                }
            }
        }
        if (lane == 0) {
            count_middle(a, MiddleResult{agg_mb, agg_mt, agg_trip, 0});
            agg_mb = agg_mt = agg_trip = 0;
        }
        __syncthreads();
    }
}

// The fast seeding kernel: one branch on the batch's variance flag (set by
// binning) picks the body; without variances the body carries no variance
// loads (3 % faster on the 100k-spacepoint events).
// GATE: the learned middle gate inside the plain routine (pass 0 with a filter
// that only gates middles); a separate instantiation, so that the plain
// kernel's registers and code stay those of plain seeding.
// One CTA per SM (shared memory holds one): the explicit minimum keeps ptxas
// from aiming at two CTAs' 64 registers per thread, which spills this routine.
template <bool SCORE, bool GATE = false>
__global__ void __launch_bounds__(SCORE ? kScoreWarps * 32 : 512, 1)
    k_seed_fast(DevConfig c, Arena a, uint32_t mpi, uint32_t nb_cap, uint32_t pass) {
    if (a.counters[kAnyVariance] != 0) seed_fast_items<SCORE, true, GATE>(c, a, mpi, nb_cap, pass);
    else seed_fast_items<SCORE, false, GATE>(c, a, mpi, nb_cap, pass);
}

// General path, for the middles the fast kernel hands over (neighbourhood not
// staged: too many spacepoints or bins, an unsorted bin, or a per-middle z
// neighbourhood other than the bin's; or a list beyond the fast capacities).
// Every warp takes one middle at a time from its tier's queue and builds the
// middle's own neighbourhood in global memory: the bins' radius-sorted copies
// (exact radial windows) when the bins are consecutive in the grid, else the
// grid in host order.
// Two tiers: the middle tier (many warps per SM, about twice the fast
// kernel's list capacities) takes every handed-over middle and passes the
// ones whose lists do not fit to the last tier (one warp per SM with large
// capacities).
constexpr size_t kGeneralSegBytes = 1024;  // per warp: segments of the middle's neighbourhood

template <typename Scratch>
__host__ __device__ constexpr size_t general_warp_bytes() {
    return (kGeneralSegBytes + sizeof(Scratch) + 127) & ~static_cast<size_t>(127);
}

template <bool SCORE, bool VAR, bool LAST, int CAPB, int CAPT, int CAPLC, int CAPCT,
          bool GATE = false>
__device__ __forceinline__ void general_middles(const DevConfig& c, const Arena& a,
                                                uint32_t pass) {
    using Scratch = WarpScratch<CAPB, CAPT, CAPLC, CAPCT>;
    extern __shared__ __align__(128) uint8_t smem[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t* wbase = smem + static_cast<size_t>(warp) * general_warp_bytes<Scratch>();
    uint32_t* seg_pos = reinterpret_cast<uint32_t*>(wbase);   // [kMaxSegments+1]
    uint32_t* seg_g = seg_pos + kMaxSegments + 1;             // [kMaxSegments]
    uint32_t* seg_bin = seg_g + kMaxSegments;                 // [kMaxSegments]
    uint32_t* misc = seg_bin + kMaxSegments;                  // [2]
    static_assert(sizeof(uint32_t) * (3 * kMaxSegments + 3) <= kGeneralSegBytes,
                  "general segment layout");
    Scratch& ws = *reinterpret_cast<Scratch*>(wbase + kGeneralSegBytes);
    const uint32_t* queue = LAST ? a.ovf2 : a.ovf;
    const uint32_t n = static_cast<uint32_t>(
        min(a.counters[LAST ? kOvf2Count : kOvfCount], 2ull * a.cap_sp));
    const uint32_t n_events = a.hdr->n_events;
    unsigned long long* fetch =
        &a.counters[LAST ? (pass ? kOvf2Fetch2 : kOvf2Fetch) : (pass ? kOvfFetch2 : kOvfFetch)];
    for (;;) {
        uint32_t idx = 0;
        if (lane == 0) idx = static_cast<uint32_t>(atomicAdd(fetch, 1ull));
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= n) break;
        const uint32_t gm = queue[idx];
        if (!LAST && c.last_tier_only) {
            if (lane == 0) {
                const unsigned long long k = atomicAdd(&a.counters[kOvf2Count], 1ull);
                if (k < 2ull * a.cap_sp) a.ovf2[k] = gm;
                else raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
                a.seed_cnt[gm] = 0;
            }
            __syncwarp();
            continue;
        }
        // event: last with sp_base <= gm
        uint32_t lo = 0, hi = n_events;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (a.events[mid].sp_base <= gm) lo = mid; else hi = mid;
        }
        const uint32_t e = lo;
        if (pass && !a.ev_mode[e]) continue;
        const uint32_t* bs = a.bin_start + static_cast<size_t>(e) * (c.nbins + 1);
        uint32_t b0 = 0, b1 = c.nbins;  // last bin with bs[b] <= gm
        while (b1 - b0 > 1) {
            const uint32_t mid = (b0 + b1) >> 1;
            if (bs[mid] <= gm) b0 = mid; else b1 = mid;
        }
        uint32_t zlo, zhi;
        z_range(c, a.g_xyzr[gm].z, zlo, zhi);
        if (lane == 0) {
            uint32_t ns;
            build_segments(c, bs, b0 % c.phi_bins, zlo, zhi, seg_pos, seg_g, &ns, seg_bin);
            // the bins' radius-sorted copies serve as one array (exact radial
            // windows) when the bins are consecutive in the grid, all sorted,
            // and few enough for the windows' scratch
            uint32_t rs = (ns >= 1 && ns <= kFastSegs) ? 1u : 0u;
            for (uint32_t s = 0; rs && s < ns; ++s) {
                if (a.bin_unsorted[static_cast<size_t>(e) * c.nbins + seg_bin[s]]) rs = 0;
                if (s + 1 < ns && seg_g[s + 1] != seg_g[s] + (seg_pos[s + 1] - seg_pos[s])) rs = 0;
            }
            misc[0] = ns;
            misc[1] = rs;
        }
        __syncwarp();
        const uint32_t nseg = misc[0];
        const uint32_t size = seg_pos[nseg];
        MiddleResult r{0, 0, 0, 1};
        if (size <= 65535u) {
            if (misc[1]) {
                const uint32_t base = seg_g[0];
                NbViewT<kNbGlobalRs> nb{a.g_rs + base, nullptr, a.g_rs_gp + base, base,
                                        a.g_xyzr, seg_pos, seg_g, nseg, size};
                r = process_middle<kNbGlobalRs, SCORE, VAR, CAPB, CAPT, CAPLC, CAPCT, GATE>(
                    c, a, nb, gm, false, 0.f, 0.f, e, ws);
            } else {
                NbViewT<kNbHost> nb{nullptr, nullptr, nullptr, 0u, a.g_xyzr, seg_pos, seg_g,
                                    nseg, size};
                r = process_middle<kNbHost, SCORE, VAR, CAPB, CAPT, CAPLC, CAPCT, GATE>(
                    c, a, nb, gm, false, 0.f, 0.f, e, ws);
            }
        }
        if (lane == 0) {
            if (!r.status) {
                count_middle(a, r);
            } else if (LAST) {
                raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
                a.seed_cnt[gm] = 0;
            } else {
                const unsigned long long k = atomicAdd(&a.counters[kOvf2Count], 1ull);
                if (k < 2ull * a.cap_sp) a.ovf2[k] = gm;
                else raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
                a.seed_cnt[gm] = 0;
            }
        }
        __syncwarp();
    }
}

// Middle tier: larger capacities than the fast kernel's, as many warps as fit
// (9 with its 23.4 KiB per warp; the launch bound leaves it the registers).
constexpr int kMidMaxWarps = 10;
template <bool SCORE, bool GATE = false>
__global__ void __launch_bounds__(kMidMaxWarps * 32) k_seed_mid(DevConfig c, Arena a, uint32_t pass) {
    if (a.counters[kAnyVariance] != 0)
        general_middles<SCORE, true, false, 1024, 1024, 512, 256, GATE>(c, a, pass);
    else
        general_middles<SCORE, false, false, 1024, 1024, 512, 256, GATE>(c, a, pass);
}

// Last tier: one warp per CTA with large capacities; always with the
// variance terms (exact for zero variances too; very few middles get here).
template <bool SCORE, bool GATE = false>
__global__ void __launch_bounds__(32) k_seed_slow(DevConfig c, Arena a, uint32_t pass) {
    general_middles<SCORE, true, true, 8192, 8192, 4096, 2048, GATE>(c, a, pass);
}

// Events whose pruned fraction (of all scored doublets) leaves the filter's
// band are marked for the fallback pass.
__global__ void k_filter_mark(DevConfig c, Arena a) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.hdr->n_events) return;
    const uint32_t* f = a.ev_filter + 4 * e;
    const uint32_t scored = f[0] + f[2], pruned = f[1] + f[3];
    uint8_t mode = 0;
    if (scored > 0) {
        const float frac = static_cast<float>(pruned) / static_cast<float>(scored);
        float lo = c.band_lo, hi = c.band_hi;
        if (c.mlp_n_classes) {
            const uint32_t k = filter_class(c, a, e);
            lo = c.mlp_class_band[k][0];
            hi = c.mlp_class_band[k][1];
        }
        mode = (frac < lo || frac > hi) ? 1 : 0;
    }
    a.ev_mode[e] = mode;
    if (mode) atomicAdd(&a.counters[kFallbackEvents], 1ull);
}

// Sum of v over the block (512 threads); every thread gets the total.
__device__ __forceinline__ uint32_t block_sum_512(uint32_t v, uint32_t* sh) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    uint32_t t = lane < (blockDim.x >> 5) ? sh[lane] : 0u;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// Exclusive prefix of v over the block (in thread order); total in *total.
__device__ __forceinline__ uint32_t block_exclusive_512(uint32_t v, uint32_t* sh,
                                                        uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += t;
    }
    __syncthreads();
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < nw ? sh[lane] : 0u;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= static_cast<uint32_t>(o)) wi += t;
        }
        if (lane < nw) sh[lane] = wi - w;
        if (lane == 31) sh[32] = wi;
    }
    __syncthreads();
    *total = sh[32];
    return sh[warp] + incl - v;
}

// Seeds of every chunk of kBinChunk middles (the binning chunks; chunk c of
// an event covers its grid positions sp_base + c kBinChunk onwards).  Also
// sets the seed count of events without spacepoints, which have no chunk.
__global__ void __launch_bounds__(512) k_seed_count(Arena a) {
    __shared__ uint32_t sh[33];
    const BatchHeader hb = *a.hdr;
    if (blockIdx.x < hb.n_events && threadIdx.x == 0) {
        const EventDesc& ev = a.events[blockIdx.x];
        if (ev.n_chunks == 0) *ev.out_size = 0;
    }
    const uint32_t chunk = blockIdx.x;
    if (chunk >= hb.total_chunks) return;
    const uint32_t e = event_of_chunk(a, hb.n_events, chunk);
    const EventDesc ev = a.events[e];
    const uint32_t end = ev.sp_base + a.n_valid[e];
    const uint32_t m0 = ev.sp_base + (chunk - ev.chunk_base) * kBinChunk;
    const uint32_t m1 = min(m0 + kBinChunk, end);
    uint32_t s = 0;
    for (uint32_t i = m0 + threadIdx.x; i < m1; i += blockDim.x) s += a.seed_cnt[i];
    s = block_sum_512(s, sh);
    if (threadIdx.x == 0) a.chunk_seeds[chunk] = s;
}

// The seeds of every event in host order (middles in grid order, each
// middle's seeds in final order) into the caller's buffer: each chunk starts
// after its event's earlier chunks and writes its middles' seeds in rounds
// of one middle per thread.  The event's last chunk with middles (chunk 0
// when it has none) sets the seed count.
__global__ void __launch_bounds__(512) k_seed_compact(Arena a) {
    __shared__ uint32_t sh[33];
    const BatchHeader hb = *a.hdr;
    const uint32_t chunk = blockIdx.x;
    if (chunk >= hb.total_chunks) return;
    const uint32_t e = event_of_chunk(a, hb.n_events, chunk);
    const EventDesc ev = a.events[e];
    const uint32_t nv = a.n_valid[e];
    const uint32_t c = chunk - ev.chunk_base;
    const uint32_t last = nv ? (nv - 1) / kBinChunk : 0u;
    if (c > last) return;
    uint32_t before = 0;
    for (uint32_t k = threadIdx.x; k < c; k += blockDim.x) before += a.chunk_seeds[ev.chunk_base + k];
    uint32_t run = block_sum_512(before, sh);
    const uint32_t m0 = ev.sp_base + c * kBinChunk;
    const uint32_t m1 = min(m0 + kBinChunk, ev.sp_base + nv);
    for (uint32_t r0 = m0; r0 < m1; r0 += blockDim.x) {
        const uint32_t i = r0 + threadIdx.x;
        const uint32_t cnt = i < m1 ? a.seed_cnt[i] : 0u;
        uint32_t round_total;
        uint32_t o = run + block_exclusive_512(cnt, sh, &round_total);
        for (uint32_t k = 0; k < cnt; ++k, ++o) {
            if (o < ev.out_cap) {
                const SeedSlot sl = a.seed_slot[static_cast<size_t>(i) * kMaxSeedsPerMiddle + k];
                ev.out_b[o] = sl.b;
                ev.out_m[o] = sl.m;
                ev.out_t[o] = sl.t;
                ev.out_q[o] = sl.q;
            }
        }
        run += round_total;
    }
    if (c == last && threadIdx.x == 0) {
        *ev.out_size = min(run, ev.out_cap);
        atomicAdd(&a.counters[kNumSeeds], static_cast<unsigned long long>(run));
        if (run > ev.out_cap) raise_status(a.counters, SEEDGB_CAPACITY_OVERFLOW);
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
// Parameters of seed i of one event into out.data[i].
__device__ __forceinline__ void params_of_seed(const ParamsConfig& c, float bx, float by,
                                               float bz, const seedgb_measurement_view& meas,
                                               const seedgb_spacepoint_view& sps,
                                               const seedgb_seed_buffer& seeds,
                                               const seedgb_params_buffer& out, uint32_t i) {
    {
        const uint32_t ib = seeds.bottom_index[i], im = seeds.middle_index[i],
                       it = seeds.top_index[i];
        if (ib >= sps.size || im >= sps.size || it >= sps.size) return;
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
        // A record is 11 16-byte words: on a 16-byte aligned buffer, 11
        // vector stores instead of the 22 of the member-wise copy (the
        // kernel waits on its load/store queue).
        static_assert(sizeof(seedgb_bound_track_parameters) == 11 * sizeof(uint4),
                      "parameter record size");
        if ((reinterpret_cast<uintptr_t>(out.data) & 15u) == 0u) {
            uint4 w[11];
            memcpy(w, &p, sizeof(p));
            uint4* dst = reinterpret_cast<uint4*>(out.data + i);
#pragma unroll
            for (int k = 0; k < 11; ++k) dst[k] = w[k];
        } else {
            out.data[i] = p;
        }
    }
}

__global__ void __launch_bounds__(128)
k_params(ParamsConfig c, float bx, float by, float bz, seedgb_measurement_view meas,
         seedgb_spacepoint_view sps, seedgb_seed_buffer seeds, seedgb_params_buffer out) {
    const uint32_t n = min(*seeds.size, seeds.capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < min(n, out.capacity);
         i += stride)
        params_of_seed(c, bx, by, bz, meas, sps, seeds, out, i);
    if (blockIdx.x == 0 && threadIdx.x == 0) *out.size = min(n, out.capacity);
}

// Many events in one launch: blockIdx.y is the event, the x blocks stride
// over its seeds.
__global__ void __launch_bounds__(128)
k_params_batch(ParamsConfig c, float bx, float by, float bz, const ParamsEvent* events) {
    const ParamsEvent& ev = events[blockIdx.y];
    const uint32_t n = min(*ev.seeds.size, ev.seeds.capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < min(n, ev.out.capacity);
         i += stride)
        params_of_seed(c, bx, by, bz, ev.meas, ev.sps, ev.seeds, ev.out, i);
    if (blockIdx.x == 0 && threadIdx.x == 0) *ev.out.size = min(n, ev.out.capacity);
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

size_t fast_kernel_smem(const TuneParams& tp) {
    return fast_scratch_offset(static_cast<uint32_t>(tp.nb_cap)) +
           static_cast<size_t>(tp.fast_warps) * sizeof(FastScratch);
}

int fast_kernel_max_warps(int nb_cap, int ctas_per_sm) {
    TuneParams t{0, 1, nb_cap, 1};
    const size_t fixed = fast_kernel_smem(t);
    // 228 KiB per SM, of which 1 KiB per resident CTA is reserved; 227 KiB per CTA
    const size_t per_sm = 228 * 1024 / static_cast<size_t>(std::max(1, ctas_per_sm));
    const size_t limit = std::min<size_t>(227 * 1024, per_sm - 1024);
    if (fixed >= limit) return 0;
    return static_cast<int>(std::min<size_t>(16, (limit - fixed) / sizeof(FastScratch)));
}

static size_t slow_kernel_smem() { return general_warp_bytes<SlowScratch>(); }

// Warps per CTA of the general path's middle tier (all that fit in 227 KiB).
static int mid_kernel_warps(bool score) {
    const int fit = static_cast<int>((227 * 1024) / general_warp_bytes<MidScratch>());
    return std::min(std::min(score ? kScoreWarps : 16, kMidMaxWarps), fit);
}
static size_t mid_kernel_smem(bool score) {
    return static_cast<size_t>(mid_kernel_warps(score)) * general_warp_bytes<MidScratch>();
}

cudaError_t prepare_kernels() {
    // per device: the attribute belongs to the current context
    static thread_local int done_for = -1;
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess || dev == done_for) return err;
    for (auto k : {k_seed_fast<false>, k_seed_fast<true>, k_seed_fast<false, true>}) {
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    }
    for (auto k : {k_seed_slow<false>, k_seed_slow<true>, k_seed_slow<false, true>}) {
        if (err == cudaSuccess)
            err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(slow_kernel_smem()));
    }
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(k_seed_mid<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(mid_kernel_smem(false)));
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(k_seed_mid<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(mid_kernel_smem(true)));
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(k_seed_mid<false, true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(mid_kernel_smem(false)));
    if (err == cudaSuccess) done_for = dev;
    return err;
}

cudaError_t launch_seeding(const DevConfig& cfg, const Arena& a, const BatchHeader& grid,
                           const TuneParams& tp, int num_sms, cudaStream_t stream,
                           cudaEvent_t* timing) {
    auto mark = [&](int i) {
        if (timing) cudaEventRecord(timing[i], stream);
    };
    const size_t fsm = fast_kernel_smem(tp);
    const size_t ssm = slow_kernel_smem();
    cudaError_t err = prepare_kernels();
    if (err != cudaSuccess) return err;
    const size_t hsm = static_cast<size_t>(kBinWarps) * cfg.nbins * sizeof(uint32_t);
    mark(0);
    if (grid.total_chunks > 0) {
        k_bin_count<<<grid.total_chunks, kBinWarps * 32, hsm, stream>>>(cfg, a);
    }
    mark(1);
    {
        const uint32_t nb = cfg.nbins;
        const uint32_t G = std::max(1u, 1024u / nb);
        const size_t ssz = (static_cast<size_t>(G) * nb + 2 * nb + 40) * sizeof(uint32_t);
        k_bin_scan<<<grid.n_events, 1024, ssz, stream>>>(cfg, a,
                                                      static_cast<uint32_t>(tp.middles_per_item));
    }
    mark(2);
    k_item_order<<<(a.max_items + 1023) / 1024, 1024, 0, stream>>>(a);
    mark(3);
    if (grid.total_chunks > 0) {
        k_bin_scatter<<<grid.total_chunks, kBinWarps * 32, hsm, stream>>>(cfg, a);
    }
    mark(4);
    k_bin_rsort<<<grid.n_events * cfg.nbins, 256, 0, stream>>>(cfg, a);
    mark(5);
    const uint32_t mpi = static_cast<uint32_t>(tp.middles_per_item);
    const uint32_t nbc = static_cast<uint32_t>(tp.nb_cap);
    const dim3 fgrid(num_sms * tp.ctas_per_sm), fblock(tp.fast_warps * 32);
    // a filter that only gates middles (and records nothing) runs inside the
    // plain routine (GATE instantiation), which keeps the plain kernel's warps
    const bool plain_gate = cfg.mlp && cfg.mlp_prune_top == SEEDGB_FILTER_GATE_MIDDLE &&
                            cfg.mlp_prune_bottom == SEEDGB_FILTER_KEEP && !a.dump && !a.tdump;
    if (plain_gate) {
        k_seed_fast<false, true><<<fgrid, fblock, fsm, stream>>>(cfg, a, mpi, nbc, 0u);
        mark(6);
        k_seed_mid<false, true><<<num_sms, mid_kernel_warps(false) * 32, mid_kernel_smem(false),
                                   stream>>>(cfg, a, 0u);
        mark(7);
        k_seed_slow<false, true><<<num_sms, 32, ssm, stream>>>(cfg, a, 0u);
        // fallback: events whose gated fraction left the band, without the gate
        k_filter_mark<<<(grid.n_events + 255) / 256, 256, 0, stream>>>(cfg, a);
        k_seed_fast<false><<<fgrid, fblock, fsm, stream>>>(cfg, a, mpi, nbc, 1u);
        k_seed_mid<false><<<num_sms, mid_kernel_warps(false) * 32, mid_kernel_smem(false),
                             stream>>>(cfg, a, 1u);
        k_seed_slow<false><<<num_sms, 32, ssm, stream>>>(cfg, a, 1u);
    } else if (cfg.mlp) {
        TuneParams ts = tp;
        ts.fast_warps = std::min(tp.fast_warps, kScoreWarps);
        k_seed_fast<true><<<fgrid, ts.fast_warps * 32, fast_kernel_smem(ts), stream>>>(
            cfg, a, mpi, nbc, 0u);
        mark(6);
        k_seed_mid<true><<<num_sms, mid_kernel_warps(true) * 32, mid_kernel_smem(true), stream>>>(
            cfg, a, 0u);
        mark(7);
        k_seed_slow<true><<<num_sms, 32, ssm, stream>>>(cfg, a, 0u);
        // fallback: events whose pruned fraction left the band, without the filter
        k_filter_mark<<<(grid.n_events + 255) / 256, 256, 0, stream>>>(cfg, a);
        k_seed_fast<false><<<fgrid, fblock, fsm, stream>>>(cfg, a, mpi, nbc, 1u);
        k_seed_mid<false><<<num_sms, mid_kernel_warps(false) * 32, mid_kernel_smem(false),
                             stream>>>(cfg, a, 1u);
        k_seed_slow<false><<<num_sms, 32, ssm, stream>>>(cfg, a, 1u);
    } else {
        k_seed_fast<false><<<fgrid, fblock, fsm, stream>>>(cfg, a, mpi, nbc, 0u);
        mark(6);
        k_seed_mid<false><<<num_sms, mid_kernel_warps(false) * 32, mid_kernel_smem(false),
                             stream>>>(cfg, a, 0u);
        mark(7);
        k_seed_slow<false><<<num_sms, 32, ssm, stream>>>(cfg, a, 0u);
    }
    mark(8);
    k_seed_count<<<std::max(std::max(grid.total_chunks, grid.n_events), 1u), 512, 0, stream>>>(a);
    mark(9);
    k_seed_compact<<<std::max(grid.total_chunks, 1u), 512, 0, stream>>>(a);
    mark(10);
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

cudaError_t launch_params_batch(const ParamsConfig& cfg, const float bfield[3],
                                const ParamsEvent* events, uint32_t n_events, int num_sms,
                                cudaStream_t stream) {
    if (n_events == 0) return cudaSuccess;
    // about one seed per thread for 100k-spacepoint events: the kernel waits
    // on its global loads, so many warps per SM pay (64 blocks of 128 per SM
    // over all events; 15 % faster than 4)
    const uint32_t gx = std::max(1u, (static_cast<uint32_t>(num_sms) * 64 + n_events - 1) / n_events);
    k_params_batch<<<dim3(gx, n_events), 128, 0, stream>>>(cfg, bfield[0], bfield[1], bfield[2],
                                                           events);
    return cudaGetLastError();
}

}  // namespace seedgb
