// Phi-z grid binning that allocates nothing.
//
// Some callers cannot allocate device memory when they bin spacepoints: code
// running while a CUDA stream is being captured into a graph (cudaMalloc is
// not permitted there), trigger and online-reconstruction processes that
// reserve all device memory once at start-up and forbid allocation on the
// event path, and plugins of frameworks that own every device allocation.
// seedgb_spacepoint_binning_noalloc serves them: the caller passes the input
// and output buffers, and the kernel's scratch memory is a fixed array in this
// library's device image (SEEDGB_NOALLOC_SCRATCH_BYTES per GPU, held by every
// GPU that loads the library until the process exits).
//
// The result is the same grid as seedgb_seeding_copy_grid returns for the
// seeding path (the reference's spacepoint_binning output).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "seedgb.h"
#include "seedgb_device.cuh"
#include "seedgb_internal.h"

namespace seedgb {
namespace {

constexpr uint32_t kNoallocWarps = 32;

// Scratch of the allocation-free binning: a status word block (256 bytes),
// the grid bin of every spacepoint (int32, SEEDGB_NOALLOC_MAX_SPACEPOINTS),
// then per-warp bin histograms (uint32, kNoallocWarps x kMaxBins) that become
// per-warp scatter offsets.
constexpr size_t kNoallocStatusBytes = 256;
constexpr size_t kNoallocBinBytes = sizeof(int32_t) * SEEDGB_NOALLOC_MAX_SPACEPOINTS;
constexpr size_t kNoallocHistBytes = sizeof(uint32_t) * kNoallocWarps * kMaxBins;
static_assert(kNoallocStatusBytes + kNoallocBinBytes + kNoallocHistBytes ==
                  SEEDGB_NOALLOC_SCRATCH_BYTES,
              "scratch size stated in seedgb.h");

static __device__ __align__(256) uint8_t g_noalloc_scratch[SEEDGB_NOALLOC_SCRATCH_BYTES];

// One CTA of kNoallocWarps warps bins one event.  Warp w owns the contiguous
// spacepoints [w L, (w+1) L), so a stable scatter per warp keeps every bin in
// ascending spacepoint order, as the reference's host binning loop does
// (core/src/seeding/spacepoint_binning.cpp:39-51).
__global__ void __launch_bounds__(kNoallocWarps * 32)
k_bin_noalloc(DevConfig c, seedgb_spacepoint_view sps, uint8_t* scratch,
              uint32_t* bin_offsets, uint32_t* bin_sps) {
    __shared__ uint32_t tmp[33];
    // classify()'s status words and counters (the host has already rejected
    // grids that cannot place every phi the finder accepts, so no status bit
    // is raised here); cleared on every call so nothing accumulates
    unsigned long long* status = reinterpret_cast<unsigned long long*>(scratch);
    int32_t* sp_bin = reinterpret_cast<int32_t*>(scratch + kNoallocStatusBytes);
    uint32_t* whist =
        reinterpret_cast<uint32_t*>(scratch + kNoallocStatusBytes + kNoallocBinBytes);
    const uint32_t nb = c.nbins;
    const uint32_t n = sps.size;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t L = (n + kNoallocWarps - 1) / kNoallocWarps;
    const uint32_t i0 = min(n, warp * L), i1 = min(n, i0 + L);

    // the status block and the histograms keep the previous call's contents:
    // clear them (classify() runs only after the barrier)
    if (threadIdx.x < kNoallocStatusBytes / sizeof(unsigned long long)) status[threadIdx.x] = 0;
    for (uint32_t i = threadIdx.x; i < kNoallocWarps * nb; i += blockDim.x) whist[i] = 0;
    __syncthreads();
    uint32_t* wh = whist + warp * nb;
    for (uint32_t base = i0; base < i1; base += 32) {
        const uint32_t i = base + lane;
        int32_t bin = -1;
        if (i < i1) {
            bin = classify(c, sps.global[3 * i], sps.global[3 * i + 1], sps.global[3 * i + 2],
                           status);
            sp_bin[i] = bin;
        }
        if (bin >= 0) atomicAdd(&wh[bin], 1u);
    }
    __syncthreads();

    // bin totals, bin starts, then absolute per-warp offsets (bin-major)
    const uint32_t per = (nb + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = min(nb, threadIdx.x * per), b1 = min(nb, b0 + per);
    uint32_t s = 0;
    for (uint32_t b = b0; b < b1; ++b)
        for (uint32_t w = 0; w < kNoallocWarps; ++w) s += whist[w * nb + b];
    uint32_t incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += v;
    }
    if (lane == 31) tmp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t v = tmp[lane];
        uint32_t wi = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= static_cast<uint32_t>(o)) wi += t;
        }
        tmp[lane] = wi - v;
        if (lane == 31) tmp[32] = wi;
    }
    __syncthreads();
    uint32_t run = tmp[warp] + incl - s;
    for (uint32_t b = b0; b < b1; ++b) {
        bin_offsets[b] = run;
        for (uint32_t w = 0; w < kNoallocWarps; ++w) {
            const uint32_t v = whist[w * nb + b];
            whist[w * nb + b] = run;
            run += v;
        }
    }
    if (threadIdx.x == 0) bin_offsets[nb] = tmp[32];
    __syncthreads();

    // stable scatter: each warp walks its spacepoints in order
    const uint32_t lt = lanemask_lt();
    for (uint32_t base = i0; base < i1; base += 32) {
        const uint32_t i = base + lane;
        const int32_t bin = (i < i1) ? sp_bin[i] : -1;
        const uint32_t peers = __match_any_sync(0xffffffffu, bin);
        const uint32_t rank = __popc(peers & lt);
        if (bin >= 0) bin_sps[wh[bin] + rank] = i;
        __syncwarp();
        if (bin >= 0 && rank == 0) wh[bin] += __popc(peers);
        __syncwarp();
    }
}

// Device address of the scratch array per device (at most 64 devices).  It is
// looked up again on every call made outside stream capture, so a context
// that was reset and created again gets the new address; during capture the
// address of the last call outside capture on this device is used.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

seedgb_status scratch_address(cudaStream_t stream, void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    if (dev < 0 || dev >= kMaxDevices) return SEEDGB_UNSUPPORTED;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    std::lock_guard<std::mutex> lock(g_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
            return SEEDGB_CUDA_ERROR;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return SEEDGB_OK;
}

// True when the grid's circular phi axis can place every phi the finder
// accepts.  The axis maps phi to ibin = int((phi - min) / (max - min) * n)
// and wraps ibin in [-n, 2n) (core/include/traccc/seeding/grids/axis.hpp:
// 277-289); ibin is monotone in phi, so the two ends of the finder's range
// (clipped to atan2f's range) decide.  A narrower grid would leave
// spacepoints out of the grid (the handle path reports that case as
// SEEDGB_BAD_CONFIG after the fact; this entry point refuses it up front).
bool grid_places_finder_phi(const seedgb_seedfinder_config& f, const seedgb_grid_axes& ax) {
    const float pi_f = 3.14159274f;  // the float nearest pi: atan2f's extreme
    const float lo = f.phiMin > -pi_f ? f.phiMin : -pi_f;
    const float hi = f.phiMax < pi_f ? f.phiMax : pi_f;
    if (!(lo <= hi)) return lo > hi;  // no phi accepted (or NaN limits: refuse)
    const float n = static_cast<float>(ax.phi_bins);
    for (const float phi : {lo, hi}) {
        const float v = (phi - ax.phi_min) / (ax.phi_max - ax.phi_min) * n;
        // int(v) in [-n, 2n)  <=>  -n - 1 < v < 2n  (truncation toward zero)
        if (!(v > -n - 1.f && v < 2.f * n)) return false;
    }
    return true;
}

}  // namespace
}  // namespace seedgb

using namespace seedgb;

extern "C" seedgb_status seedgb_spacepoint_binning_noalloc(
    const seedgb_seedfinder_config* finder, const seedgb_spacepoint_grid_config* grid,
    const seedgb_spacepoint_view* sps, uint32_t* bin_offsets, uint32_t* bin_sps,
    void* stream) {
    if (!finder || !grid || !sps || !bin_offsets) return SEEDGB_INVALID_ARGUMENT;
    if (sps->size > SEEDGB_NOALLOC_MAX_SPACEPOINTS) return SEEDGB_SIZE_LIMIT;
    if (sps->size > 0 && (!sps->global || !bin_sps)) return SEEDGB_INVALID_ARGUMENT;
    seedgb_grid_axes ax;
    const seedgb_status st = seedgb_get_axes(grid, &ax);
    if (st != SEEDGB_OK) return st;
    const uint64_t nbins = static_cast<uint64_t>(ax.phi_bins) * ax.z_bins;
    if (ax.phi_bins == 0 || nbins > static_cast<uint64_t>(kMaxBins)) return SEEDGB_SIZE_LIMIT;
    if (!grid_places_finder_phi(*finder, ax)) return SEEDGB_BAD_CONFIG;
    void* scratch = nullptr;
    const seedgb_status sst = scratch_address(static_cast<cudaStream_t>(stream), &scratch);
    if (sst != SEEDGB_OK) return sst;
    seedgb_seedfilter_config flt;
    seedgb_seedfilter_config_default(&flt);
    const DevConfig dc = make_dev_config(*finder, flt, ax);
    k_bin_noalloc<<<1, kNoallocWarps * 32, 0, static_cast<cudaStream_t>(stream)>>>(
        dc, *sps, static_cast<uint8_t*>(scratch), bin_offsets, bin_sps);
    return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}
