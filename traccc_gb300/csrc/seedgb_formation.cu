// Spacepoint formation: measurements on their surfaces -> spacepoints, the
// step in front of the seeding path.  Stable (measurement-order) compaction
// in three launches: per-block counts, one scan of the block counts, and the
// scattered write.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "seedgb.h"

namespace {

constexpr int kFormThreads = 1024;

struct DevSurface {
    uint32_t type;
    float radius;
    float rot[9];
    float t[3];
};
static_assert(sizeof(DevSurface) == sizeof(seedgb_surface), "surface layout");

__device__ __forceinline__ bool formable(const seedgb_measurement_view& m, const uint8_t* dims,
                                         uint32_t n_surfaces, uint32_t i) {
    return (dims == nullptr || dims[i] == 2u) && m.surface_link[i] < n_surfaces;
}

__global__ void __launch_bounds__(kFormThreads)
k_form_count(seedgb_measurement_view m, const uint8_t* dims, uint32_t n_surfaces,
             uint32_t* block_counts) {
    __shared__ uint32_t warp_sum[32];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = i < m.size && formable(m, dims, n_surfaces, i);
    const uint32_t c = __popc(__ballot_sync(0xffffffffu, ok));
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = threadIdx.x < blockDim.x / 32 ? warp_sum[threadIdx.x] : 0u;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) block_counts[blockIdx.x] = v;
    }
}

// One block: exclusive scan of the block counts (in place), total to n_out.
__device__ __forceinline__ void k_form_scan_body(uint32_t* block_counts, uint32_t n_blocks,
                                                 uint32_t* n_out) {
    __shared__ uint32_t warp_sum[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n_blocks; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < n_blocks ? block_counts[i] : 0u;
        uint32_t incl = v;
        const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += x;
        }
        if (lane == 31) warp_sum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = warp_sum[lane];
            uint32_t wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t x = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= static_cast<uint32_t>(o)) wi += x;
            }
            warp_sum[lane] = wi - w;
        }
        __syncthreads();
        const uint32_t c0 = carry;
        if (i < n_blocks) block_counts[i] = c0 + warp_sum[warp] + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = c0 + warp_sum[warp] + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *n_out = carry;
}

__global__ void __launch_bounds__(kFormThreads)
k_form_scan(uint32_t* block_counts, uint32_t n_blocks, uint32_t* n_out) {
    k_form_scan_body(block_counts, n_blocks, n_out);
}

// Spacepoint k from measurement i (silicon_pixel_spacepoint_formation.hpp:
// 31-60 with the surface's local_to_global).
__device__ __forceinline__ void form_one(const DevSurface* __restrict__ surf,
                                         const seedgb_measurement_view& m, uint32_t i, uint32_t k,
                                         uint32_t* mi1, uint32_t* mi2, float* global, float* zvar,
                                         float* rvar) {
    const DevSurface S = surf[m.surface_link[i]];
    const float l0 = m.local_position[2 * i], l1 = m.local_position[2 * i + 1];
    float a, b, c;
    if (S.type == 1u) {
        // detray cylinder2D: local (r phi, z) -> (r cos phi, r sin phi, z)
        const double phi = static_cast<double>(l0) / static_cast<double>(S.radius);
        a = S.radius * static_cast<float>(cos(phi));
        b = S.radius * static_cast<float>(sin(phi));
        c = l1;
    } else {
        a = l0;
        b = l1;
        c = 0.f;
    }
    float g[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) g[r] = (S.rot[3 * r] * a + S.rot[3 * r + 1] * b) + S.rot[3 * r + 2] * c + S.t[r];
    mi1[k] = i;
    mi2[k] = SEEDGB_INVALID_MEASUREMENT_INDEX;
    global[3 * k] = g[0];
    global[3 * k + 1] = g[1];
    global[3 * k + 2] = g[2];
    zvar[k] = 0.f;
    rvar[k] = 0.f;
}

__global__ void __launch_bounds__(kFormThreads)
k_form_write(const DevSurface* __restrict__ surf, uint32_t n_surfaces,
             seedgb_measurement_view m, const uint8_t* dims, const uint32_t* block_offsets,
             uint32_t* mi1, uint32_t* mi2, float* global, float* zvar, float* rvar) {
    __shared__ uint32_t warp_off[32];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool ok = i < m.size && formable(m, dims, n_surfaces, i);
    const uint32_t mask = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) warp_off[warp] = __popc(mask);
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < blockDim.x / 32 ? warp_off[lane] : 0u;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= static_cast<uint32_t>(o)) wi += x;
        }
        warp_off[lane] = wi - w;
    }
    __syncthreads();
    if (!ok) return;
    const uint32_t k = block_offsets[blockIdx.x] + warp_off[warp] +
                       __popc(mask & ((1u << lane) - 1u));
    form_one(surf, m, i, k, mi1, mi2, global, zvar, rvar);
}

// ---------------------------------------------------------------------------
// Many events in one launch sequence (seedgb_formation_run_batch): the same
// three steps over the blocks of all events, each block owning 1024
// measurements of one event; block b belongs to the event e with
// block0[e] <= b < block0[e] + n_blocks[e].
// ---------------------------------------------------------------------------

struct FormEvent {
    seedgb_measurement_view meas;
    const uint8_t* dims;
    seedgb_spacepoint_buffer out;
    uint32_t block0, n_blocks;
};

__device__ __forceinline__ uint32_t event_of_block(const FormEvent* ev, uint32_t n_events,
                                                   uint32_t b) {
    uint32_t lo = 0, hi = n_events - 1;
    while (lo < hi) {  // last event with block0 <= b
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (ev[mid].block0 <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kFormThreads)
k_form_count_batch(const FormEvent* ev, uint32_t n_events, uint32_t n_surfaces,
                   uint32_t* block_counts) {
    __shared__ uint32_t warp_sum[32];
    const uint32_t e = event_of_block(ev, n_events, blockIdx.x);
    const FormEvent& E = ev[e];
    const uint32_t i = (blockIdx.x - E.block0) * blockDim.x + threadIdx.x;
    const bool ok = i < E.meas.size && formable(E.meas, E.dims, n_surfaces, i);
    const uint32_t c = __popc(__ballot_sync(0xffffffffu, ok));
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = threadIdx.x < blockDim.x / 32 ? warp_sum[threadIdx.x] : 0u;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) block_counts[blockIdx.x] = v;
    }
}

// One block per event: exclusive scan of the event's block counts, the
// event's count to its output size.
__global__ void __launch_bounds__(kFormThreads)
k_form_scan_batch(const FormEvent* ev, uint32_t* block_counts) {
    const FormEvent& E = ev[blockIdx.x];
    k_form_scan_body(block_counts + E.block0, E.n_blocks, E.out.size);
}

__global__ void __launch_bounds__(kFormThreads)
k_form_write_batch(const DevSurface* __restrict__ surf, uint32_t n_surfaces, const FormEvent* ev,
                   uint32_t n_events, const uint32_t* block_offsets) {
    __shared__ uint32_t warp_off[32];
    const uint32_t e = event_of_block(ev, n_events, blockIdx.x);
    const FormEvent& E = ev[e];
    const uint32_t i = (blockIdx.x - E.block0) * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool ok = i < E.meas.size && formable(E.meas, E.dims, n_surfaces, i);
    const uint32_t mask = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) warp_off[warp] = __popc(mask);
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < blockDim.x / 32 ? warp_off[lane] : 0u;
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= static_cast<uint32_t>(o)) wi += x;
        }
        warp_off[lane] = wi - w;
    }
    __syncthreads();
    if (!ok) return;
    const uint32_t k = block_offsets[blockIdx.x] + warp_off[warp] +
                       __popc(mask & ((1u << lane) - 1u));
    form_one(surf, E.meas, i, k, E.out.measurement_index_1, E.out.measurement_index_2,
             E.out.global, E.out.z_variance, E.out.radius_variance);
}

// Per-thread scratch for the block counts and the surface table, grown as
// needed (one stream per host thread, as for the seeding handles).
struct FormScratch {
    void* p = nullptr;
    size_t bytes = 0;
    int device = -1;
    ~FormScratch() {
        if (p) cudaFree(p);
    }
};

}  // namespace

extern "C" seedgb_status seedgb_form_spacepoints(const seedgb_surface* surfaces_host,
                                                 uint32_t n_surfaces,
                                                 const seedgb_measurement_view* meas,
                                                 const uint8_t* dimensions, uint32_t* mi1,
                                                 uint32_t* mi2, float* global, float* zvar,
                                                 float* rvar, uint32_t* n_out, void* stream) {
    if (!meas || !n_out || (n_surfaces && !surfaces_host)) return SEEDGB_INVALID_ARGUMENT;
    if (meas->size && (!meas->local_position || !meas->surface_link || !mi1 || !mi2 ||
                       !global || !zvar || !rvar))
        return SEEDGB_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (meas->size == 0)
        return cudaMemsetAsync(n_out, 0, sizeof(uint32_t), s) == cudaSuccess ? SEEDGB_OK
                                                                              : SEEDGB_CUDA_ERROR;
    static thread_local FormScratch scratch;
    const uint32_t n_blocks = (meas->size + kFormThreads - 1) / kFormThreads;
    const size_t surf_bytes = sizeof(DevSurface) * n_surfaces;
    const size_t need = ((surf_bytes + 255) / 256) * 256 + sizeof(uint32_t) * n_blocks;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    if (scratch.bytes < need || scratch.device != dev) {
        // the previous scratch may still be in use by work on any stream
        if (scratch.p && (cudaDeviceSynchronize() != cudaSuccess)) return SEEDGB_CUDA_ERROR;
        if (scratch.p) cudaFree(scratch.p);
        scratch.p = nullptr;
        scratch.bytes = 0;
        if (cudaMalloc(&scratch.p, need) != cudaSuccess) return SEEDGB_CUDA_ERROR;
        scratch.bytes = need;
        scratch.device = dev;
    }
    DevSurface* d_surf = static_cast<DevSurface*>(scratch.p);
    uint32_t* d_counts =
        reinterpret_cast<uint32_t*>(static_cast<char*>(scratch.p) + ((surf_bytes + 255) / 256) * 256);
    cudaError_t err = cudaSuccess;
    if (n_surfaces)
        err = cudaMemcpyAsync(d_surf, surfaces_host, surf_bytes, cudaMemcpyHostToDevice, s);
    if (err != cudaSuccess) return SEEDGB_CUDA_ERROR;
    k_form_count<<<n_blocks, kFormThreads, 0, s>>>(*meas, dimensions, n_surfaces, d_counts);
    k_form_scan<<<1, kFormThreads, 0, s>>>(d_counts, n_blocks, n_out);
    k_form_write<<<n_blocks, kFormThreads, 0, s>>>(d_surf, n_surfaces, *meas, dimensions, d_counts,
                                                   mi1, mi2, global, zvar, rvar);
    if (cudaGetLastError() != cudaSuccess) return SEEDGB_CUDA_ERROR;
    // the surface copy reads surfaces_host: finish it before returning
    return cudaStreamSynchronize(s) == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}

// ---------------------------------------------------------------------------
// Formation handle: the surface table resident on the device, event
// descriptors staged through two pinned slots used in turn.
// ---------------------------------------------------------------------------

namespace {

struct FormSlot {
    FormEvent* host = nullptr;
    FormEvent* dev = nullptr;
    uint32_t cap = 0;
    cudaEvent_t copied = nullptr;
};

}  // namespace

struct seedgb_formation {
    DevSurface* surf = nullptr;
    uint32_t n_surfaces = 0;
    uint32_t* counts = nullptr;
    uint32_t counts_cap = 0;
    FormSlot slot[2];
    int next = 0;
    ~seedgb_formation() {
        cudaDeviceSynchronize();
        for (auto& sl : slot) {
            if (sl.copied) cudaEventDestroy(sl.copied);
            if (sl.host) cudaFreeHost(sl.host);
            if (sl.dev) cudaFree(sl.dev);
        }
        if (surf) cudaFree(surf);
        if (counts) cudaFree(counts);
    }
};

extern "C" seedgb_status seedgb_formation_create(const seedgb_surface* surfaces_host,
                                                 uint32_t n_surfaces, seedgb_formation** out) {
    if (!out || (n_surfaces && !surfaces_host)) return SEEDGB_INVALID_ARGUMENT;
    *out = nullptr;
    seedgb_formation* h = new seedgb_formation();
    h->n_surfaces = n_surfaces;
    if (n_surfaces &&
        (cudaMalloc(&h->surf, sizeof(DevSurface) * n_surfaces) != cudaSuccess ||
         cudaMemcpy(h->surf, surfaces_host, sizeof(DevSurface) * n_surfaces,
                    cudaMemcpyHostToDevice) != cudaSuccess)) {
        delete h;
        return SEEDGB_CUDA_ERROR;
    }
    *out = h;
    return SEEDGB_OK;
}

extern "C" seedgb_status seedgb_formation_destroy(seedgb_formation* h) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    delete h;
    return SEEDGB_OK;
}

extern "C" seedgb_status seedgb_formation_run_batch(seedgb_formation* h,
                                                    const seedgb_measurement_view* meas,
                                                    const uint8_t* const* dimensions,
                                                    seedgb_spacepoint_buffer* outs,
                                                    uint32_t n_events, void* stream) {
    if (!h || (n_events && (!meas || !outs))) return SEEDGB_INVALID_ARGUMENT;
    if (n_events == 0) return SEEDGB_OK;
    if (n_events > 65535u) return SEEDGB_SIZE_LIMIT;
    uint64_t blocks = 0;
    for (uint32_t e = 0; e < n_events; ++e) {
        const seedgb_measurement_view& m = meas[e];
        const seedgb_spacepoint_buffer& o = outs[e];
        if (!o.size || o.capacity < m.size) return SEEDGB_INVALID_ARGUMENT;
        if (m.size && (!m.local_position || !m.surface_link || !o.measurement_index_1 ||
                       !o.measurement_index_2 || !o.global || !o.z_variance ||
                       !o.radius_variance))
            return SEEDGB_INVALID_ARGUMENT;
        blocks += (m.size + kFormThreads - 1) / kFormThreads;
    }
    if (blocks > 0x7fffffffull) return SEEDGB_SIZE_LIMIT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    FormSlot& sl = h->slot[h->next];
    // the previous copy out of this slot's pinned descriptors must be done
    if (sl.copied && cudaEventSynchronize(sl.copied) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    const uint32_t nb = static_cast<uint32_t>(blocks);
    if (sl.cap < n_events || h->counts_cap < nb) {
        // in-flight launches may still read the old descriptors and counts
        if (cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
    }
    if (sl.cap < n_events) {
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.dev) cudaFree(sl.dev);
        sl.host = nullptr;
        sl.dev = nullptr;
        sl.cap = 0;
        const uint32_t cap = n_events > 64u ? n_events : 64u;
        if (cudaMallocHost(reinterpret_cast<void**>(&sl.host), sizeof(FormEvent) * cap) !=
                cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&sl.dev), sizeof(FormEvent) * cap) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
        sl.cap = cap;
    }
    if (h->counts_cap < nb) {
        if (h->counts) cudaFree(h->counts);
        h->counts = nullptr;
        h->counts_cap = 0;
        const uint32_t cap = nb > 1024u ? nb + nb / 4 : 1024u;
        if (cudaMalloc(reinterpret_cast<void**>(&h->counts), sizeof(uint32_t) * cap) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
        h->counts_cap = cap;
    }
    if (!sl.copied && cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    uint32_t b0 = 0;
    for (uint32_t e = 0; e < n_events; ++e) {
        const uint32_t n = (meas[e].size + kFormThreads - 1) / kFormThreads;
        sl.host[e] = FormEvent{meas[e], dimensions ? dimensions[e] : nullptr, outs[e], b0, n};
        b0 += n;
    }
    if (cudaMemcpyAsync(sl.dev, sl.host, sizeof(FormEvent) * n_events, cudaMemcpyHostToDevice, s) !=
            cudaSuccess ||
        cudaEventRecord(sl.copied, s) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    h->next ^= 1;
    if (nb) k_form_count_batch<<<nb, kFormThreads, 0, s>>>(sl.dev, n_events, h->n_surfaces, h->counts);
    k_form_scan_batch<<<n_events, kFormThreads, 0, s>>>(sl.dev, h->counts);
    if (nb)
        k_form_write_batch<<<nb, kFormThreads, 0, s>>>(h->surf, h->n_surfaces, sl.dev, n_events,
                                                       h->counts);
    return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}
