// Hand-off of the estimated track parameters to the combinatorial Kalman
// filter: the library's parameter records (surface link, 6 parameters,
// row-major covariance) rewritten on the device as the record the
// reference's track finding takes (detray's bound_track_parameters over the
// array algebra: parameter vector, surface barcode, column-major covariance;
// seedgb_ckf_bound_track_parameters in seedgb.h).  The reference feeds
// seed_parameter_estimation_algorithm's buffer straight into
// combinatorial_kalman_filter_algorithm
// (examples/run/cuda/src/full_chain_algorithm.cpp:241-247).
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "seedgb.h"

namespace {

static_assert(sizeof(seedgb_bound_track_parameters) == 176, "input record");
static_assert(sizeof(seedgb_ckf_bound_track_parameters) == 176, "output record");
static_assert(offsetof(seedgb_ckf_bound_track_parameters, barcode) == 24, "barcode offset");
static_assert(offsetof(seedgb_ckf_bound_track_parameters, covariance) == 32, "cov offset");

constexpr int kWords = 11;  // 176-byte records as 16-byte words

// One record per thread: eleven 16-byte loads, the first two words
// permuted (link | p0 p1 | p2 p3 | p4 p5  ->  p0..p5 | link), the
// covariance transposed in registers (row-major -> array of columns), eleven
// 16-byte stores.  HBM-bound: 352 bytes moved per record.
__global__ void __launch_bounds__(128)
k_params_to_ckf(const uint4* __restrict__ in, const uint32_t* __restrict__ in_size,
                uint32_t in_capacity, uint4* __restrict__ out, uint32_t capacity,
                uint32_t* out_size) {
    const uint32_t n = min(min(*in_size, in_capacity), capacity);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint4* src = in + static_cast<size_t>(i) * kWords;
        uint4 w[kWords];
#pragma unroll
        for (int k = 0; k < kWords; ++k) w[k] = src[k];
        // words 0-1: link (x, y), p0 p1 (z, w) | p2 p3 p4 p5
        const uint4 v0 = make_uint4(w[0].z, w[0].w, w[1].x, w[1].y);  // p0 p1 p2 p3
        const uint4 v1 = make_uint4(w[1].z, w[1].w, w[0].x, w[0].y);  // p4 p5 link
        uint32_t c[36], t[36];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            c[4 * k] = w[2 + k].x;
            c[4 * k + 1] = w[2 + k].y;
            c[4 * k + 2] = w[2 + k].z;
            c[4 * k + 3] = w[2 + k].w;
        }
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
            for (int col = 0; col < 6; ++col) t[col * 6 + r] = c[r * 6 + col];
        uint4* dst = out + static_cast<size_t>(i) * kWords;
        dst[0] = v0;
        dst[1] = v1;
#pragma unroll
        for (int k = 0; k < 9; ++k)
            dst[2 + k] = make_uint4(t[4 * k], t[4 * k + 1], t[4 * k + 2], t[4 * k + 3]);
    }
    if (out_size && blockIdx.x == 0 && threadIdx.x == 0) *out_size = n;
}

}  // namespace

extern "C" seedgb_status seedgb_params_to_ckf(const seedgb_params_buffer* in,
                                              seedgb_ckf_bound_track_parameters* out,
                                              uint32_t capacity, uint32_t* out_size,
                                              void* stream) {
    if (!in || !in->size || (in->capacity && !in->data) || (capacity && !out))
        return SEEDGB_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(in->data) | reinterpret_cast<uintptr_t>(out)) % 16)
        return SEEDGB_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    const uint32_t need = (capacity + 127u) / 128u;
    const uint32_t blocks = need < static_cast<uint32_t>(sms) * 8u ? (need ? need : 1u)
                                                                   : static_cast<uint32_t>(sms) * 8u;
    k_params_to_ckf<<<blocks, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const uint4*>(in->data), in->size, in->capacity,
        reinterpret_cast<uint4*>(out), capacity, out_size);
    return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}
