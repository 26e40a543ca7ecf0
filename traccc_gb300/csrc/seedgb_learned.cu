// Training and stand-alone inference of the learned doublet filter's network
// (MLP 8 -> 32 -> 32 -> 1, bf16 operands, fp32 accumulate on the tensor cores
// with mma.sync m16n8k16).  No counterpart in the reference.
//
// Forward numerics are those of seedgb_mlp.cuh (the seeding kernel's filter
// runs the same tile function).  The backward pass of the weighted logistic
// loss L = -(p y log s(z) + (1 - y) log(1 - s(z))) / n, per 16-sample tile:
//   g3  = dL/dz3 (fp32),                       db3 = sum g3
//   dz2 = g3 * w3 * [z2 > 0] (fp32),            db2 = sum dz2
//   dW3 = h2^T bf16(g3)           (tensor cores)
//   dW2 = h1^T bf16(dz2)          (tensor cores)
//   dz1 = (bf16(dz2) W2^T) * [z1 > 0],          db1 = sum dz1
//   dW1 = x^T bf16(dz1)           (tensor cores)
// with w3, W2 the bf16-rounded weights of the forward pass.  Per-warp fp32
// accumulators are reduced per CTA in shared memory and then into the global
// gradient with atomics (summation order is not fixed).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "seedgb.h"
#include "seedgb_internal.h"
#include "seedgb_mlp.cuh"

namespace seedgb {
namespace {

constexpr int kTrainWarps = 8;
constexpr int kGradRow = kMlpParams + 3;  // gradient, loss, padding to 16 bytes

// Packs the bf16 B fragments of the forward pass from the fp32 parameters.
__device__ void build_frag(MlpFrag& f, const float* __restrict__ P, const float* __restrict__ norm) {
    const uint32_t tid = threadIdx.x, nt_ = blockDim.x;
    for (uint32_t i = tid; i < 4 * 32; i += nt_) {
        const uint32_t nt = i >> 5, lane = i & 31, g = lane >> 2, t = lane & 3;
        const uint32_t col = nt * 8 + g;
        f.w1[nt][lane] = make_uint2(pack_bf16(P[kOffW1 + (2 * t) * kMlpH + col],
                                              P[kOffW1 + (2 * t + 1) * kMlpH + col]),
                                    0u);
    }
    for (uint32_t i = tid; i < 2 * 4 * 32; i += nt_) {
        const uint32_t ks = i >> 7, nt = (i >> 5) & 3, lane = i & 31, g = lane >> 2, t = lane & 3;
        const uint32_t col = nt * 8 + g, k0 = ks * 16 + 2 * t;
        f.w2[ks][nt][lane] = make_uint2(
            pack_bf16(P[kOffW2 + k0 * kMlpH + col], P[kOffW2 + (k0 + 1) * kMlpH + col]),
            pack_bf16(P[kOffW2 + (k0 + 8) * kMlpH + col], P[kOffW2 + (k0 + 9) * kMlpH + col]));
    }
    for (uint32_t i = tid; i < 2 * 32; i += nt_) {
        const uint32_t ks = i >> 5, lane = i & 31, g = lane >> 2, t = lane & 3;
        const uint32_t k0 = ks * 16 + 2 * t;
        f.w3[ks][lane] = g == 0 ? make_uint2(pack_bf16(P[kOffW3 + k0], P[kOffW3 + k0 + 1]),
                                             pack_bf16(P[kOffW3 + k0 + 8], P[kOffW3 + k0 + 9]))
                                : make_uint2(0u, 0u);
    }
    for (uint32_t i = tid; i < kMlpH; i += nt_) {
        f.b1[i] = P[kOffB1 + i];
        f.b2[i] = P[kOffB2 + i];
    }
    for (uint32_t i = tid; i < kMlpIn; i += nt_) {
        f.mu[i] = norm[i];
        f.isd[i] = norm[kMlpIn + i];
    }
    if (tid == 0) {
        f.b3 = P[kOffB3];
        f.n_edges = 0;
        f.threshold[0] = f.threshold[1] = 0.f;
        f.prune_bottom = f.prune_top = 0;
    }
}

// Packed standardised inputs of row `row` (zero past n).
__device__ __forceinline__ void load_row(const MlpFrag& f, const float* __restrict__ feat,
                                         uint32_t n, uint64_t row, uint32_t (&p)[4]) {
    if (row < n) {
        float x[kMlpIn];
        const float4* src = reinterpret_cast<const float4*>(feat + row * kMlpIn);
        const float4 u = src[0], v = src[1];
        x[0] = u.x; x[1] = u.y; x[2] = u.z; x[3] = u.w;
        x[4] = v.x; x[5] = v.y; x[6] = v.z; x[7] = v.w;
        mlp_pack_inputs(f.mu, f.isd, x, p);
    } else {
        p[0] = p[1] = p[2] = p[3] = 0u;
    }
}

__global__ void __launch_bounds__(kTrainWarps * 32)
k_mlp_forward(const float* __restrict__ P, const float* __restrict__ norm,
              const float* __restrict__ feat, uint32_t n, float* __restrict__ logits) {
    __shared__ MlpFrag f;
    __shared__ uint32_t xs[kTrainWarps][16 * 4];
    build_frag(f, P, norm);
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tiles = (n + 15) / 16;
    for (uint32_t tile = blockIdx.x * kTrainWarps + warp; tile < tiles;
         tile += gridDim.x * kTrainWarps) {
        if (lane < 16) {
            uint32_t p[4];
            load_row(f, feat, n, static_cast<uint64_t>(tile) * 16 + lane, p);
#pragma unroll
            for (int i = 0; i < 4; ++i) xs[warp][4 * lane + i] = p[i];
        }
        __syncwarp();
        float lo, hi;
        mlp_tile16(f, xs[warp], lane, lo, hi);
        if ((lane & 3) == 0) {
            const uint32_t g = lane >> 2;
            const uint64_t r0 = static_cast<uint64_t>(tile) * 16 + g, r1 = r0 + 8;
            if (r0 < n) logits[r0] = lo;
            if (r1 < n) logits[r1] = hi;
        }
        __syncwarp();
    }
}

struct TrainSmem {
    MlpFrag f;
    uint2 w2t[2][4][32];  // B fragments of W2^T (bf16)
    float w3r[kMlpH];     // bf16-rounded w3
    // per-warp gradient and loss (index kMlpParams); every entry has exactly
    // one owning lane, so the CTA sum runs in a fixed order
    float wg[kTrainWarps][kGradRow];
    struct Warp {
        uint32_t xs[16 * 4];         // packed inputs, row-major (16 x 8 bf16)
        __nv_bfloat16 h1[16][kMlpH];  // [sample][feature]
        __nv_bfloat16 h2[16][kMlpH];
        __nv_bfloat16 dz2[16][kMlpH];
        __nv_bfloat16 dz1[16][kMlpH];
        __nv_bfloat16 g3[16];
    } w[kTrainWarps];
};

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return static_cast<uint32_t>(__bfloat16_as_ushort(lo)) |
           (static_cast<uint32_t>(__bfloat16_as_ushort(hi)) << 16);
}

__device__ __forceinline__ float softplus(float x) {
    return fmaxf(x, 0.f) + log1pf(expf(-fabsf(x)));
}

__global__ void __launch_bounds__(kTrainWarps * 32)
k_mlp_grad(const float* __restrict__ P, const float* __restrict__ norm,
           const float* __restrict__ feat, const float* __restrict__ label, uint32_t n,
           float pos_weight, float* __restrict__ part) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    build_frag(S.f, P, norm);
    for (uint32_t i = threadIdx.x; i < 2 * 4 * 32; i += blockDim.x) {
        const uint32_t ks = i >> 7, nt = (i >> 5) & 3, lane = i & 31, g = lane >> 2, t = lane & 3;
        // W2^T[k][j] = W2[j][k]: rows k = ks*16 + 2t (+1, +8, +9), column j = nt*8 + g
        const uint32_t j = nt * 8 + g, k0 = ks * 16 + 2 * t;
        S.w2t[ks][nt][lane] = make_uint2(
            pack_bf16(P[kOffW2 + j * kMlpH + k0], P[kOffW2 + j * kMlpH + k0 + 1]),
            pack_bf16(P[kOffW2 + j * kMlpH + k0 + 8], P[kOffW2 + j * kMlpH + k0 + 9]));
    }
    for (uint32_t i = threadIdx.x; i < kMlpH; i += blockDim.x) S.w3r[i] = bf16_round(P[kOffW3 + i]);
    __syncthreads();

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t g = lane >> 2, t = lane & 3;
    auto& W = S.w[warp];
    const MlpFrag& f = S.f;
    const float inv_n = 1.f / static_cast<float>(max(n, 1u));

    float aW1[4][4] = {}, aW2[2][4][4] = {}, aW3[2][4] = {};
    float aB1[4][2] = {}, aB2[4][2] = {}, aB3 = 0.f, aL = 0.f;

    const uint32_t tiles = (n + 15) / 16;
    for (uint32_t tile = blockIdx.x * kTrainWarps + warp; tile < tiles;
         tile += gridDim.x * kTrainWarps) {
        const uint64_t row0 = static_cast<uint64_t>(tile) * 16;
        if (lane < 16) {
            uint32_t p[4];
            load_row(f, feat, n, row0 + lane, p);
#pragma unroll
            for (int i = 0; i < 4; ++i) W.xs[4 * lane + i] = p[i];
        }
        __syncwarp();
        // ---- forward (as mlp_tile16, keeping the pre-activations)
        uint32_t a[4] = {W.xs[4 * g + t], W.xs[4 * (g + 8) + t], 0u, 0u};
        float z1[4][4], z2[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const float c0 = f.b1[nt * 8 + 2 * t], c1 = f.b1[nt * 8 + 2 * t + 1];
            z1[nt][0] = c0; z1[nt][1] = c1; z1[nt][2] = c0; z1[nt][3] = c1;
            const uint2 b = f.w1[nt][lane];
            mma_bf16(z1[nt], a, b.x, b.y);
        }
        uint32_t ah[2][4];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            ah[ks][0] = pack_bf16(fmaxf(z1[2 * ks][0], 0.f), fmaxf(z1[2 * ks][1], 0.f));
            ah[ks][1] = pack_bf16(fmaxf(z1[2 * ks][2], 0.f), fmaxf(z1[2 * ks][3], 0.f));
            ah[ks][2] = pack_bf16(fmaxf(z1[2 * ks + 1][0], 0.f), fmaxf(z1[2 * ks + 1][1], 0.f));
            ah[ks][3] = pack_bf16(fmaxf(z1[2 * ks + 1][2], 0.f), fmaxf(z1[2 * ks + 1][3], 0.f));
        }
        // h1 to shared memory, [sample][feature]
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            *reinterpret_cast<uint32_t*>(&W.h1[g][ks * 16 + 2 * t]) = ah[ks][0];
            *reinterpret_cast<uint32_t*>(&W.h1[g + 8][ks * 16 + 2 * t]) = ah[ks][1];
            *reinterpret_cast<uint32_t*>(&W.h1[g][ks * 16 + 8 + 2 * t]) = ah[ks][2];
            *reinterpret_cast<uint32_t*>(&W.h1[g + 8][ks * 16 + 8 + 2 * t]) = ah[ks][3];
        }
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const float c0 = f.b2[nt * 8 + 2 * t], c1 = f.b2[nt * 8 + 2 * t + 1];
            z2[nt][0] = c0; z2[nt][1] = c1; z2[nt][2] = c0; z2[nt][3] = c1;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                const uint2 b = f.w2[ks][nt][lane];
                mma_bf16(z2[nt], ah[ks], b.x, b.y);
            }
        }
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            ah[ks][0] = pack_bf16(fmaxf(z2[2 * ks][0], 0.f), fmaxf(z2[2 * ks][1], 0.f));
            ah[ks][1] = pack_bf16(fmaxf(z2[2 * ks][2], 0.f), fmaxf(z2[2 * ks][3], 0.f));
            ah[ks][2] = pack_bf16(fmaxf(z2[2 * ks + 1][0], 0.f), fmaxf(z2[2 * ks + 1][1], 0.f));
            ah[ks][3] = pack_bf16(fmaxf(z2[2 * ks + 1][2], 0.f), fmaxf(z2[2 * ks + 1][3], 0.f));
            *reinterpret_cast<uint32_t*>(&W.h2[g][ks * 16 + 2 * t]) = ah[ks][0];
            *reinterpret_cast<uint32_t*>(&W.h2[g + 8][ks * 16 + 2 * t]) = ah[ks][1];
            *reinterpret_cast<uint32_t*>(&W.h2[g][ks * 16 + 8 + 2 * t]) = ah[ks][2];
            *reinterpret_cast<uint32_t*>(&W.h2[g + 8][ks * 16 + 8 + 2 * t]) = ah[ks][3];
        }
        float o[4] = {t == 0 ? f.b3 : 0.f, 0.f, t == 0 ? f.b3 : 0.f, 0.f};
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            const uint2 b = f.w3[ks][lane];
            mma_bf16(o, ah[ks], b.x, b.y);
        }
        // ---- loss gradient at the logits (lanes t == 0 hold rows g, g + 8)
        float g3lo = 0.f, g3hi = 0.f;
        if (t == 0) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint64_t r = row0 + g + 8 * h;
                float gz = 0.f;
                if (r < n) {
                    const float z = h ? o[2] : o[0];
                    const float y = label[r];
                    const float s = 1.f / (1.f + expf(-z));
                    gz = (pos_weight * y * (s - 1.f) + (1.f - y) * s) * inv_n;
                    aL += (pos_weight * y * softplus(-z) + (1.f - y) * softplus(z)) * inv_n;
                }
                if (h) g3hi = gz; else g3lo = gz;
            }
            aB3 += g3lo + g3hi;
            W.g3[g] = __float2bfloat16_rn(g3lo);
            W.g3[g + 8] = __float2bfloat16_rn(g3hi);
        }
        g3lo = __shfl_sync(0xffffffffu, g3lo, lane & ~3u);
        g3hi = __shfl_sync(0xffffffffu, g3hi, lane & ~3u);
        // ---- dz2 = g3 w3 [z2 > 0]
        float dz2[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const float w0 = S.w3r[nt * 8 + 2 * t], w1 = S.w3r[nt * 8 + 2 * t + 1];
            dz2[nt][0] = z2[nt][0] > 0.f ? g3lo * w0 : 0.f;
            dz2[nt][1] = z2[nt][1] > 0.f ? g3lo * w1 : 0.f;
            dz2[nt][2] = z2[nt][2] > 0.f ? g3hi * w0 : 0.f;
            dz2[nt][3] = z2[nt][3] > 0.f ? g3hi * w1 : 0.f;
            aB2[nt][0] += dz2[nt][0] + dz2[nt][2];
            aB2[nt][1] += dz2[nt][1] + dz2[nt][3];
        }
        uint32_t ad[2][4];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            ad[ks][0] = pack_bf16(dz2[2 * ks][0], dz2[2 * ks][1]);
            ad[ks][1] = pack_bf16(dz2[2 * ks][2], dz2[2 * ks][3]);
            ad[ks][2] = pack_bf16(dz2[2 * ks + 1][0], dz2[2 * ks + 1][1]);
            ad[ks][3] = pack_bf16(dz2[2 * ks + 1][2], dz2[2 * ks + 1][3]);
            *reinterpret_cast<uint32_t*>(&W.dz2[g][ks * 16 + 2 * t]) = ad[ks][0];
            *reinterpret_cast<uint32_t*>(&W.dz2[g + 8][ks * 16 + 2 * t]) = ad[ks][1];
            *reinterpret_cast<uint32_t*>(&W.dz2[g][ks * 16 + 8 + 2 * t]) = ad[ks][2];
            *reinterpret_cast<uint32_t*>(&W.dz2[g + 8][ks * 16 + 8 + 2 * t]) = ad[ks][3];
        }
        // ---- dz1 = (bf16(dz2) W2^T) [z1 > 0]
        float dz1[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            dz1[nt][0] = dz1[nt][1] = dz1[nt][2] = dz1[nt][3] = 0.f;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                const uint2 b = S.w2t[ks][nt][lane];
                mma_bf16(dz1[nt], ad[ks], b.x, b.y);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) dz1[nt][q] = z1[nt][q] > 0.f ? dz1[nt][q] : 0.f;
            aB1[nt][0] += dz1[nt][0] + dz1[nt][2];
            aB1[nt][1] += dz1[nt][1] + dz1[nt][3];
            *reinterpret_cast<uint32_t*>(&W.dz1[g][nt * 8 + 2 * t]) =
                pack_bf16(dz1[nt][0], dz1[nt][1]);
            *reinterpret_cast<uint32_t*>(&W.dz1[g + 8][nt * 8 + 2 * t]) =
                pack_bf16(dz1[nt][2], dz1[nt][3]);
        }
        __syncwarp();
        // ---- weight gradients: (activation^T) x (delta), K = the 16 samples
        // dW2[i][j] += sum_s h1[s][i] dz2[s][j]
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            uint32_t A[4];
            const int i0 = mt * 16 + g;
            A[0] = pack2(W.h1[2 * t][i0], W.h1[2 * t + 1][i0]);
            A[1] = pack2(W.h1[2 * t][i0 + 8], W.h1[2 * t + 1][i0 + 8]);
            A[2] = pack2(W.h1[2 * t + 8][i0], W.h1[2 * t + 9][i0]);
            A[3] = pack2(W.h1[2 * t + 8][i0 + 8], W.h1[2 * t + 9][i0 + 8]);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int j = nt * 8 + g;
                const uint32_t b0 = pack2(W.dz2[2 * t][j], W.dz2[2 * t + 1][j]);
                const uint32_t b1 = pack2(W.dz2[2 * t + 8][j], W.dz2[2 * t + 9][j]);
                mma_bf16(aW2[mt][nt], A, b0, b1);
            }
            // dW3[i] += sum_s h2[s][i] g3[s]
            uint32_t H[4];
            H[0] = pack2(W.h2[2 * t][i0], W.h2[2 * t + 1][i0]);
            H[1] = pack2(W.h2[2 * t][i0 + 8], W.h2[2 * t + 1][i0 + 8]);
            H[2] = pack2(W.h2[2 * t + 8][i0], W.h2[2 * t + 9][i0]);
            H[3] = pack2(W.h2[2 * t + 8][i0 + 8], W.h2[2 * t + 9][i0 + 8]);
            const uint32_t gb0 = g == 0 ? pack2(W.g3[2 * t], W.g3[2 * t + 1]) : 0u;
            const uint32_t gb1 = g == 0 ? pack2(W.g3[2 * t + 8], W.g3[2 * t + 9]) : 0u;
            mma_bf16(aW3[mt], H, gb0, gb1);
        }
        // dW1[i][j] += sum_s x[s][i] dz1[s][j]  (input rows 8..15 are zero)
        {
            const __nv_bfloat16* xb = reinterpret_cast<const __nv_bfloat16*>(W.xs);
            uint32_t A[4];
            A[0] = pack2(xb[(2 * t) * 8 + g], xb[(2 * t + 1) * 8 + g]);
            A[1] = 0u;
            A[2] = pack2(xb[(2 * t + 8) * 8 + g], xb[(2 * t + 9) * 8 + g]);
            A[3] = 0u;
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int j = nt * 8 + g;
                const uint32_t b0 = pack2(W.dz1[2 * t][j], W.dz1[2 * t + 1][j]);
                const uint32_t b1 = pack2(W.dz1[2 * t + 8][j], W.dz1[2 * t + 9][j]);
                mma_bf16(aW1[nt], A, b0, b1);
            }
        }
        __syncwarp();
    }

    // ---- reduce in a fixed order: lanes -> the warp's slice (one owner per
    //      entry) -> the CTA's row of `part` (warps in order); k_grad_sum adds
    //      the rows in CTA order, so a training run is reproducible
    float* wg = S.wg[warp];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const int j = nt * 8 + 2 * t;
        // dW1 rows g (< 8); rows g + 8 are padding
        wg[kOffW1 + g * kMlpH + j] = aW1[nt][0];
        wg[kOffW1 + g * kMlpH + j + 1] = aW1[nt][1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int i = mt * 16 + g;
            wg[kOffW2 + i * kMlpH + j] = aW2[mt][nt][0];
            wg[kOffW2 + i * kMlpH + j + 1] = aW2[mt][nt][1];
            wg[kOffW2 + (i + 8) * kMlpH + j] = aW2[mt][nt][2];
            wg[kOffW2 + (i + 8) * kMlpH + j + 1] = aW2[mt][nt][3];
        }
        float b1x = aB1[nt][0], b1y = aB1[nt][1], b2x = aB2[nt][0], b2y = aB2[nt][1];
        for (int o = 4; o < 32; o <<= 1) {
            b1x += __shfl_xor_sync(0xffffffffu, b1x, o);
            b1y += __shfl_xor_sync(0xffffffffu, b1y, o);
            b2x += __shfl_xor_sync(0xffffffffu, b2x, o);
            b2y += __shfl_xor_sync(0xffffffffu, b2y, o);
        }
        if (g == 0) {
            wg[kOffB1 + j] = b1x;
            wg[kOffB1 + j + 1] = b1y;
            wg[kOffB2 + j] = b2x;
            wg[kOffB2 + j + 1] = b2y;
        }
    }
    if (t == 0) {
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            wg[kOffW3 + mt * 16 + g] = aW3[mt][0];
            wg[kOffW3 + mt * 16 + g + 8] = aW3[mt][2];
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        aB3 += __shfl_xor_sync(0xffffffffu, aB3, o);
        aL += __shfl_xor_sync(0xffffffffu, aL, o);
    }
    if (lane == 0) {
        wg[kOffB3] = aB3;
        wg[kMlpParams] = aL;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i <= kMlpParams; i += blockDim.x) {
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < kTrainWarps; ++w) sum += S.wg[w][i];
        part[static_cast<size_t>(blockIdx.x) * kGradRow + i] = sum;
    }
}

// grad / loss = the CTA rows of `part` added in CTA order.
__global__ void k_grad_sum(const float* __restrict__ part, uint32_t rows,
                           float* __restrict__ grad, float* __restrict__ loss) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > static_cast<uint32_t>(kMlpParams)) return;
    float sum = 0.f;
    for (uint32_t r = 0; r < rows; ++r) sum += part[static_cast<size_t>(r) * kGradRow + i];
    if (i < static_cast<uint32_t>(kMlpParams)) grad[i] = sum;
    else *loss = sum;
}

// Per-thread scratch for the CTA rows of the gradient (one stream per host
// thread, as for the seeding handles).
struct GradScratch {
    float* p = nullptr;
    uint32_t rows = 0;
    int device = -1;
    ~GradScratch() {
        if (p) cudaFree(p);
    }
};

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                       float* __restrict__ V, uint32_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = G[i];
    const float m = b1 * M[i] + (1.f - b1) * gi;
    const float v = b2 * V[i] + (1.f - b2) * gi * gi;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

int device_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    return n;
}

}  // namespace

// Host packing of the fragments the seeding kernel reads (bit-identical to
// build_frag: bf16 round-to-nearest-even).
static uint16_t host_bf16(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u && (u & 0x007fffffu)) return static_cast<uint16_t>((u | 0x00400000u) >> 16);
    u += 0x7fffu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
}
static uint32_t host_pack(float lo, float hi) {
    return static_cast<uint32_t>(host_bf16(lo)) | (static_cast<uint32_t>(host_bf16(hi)) << 16);
}

size_t mlp_frag_bytes() { return sizeof(MlpFrag); }

void pack_mlp_frag(const seedgb_doublet_filter& m, MlpFrag& f) {
    std::memset(&f, 0, sizeof f);
    for (int nt = 0; nt < 4; ++nt)
        for (int lane = 0; lane < 32; ++lane) {
            const int g = lane >> 2, t = lane & 3, col = nt * 8 + g;
            f.w1[nt][lane] = make_uint2(host_pack(m.w1[(2 * t) * kMlpH + col],
                                                  m.w1[(2 * t + 1) * kMlpH + col]), 0u);
        }
    for (int ks = 0; ks < 2; ++ks)
        for (int nt = 0; nt < 4; ++nt)
            for (int lane = 0; lane < 32; ++lane) {
                const int g = lane >> 2, t = lane & 3, col = nt * 8 + g, k0 = ks * 16 + 2 * t;
                f.w2[ks][nt][lane] =
                    make_uint2(host_pack(m.w2[k0 * kMlpH + col], m.w2[(k0 + 1) * kMlpH + col]),
                               host_pack(m.w2[(k0 + 8) * kMlpH + col], m.w2[(k0 + 9) * kMlpH + col]));
            }
    for (int ks = 0; ks < 2; ++ks)
        for (int lane = 0; lane < 32; ++lane) {
            const int g = lane >> 2, t = lane & 3, k0 = ks * 16 + 2 * t;
            f.w3[ks][lane] = g == 0 ? make_uint2(host_pack(m.w3[k0], m.w3[k0 + 1]),
                                                 host_pack(m.w3[k0 + 8], m.w3[k0 + 9]))
                                    : make_uint2(0u, 0u);
        }
    for (int i = 0; i < kMlpH; ++i) {
        f.b1[i] = m.b1[i];
        f.b2[i] = m.b2[i];
    }
    f.b3 = m.b3;
    for (int i = 0; i < kMlpIn; ++i) {
        f.mu[i] = m.mu[i];
        f.isd[i] = m.isd[i];
    }
    f.threshold[0] = m.threshold[0];
    f.threshold[1] = m.threshold[1];
    f.n_edges = std::min<uint32_t>(m.n_edges, kMaxBandEdges);
    for (uint32_t i = 0; i < f.n_edges; ++i) f.edges[i] = m.edges[i];
    f.prune_bottom = m.prune_bottom;
    f.prune_top = m.prune_top;
}

}  // namespace seedgb

using namespace seedgb;

extern "C" {

uint32_t seedgb_mlp_num_params(void) { return kMlpParams; }

seedgb_status seedgb_mlp_forward(const float* params, const float* norm, const float* features,
                                 uint32_t n, float* logits, void* stream) {
    if (!params || !norm || (n && (!features || !logits))) return SEEDGB_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(features) % 16) return SEEDGB_INVALID_ARGUMENT;
    if (n == 0) return SEEDGB_OK;
    const int sms = device_sms();
    if (sms <= 0) return SEEDGB_CUDA_ERROR;
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t grid = std::min<uint32_t>((tiles + kTrainWarps - 1) / kTrainWarps,
                                             static_cast<uint32_t>(sms) * 8);
    k_mlp_forward<<<grid, kTrainWarps * 32, 0, static_cast<cudaStream_t>(stream)>>>(
        params, norm, features, n, logits);
    return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}

seedgb_status seedgb_mlp_grad(const float* params, const float* norm, const float* features,
                              const float* labels, uint32_t n, float pos_weight, float* grad,
                              float* loss, void* stream) {
    if (!params || !norm || !grad || !loss || (n && (!features || !labels)))
        return SEEDGB_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(features) % 16) return SEEDGB_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        cudaError_t err = cudaMemsetAsync(grad, 0, sizeof(float) * kMlpParams, s);
        if (err == cudaSuccess) err = cudaMemsetAsync(loss, 0, sizeof(float), s);
        return err == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
    }
    static thread_local int attr_dev = -1;  // the attribute is per context
    static thread_local GradScratch scratch;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    if (attr_dev != dev) {
        if (cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(TrainSmem))) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
        attr_dev = dev;
    }
    const int sms = device_sms();
    if (sms <= 0) return SEEDGB_CUDA_ERROR;
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t grid = std::min<uint32_t>((tiles + kTrainWarps - 1) / kTrainWarps,
                                             static_cast<uint32_t>(sms));
    if (scratch.rows < grid || scratch.device != dev) {
        // the previous scratch may still be in use by work on any stream
        if (scratch.p && cudaDeviceSynchronize() != cudaSuccess) return SEEDGB_CUDA_ERROR;
        if (scratch.p) cudaFree(scratch.p);
        scratch.p = nullptr;
        scratch.rows = 0;
        const uint32_t rows = std::max<uint32_t>(grid, static_cast<uint32_t>(sms));
        if (cudaMalloc(&scratch.p, sizeof(float) * kGradRow * rows) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
        scratch.rows = rows;
        scratch.device = dev;
    }
    k_mlp_grad<<<grid, kTrainWarps * 32, sizeof(TrainSmem), s>>>(params, norm, features, labels,
                                                                n, pos_weight, scratch.p);
    k_grad_sum<<<(kMlpParams + 1 + 255) / 256, 256, 0, s>>>(scratch.p, grid, grad, loss);
    return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}

seedgb_status seedgb_mlp_adam(float* params, const float* grad, float* m, float* v, uint32_t n,
                              uint32_t step, float lr, float beta1, float beta2, float eps,
                              void* stream) {
    if (!params || !grad || !m || !v || step == 0) return SEEDGB_INVALID_ARGUMENT;
    if (n == 0) return SEEDGB_OK;
    const float c1 = 1.f - std::pow(beta1, static_cast<float>(step));
    const float c2 = 1.f - std::pow(beta2, static_cast<float>(step));
    k_adam<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, grad, m, v, n, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}

}  // extern "C"
