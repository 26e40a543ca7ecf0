// The learned doublet filter's network on the tensor cores: an MLP
// 8 -> 32 -> 32 -> 1 evaluated by one warp on tiles of 16 doublets with
// mma.sync m16n8k16 (bf16 operands, fp32 accumulate).
//
// Numerics (the same as the CPU restatement in the oracle): inputs are
// standardised in fp32 ((f - mu) * isd) and rounded to bf16; weights are bf16;
// each layer accumulates in fp32 starting from its fp32 bias; ReLU; hidden
// activations are rounded to bf16 before the next layer; the output is a
// logit.  The tensor cores' internal summation order is not specified, so a
// logit may differ from a sequential fp32 sum in its last bits.
//
// Fragment layouts of mma.m16n8k16 (PTX ISA, "Matrix fragments for
// mma.m16n8k16"): with g = lane / 4 and t = lane % 4,
//   A (16x16, row): a0 = (g, 2t..2t+1), a1 = (g+8, 2t..), a2 = (g, 2t+8..),
//                   a3 = (g+8, 2t+8..)
//   B (16x8, col):  b0 = (2t..2t+1, g), b1 = (2t+8..2t+9, g)
//   C/D (16x8):     d0 = (g, 2t), d1 = (g, 2t+1), d2 = (g+8, 2t), d3 = (g+8, 2t+1)
// Two bf16 per 32-bit register, the lower index in the lower half.  The D
// fragments of n-tiles 2k and 2k+1 of one layer are exactly the A fragment of
// k-step k of the next layer, so activations never leave registers.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace seedgb {

constexpr int kMlpIn = 8;
constexpr int kMlpH = 32;
constexpr int kMaxBandEdges = 15;
// fp32 master parameter block: w1[8][32], b1[32], w2[32][32], b2[32], w3[32], b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpIn * kMlpH;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpH;
constexpr int kMlpParams = kOffB3 + 1;  // 1377

// The network packed as per-lane B fragments (what one warp loads per mma)
// plus what the feature stage needs.  Built on the host from the fp32 model.
struct MlpFrag {
    uint2 w1[4][32];      // [n-tile][lane] {b0, b1} (k rows 8..15 are zero)
    uint2 w2[2][4][32];   // [k-step][n-tile][lane]
    uint2 w3[2][32];      // [k-step][lane] (column 0 only)
    float b1[kMlpH], b2[kMlpH], b3;
    float mu[kMlpIn], isd[kMlpIn];
    float threshold[2];   // keep when logit >= threshold[role], role 1 = top
    float edges[kMaxBandEdges];
    uint32_t n_edges;
    uint32_t prune_bottom, prune_top;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half)
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ float bf16_round(float x) {
    return __bfloat162float(__float2bfloat16_rn(x));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Radial band of r: the number of band edges <= r (edges ascending).
__device__ __forceinline__ uint32_t mlp_band(const float* edges, uint32_t n_edges, float r) {
    uint32_t b = 0;
#pragma unroll
    for (uint32_t i = 0; i < kMaxBandEdges; ++i) b += (i < n_edges && edges[i] <= r) ? 1u : 0u;
    return b;
}

// The 8 features of doublet (m, o): r_m, z_m, r_o - r_m, z_o - z_m, the
// lin_circle's cot(theta), s = y / |dxy| (the sine of the doublet's azimuthal
// angle to the middle spacepoint's radial direction), the lin_circle's Zo and
// the layer-pair id band(r_m) * (n_edges + 1) + band(r_o).
__device__ __forceinline__ void mlp_features(const float* edges, uint32_t n_edges,
                                             const float4 m, const float4 o, float cot,
                                             float s, float zo, float (&x)[kMlpIn]) {
    x[0] = m.w;
    x[1] = m.z;
    x[2] = o.w - m.w;
    x[3] = o.z - m.z;
    x[4] = cot;
    x[5] = s;
    x[6] = zo;
    x[7] = static_cast<float>(mlp_band(edges, n_edges, m.w) * (n_edges + 1) +
                              mlp_band(edges, n_edges, o.w));
}

// Standardised bf16 inputs of one doublet as 4 packed registers (k 0..7).
__device__ __forceinline__ void mlp_pack_inputs(const float* mu, const float* isd,
                                                const float (&x)[kMlpIn], uint32_t (&p)[4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
        p[i] = pack_bf16((x[2 * i] - mu[2 * i]) * isd[2 * i],
                         (x[2 * i + 1] - mu[2 * i + 1]) * isd[2 * i + 1]);
}

// Logits of 16 doublets.  xs: the warp's packed inputs, 16 rows x 4 words
// (row r at xs[4 r]).  Returns the logits of rows g and g+8 in lanes with
// t == 0 (lo, hi); other lanes return unspecified values.
__device__ __forceinline__ void mlp_tile16(const MlpFrag& f, const uint32_t* xs, uint32_t lane,
                                           float& lo, float& hi) {
    const uint32_t g = lane >> 2, t = lane & 3;
    uint32_t a[4];
    a[0] = xs[4 * g + t];
    a[1] = xs[4 * (g + 8) + t];
    a[2] = 0u;
    a[3] = 0u;
    float h[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const float c0 = f.b1[nt * 8 + 2 * t], c1 = f.b1[nt * 8 + 2 * t + 1];
        h[nt][0] = c0; h[nt][1] = c1; h[nt][2] = c0; h[nt][3] = c1;
        const uint2 b = f.w1[nt][lane];
        mma_bf16(h[nt], a, b.x, b.y);
    }
    // layer 2: the D fragments of layer 1 are the A fragments
    uint32_t a2[2][4];
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        a2[ks][0] = pack_bf16(fmaxf(h[2 * ks][0], 0.f), fmaxf(h[2 * ks][1], 0.f));
        a2[ks][1] = pack_bf16(fmaxf(h[2 * ks][2], 0.f), fmaxf(h[2 * ks][3], 0.f));
        a2[ks][2] = pack_bf16(fmaxf(h[2 * ks + 1][0], 0.f), fmaxf(h[2 * ks + 1][1], 0.f));
        a2[ks][3] = pack_bf16(fmaxf(h[2 * ks + 1][2], 0.f), fmaxf(h[2 * ks + 1][3], 0.f));
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const float c0 = f.b2[nt * 8 + 2 * t], c1 = f.b2[nt * 8 + 2 * t + 1];
        h[nt][0] = c0; h[nt][1] = c1; h[nt][2] = c0; h[nt][3] = c1;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            const uint2 b = f.w2[ks][nt][lane];
            mma_bf16(h[nt], a2[ks], b.x, b.y);
        }
    }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        a2[ks][0] = pack_bf16(fmaxf(h[2 * ks][0], 0.f), fmaxf(h[2 * ks][1], 0.f));
        a2[ks][1] = pack_bf16(fmaxf(h[2 * ks][2], 0.f), fmaxf(h[2 * ks][3], 0.f));
        a2[ks][2] = pack_bf16(fmaxf(h[2 * ks + 1][0], 0.f), fmaxf(h[2 * ks + 1][1], 0.f));
        a2[ks][3] = pack_bf16(fmaxf(h[2 * ks + 1][2], 0.f), fmaxf(h[2 * ks + 1][3], 0.f));
    }
    float o[4] = {t == 0 ? f.b3 : 0.f, 0.f, t == 0 ? f.b3 : 0.f, 0.f};
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        const uint2 b = f.w3[ks][lane];
        mma_bf16(o, a2[ks], b.x, b.y);
    }
    lo = o[0];
    hi = o[2];
}

// mlp_tile16 computed two output n-tiles at a time, so that few fragments and
// accumulators are live at once (for code that calls it with many registers
// of its own live).  Same operands, same mma sequence per output element,
// hence the same logits.
__device__ __forceinline__ void mlp_tile16_lean(const MlpFrag& f, const uint32_t* xs,
                                                uint32_t lane, float& lo, float& hi) {
    const uint32_t g = lane >> 2, t = lane & 3;
    const uint32_t a[4] = {xs[4 * g + t], xs[4 * (g + 8) + t], 0u, 0u};
    uint32_t a2[2][4], a3[2][4];
#pragma unroll 1
    for (int ks = 0; ks < 2; ++ks) {
        float h0[4], h1[4];
        const int n0 = 2 * ks, n1 = 2 * ks + 1;
        h0[0] = h0[2] = f.b1[n0 * 8 + 2 * t];
        h0[1] = h0[3] = f.b1[n0 * 8 + 2 * t + 1];
        h1[0] = h1[2] = f.b1[n1 * 8 + 2 * t];
        h1[1] = h1[3] = f.b1[n1 * 8 + 2 * t + 1];
        const uint2 b0 = f.w1[n0][lane], b1 = f.w1[n1][lane];
        mma_bf16(h0, a, b0.x, b0.y);
        mma_bf16(h1, a, b1.x, b1.y);
        const uint32_t p0 = pack_bf16(fmaxf(h0[0], 0.f), fmaxf(h0[1], 0.f));
        const uint32_t p1 = pack_bf16(fmaxf(h0[2], 0.f), fmaxf(h0[3], 0.f));
        const uint32_t p2 = pack_bf16(fmaxf(h1[0], 0.f), fmaxf(h1[1], 0.f));
        const uint32_t p3 = pack_bf16(fmaxf(h1[2], 0.f), fmaxf(h1[3], 0.f));
        if (ks == 0) { a2[0][0] = p0; a2[0][1] = p1; a2[0][2] = p2; a2[0][3] = p3; }
        else { a2[1][0] = p0; a2[1][1] = p1; a2[1][2] = p2; a2[1][3] = p3; }
    }
#pragma unroll 1
    for (int ks = 0; ks < 2; ++ks) {
        float h0[4], h1[4];
        const int n0 = 2 * ks, n1 = 2 * ks + 1;
        h0[0] = h0[2] = f.b2[n0 * 8 + 2 * t];
        h0[1] = h0[3] = f.b2[n0 * 8 + 2 * t + 1];
        h1[0] = h1[2] = f.b2[n1 * 8 + 2 * t];
        h1[1] = h1[3] = f.b2[n1 * 8 + 2 * t + 1];
#pragma unroll 1
        for (int k = 0; k < 2; ++k) {
            const uint2 b0 = f.w2[k][n0][lane], b1 = f.w2[k][n1][lane];
            mma_bf16(h0, a2[k], b0.x, b0.y);
            mma_bf16(h1, a2[k], b1.x, b1.y);
        }
        const uint32_t p0 = pack_bf16(fmaxf(h0[0], 0.f), fmaxf(h0[1], 0.f));
        const uint32_t p1 = pack_bf16(fmaxf(h0[2], 0.f), fmaxf(h0[3], 0.f));
        const uint32_t p2 = pack_bf16(fmaxf(h1[0], 0.f), fmaxf(h1[1], 0.f));
        const uint32_t p3 = pack_bf16(fmaxf(h1[2], 0.f), fmaxf(h1[3], 0.f));
        if (ks == 0) { a3[0][0] = p0; a3[0][1] = p1; a3[0][2] = p2; a3[0][3] = p3; }
        else { a3[1][0] = p0; a3[1][1] = p1; a3[1][2] = p2; a3[1][3] = p3; }
    }
    float o[4] = {t == 0 ? f.b3 : 0.f, 0.f, t == 0 ? f.b3 : 0.f, 0.f};
#pragma unroll 1
    for (int ks = 0; ks < 2; ++ks) {
        const uint2 b = f.w3[ks][lane];
        mma_bf16(o, a3[ks], b.x, b.y);
    }
    lo = o[0];
    hi = o[2];
}

// The network held in registers by one warp (per-lane B fragments and the
// biases of the lane's output columns), for loops over many tiles.
struct MlpRegs {
    uint2 w1[4], w2[2][4], w3[2];
    float b1[8], b2[8], b3;
};

__device__ __forceinline__ void mlp_load_regs(const MlpFrag& f, uint32_t lane, MlpRegs& r) {
    const uint32_t t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        r.w1[nt] = f.w1[nt][lane];
        r.w2[0][nt] = f.w2[0][nt][lane];
        r.w2[1][nt] = f.w2[1][nt][lane];
        r.b1[2 * nt] = f.b1[nt * 8 + 2 * t];
        r.b1[2 * nt + 1] = f.b1[nt * 8 + 2 * t + 1];
        r.b2[2 * nt] = f.b2[nt * 8 + 2 * t];
        r.b2[2 * nt + 1] = f.b2[nt * 8 + 2 * t + 1];
    }
    r.w3[0] = f.w3[0][lane];
    r.w3[1] = f.w3[1][lane];
    r.b3 = t == 0 ? f.b3 : 0.f;
}

// mlp_tile16 with the network in registers (same arithmetic).
__device__ __forceinline__ void mlp_tile16_regs(const MlpRegs& r, const uint32_t* xs,
                                                uint32_t lane, float& lo, float& hi) {
    const uint32_t g = lane >> 2, t = lane & 3;
    uint32_t a[4] = {xs[4 * g + t], xs[4 * (g + 8) + t], 0u, 0u};
    float h[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        h[nt][0] = r.b1[2 * nt]; h[nt][1] = r.b1[2 * nt + 1];
        h[nt][2] = r.b1[2 * nt]; h[nt][3] = r.b1[2 * nt + 1];
        mma_bf16(h[nt], a, r.w1[nt].x, r.w1[nt].y);
    }
    uint32_t a2[2][4];
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        a2[ks][0] = pack_bf16(fmaxf(h[2 * ks][0], 0.f), fmaxf(h[2 * ks][1], 0.f));
        a2[ks][1] = pack_bf16(fmaxf(h[2 * ks][2], 0.f), fmaxf(h[2 * ks][3], 0.f));
        a2[ks][2] = pack_bf16(fmaxf(h[2 * ks + 1][0], 0.f), fmaxf(h[2 * ks + 1][1], 0.f));
        a2[ks][3] = pack_bf16(fmaxf(h[2 * ks + 1][2], 0.f), fmaxf(h[2 * ks + 1][3], 0.f));
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        h[nt][0] = r.b2[2 * nt]; h[nt][1] = r.b2[2 * nt + 1];
        h[nt][2] = r.b2[2 * nt]; h[nt][3] = r.b2[2 * nt + 1];
        mma_bf16(h[nt], a2[0], r.w2[0][nt].x, r.w2[0][nt].y);
        mma_bf16(h[nt], a2[1], r.w2[1][nt].x, r.w2[1][nt].y);
    }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        a2[ks][0] = pack_bf16(fmaxf(h[2 * ks][0], 0.f), fmaxf(h[2 * ks][1], 0.f));
        a2[ks][1] = pack_bf16(fmaxf(h[2 * ks][2], 0.f), fmaxf(h[2 * ks][3], 0.f));
        a2[ks][2] = pack_bf16(fmaxf(h[2 * ks + 1][0], 0.f), fmaxf(h[2 * ks + 1][1], 0.f));
        a2[ks][3] = pack_bf16(fmaxf(h[2 * ks + 1][2], 0.f), fmaxf(h[2 * ks + 1][3], 0.f));
    }
    float o[4] = {r.b3, 0.f, r.b3, 0.f};
    mma_bf16(o, a2[0], r.w3[0].x, r.w3[0].y);
    mma_bf16(o, a2[1], r.w3[1].x, r.w3[1].y);
    lo = o[0];
    hi = o[2];
}

}  // namespace seedgb
