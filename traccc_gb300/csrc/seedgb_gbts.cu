// GBTS seeding (graph-based track seeding) on the GB300.
//
// The reference's GBTS chain (device/common/src/gbts_seeding/
// gbts_seeding_algorithm.cpp, kernels in device/common/include/traccc/
// gbts_seeding/device/impl) builds a graph of spacepoint pairs (edges) between
// linked layer-eta bins, links edges that continue each other, finds the
// longest chains with a cellular automaton, fits every chain with a Kalman
// filter and resolves shared edges and hits by bidding.  Its results depend on
// the order in which its atomics land in several places; this library
// computes the same chain in one fixed order, so results are reproducible and
// equal to the CPU oracle bit for bit:
//   - nodes of one (eta, phi) cell in ascending spacepoint index;
//   - edges by (work item, thread, outer node, inner node), each work item a
//     bin pair with a bin-1 chunk of at most 128 nodes, 128 threads per item
//     taking the outer nodes t, t + 128, ... with the reference's
//     sliding-window state;
//   - every node's outgoing edges in ascending edge index;
//   - connected edges numbered in ascending edge index (a scan, not atomics);
//   - terminus edges in ascending connected-edge index, the path store as a
//     depth-first pre-order walk below each terminus edge;
//   - seed proposals in path-store order, seeds by proposal.
// Ordered outputs come from count / scan / write passes; the bidding's
// outcome does not depend on the order of its atomics once each round's
// bidders are fixed before it starts (the reference decides that inside the
// racing kernel).
//
// Layout in HBM: one arena sized from the event's spacepoint count (nodes,
// edges up to max_edges_factor x nodes, the graph rows, the automaton's
// levels) and one sized from the path count, which the host reads back once
// in the middle of the run (the reference reads its counters back six times).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "seedgb.h"

namespace cg = cooperative_groups;

namespace {

constexpr uint32_t kMaxCca = 15u;       // gbts_consts::max_cca_iter
constexpr uint32_t kNodeBuffer = 128u;  // gbts_consts::node_buffer_length
constexpr int kEdgeThreads = 128;       // threads of one edge work item
constexpr int kThreads = 256;
constexpr int kScanThreads = 1024;
constexpr uint32_t kScanTile = 4u * kScanThreads;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 2.0f * kPi;
constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int32_t kPathCountLimit = 1 << 30;
constexpr uint32_t kGrid = 152u * 8u;
constexpr uint32_t kFlagSlots = 64u;  // automaton iterations, then bidding rounds  // grid-stride kernels: 8 blocks per SM

#define GRID_STRIDE(i, n) \
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// device-resident sizes and status of one run
enum Size : uint32_t {
    S_NODES = 0,
    S_ITEMS,
    S_UNITS,
    S_RECS,
    S_UNIT_NEXT,  // next unit for k_edge_masks' warps
    S_EDGES_MADE,
    S_EDGES,
    S_CONN,
    S_CONNECTED,
    S_TERMINUS,
    S_PATHS,
    S_PROPS,
    S_REJECTED,
    S_SEEDS,
    S_STATUS,
    S_BAD_INPUT,
    S_COUNT
};

struct Tables {
    seedgb_gbts_config c;
    uint32_t n_layers, n_eta, n_pairs, n_volumes, n_surfaces, n_tau_lut;
    const int8_t* layer_type;
    const uint32_t* eta_bin0;
    const uint32_t* n_eta_l;
    const float* min_eta;
    const float* eta_width;
    const uint32_t* pairs;
    const int16_t* vmap;
    const uint32_t* smap;
    const float* tau_lut;
};

// work buffers of one run
struct Work {
    // spacepoints
    float4* red;
    float* sp_phi;
    uint32_t* sp_cell;
    // cells and nodes
    uint32_t *cell_cnt, *cell_off, *cell_cur;
    uint32_t* node_sp;
    float4* node_p;
    float* node_phi;
    uint32_t* view;
    float* rads;
    // work items
    uint32_t *item_cnt, *item_off;
    uint4* items;
    float* item_dphi;
    uint32_t* item_eta;  // eta bin of bin 1, top bit: the bin holds a node wrapped to phi bin 0
    uint32_t *unit_cnt, *unit_off, *unit_pos, *unit_nrec;  // per (item, quarter)
    uint2* rec_a;        // records: (outer node index, first edge's position in the unit)
    ulonglong2* rec_m;   // records: inner-node mask
    // edges
    uint32_t *e_in, *e_out;
    float4* e_p;
    uint32_t *out_cnt, *lstart, *lcur, *links, *links_tmp;
    uint32_t *in_cnt, *instart, *incur, *in_list;  // the edges entering each node (by outer node)
    uint8_t* nnei;
    uint32_t *nei, *kept, *kbase;
    // graph and automaton
    uint32_t* graph;
    uint8_t* levels;
    int8_t* active;
    int32_t* opx;
    int16_t* opy;
    uint32_t *tflag, *tidx, *tpaths, *pbase;
    unsigned long long *ebid, *hbid;
    unsigned long long* tstate;  // scan tile states
    uint32_t* flags;  // per automaton iteration / bidding round: anything left to do
    // path-sized buffers
    int2* store;
    uint32_t *term_edge, *term_pos;
    uint32_t *fflag, *fidx;
    int32_t* fqual;
    int2* props;
    int8_t* ambi;
    uint8_t* bidder;
    uint32_t *ecount, *eoff;
    uint4* seeds3;
    unsigned long long* tstate_b;
    // sizes
    uint32_t* sz;
    uint64_t ecap;  // edge capacity (max_edges_factor x spacepoints)
    uint64_t pcap;  // path store capacity
};

__device__ __forceinline__ void set_status(uint32_t* sz, uint32_t s) { atomicMax(&sz[S_STATUS], s); }

__device__ __forceinline__ uint64_t field(uint64_t v, uint32_t shift, uint32_t bits) {
    const uint64_t m = bits >= 64 ? ~0ull : ((1ull << bits) - 1ull);
    return shift >= 64 ? 0 : ((v >> shift) & m);
}

// std::min / std::max as the reference calls them (comparison based)
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

// correctly rounded float atan2 / log: the double-precision result rounded
__device__ __forceinline__ float cr_atan2f(float y, float x) {
    return static_cast<float>(atan2(static_cast<double>(y), static_cast<double>(x)));
}
__device__ __forceinline__ float cr_logf(float x) {
    return static_cast<float>(log(static_cast<double>(x)));
}

// traccc::detail::wrap_phi (core/include/traccc/utils/trigonometric_helpers.hpp:18-38)
__device__ __forceinline__ float wrap_phi(float phi) {
    const float diff = phi - (-kPi);
    return ((0 <= diff) && (diff < kTwoPi)) ? phi : (phi - kTwoPi * floorf(diff / kTwoPi));
}

__device__ __forceinline__ uint32_t load_n(const uint32_t* n_dev, uint32_t n_host, uint32_t add) {
    return n_dev ? *n_dev + add : n_host;
}

// ---------------------------------------------------------------------------
// Exclusive scan of n values (n on the host or in device memory): out[i] =
// sum of in[0, i), out[n] = total, *total_dst = total.  Three launches over a
// grid sized for the capacity; blocks past n exit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t ws[32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += x;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    const uint32_t nw = blockDim.x >> 5;
    if (warp == 0) {
        uint32_t s = lane < nw ? ws[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= static_cast<uint32_t>(o)) s += x;
        }
        if (lane < nw) ws[lane] = s;
    }
    __syncthreads();
    const uint32_t before = warp ? ws[warp - 1] : 0u;
    *total = ws[nw - 1];
    __syncthreads();
    return before + incl - v;
}

// Single-pass scan with decoupled look-back: each block takes the next tile
// id from a running ticket (so every tile before it is already running),
// scans its tile, publishes the tile's sum, then walks back over earlier
// tiles' published sums until one holds an inclusive prefix.  A tile state
// is (epoch:30, flag:2, value:32); states of another scan (epoch) read as
// not yet published.  The wait for a predecessor is bounded: past the limit
// the run's status becomes SEEDGB_TIMEOUT.
constexpr uint32_t kFlagAggregate = 1u, kFlagPrefix = 2u;
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ unsigned long long tile_word(uint32_t epoch, uint32_t flag, uint32_t v) {
    return (static_cast<unsigned long long>(epoch & 0x3FFFFFFFu) << 34) |
           (static_cast<unsigned long long>(flag) << 32) | v;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan(const uint32_t* in, uint32_t* out, const uint32_t* n_dev, uint32_t n_host, uint32_t add,
       unsigned long long* state, unsigned long long* ticket, unsigned long long ticket_base,
       uint32_t epoch, uint32_t* total_dst, uint32_t* sz) {
    __shared__ uint32_t s_tile, s_prefix;
    if (threadIdx.x == 0) s_tile = static_cast<uint32_t>(atomicAdd(ticket, 1ull) - ticket_base);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t n = load_n(n_dev, n_host, add);
    const uint32_t n_tiles = n ? (n + kScanTile - 1) / kScanTile : 1u;
    if (tile >= n_tiles) return;
    const uint32_t base = tile * kScanTile;
    uint32_t v[4];
    uint32_t sum = 0;
    for (int j = 0; j < 4; ++j) {
        const uint32_t i = base + 4u * threadIdx.x + j;
        v[j] = i < n ? in[i] : 0u;
        sum += v[j];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(sum, &total);
    // look-back by the first warp: 32 predecessor states per step, nearest
    // first; the step stops at the nearest inclusive prefix, else adds the 32
    // aggregates and moves on; a state not yet published makes the warp
    // re-read (bounded)
    if (threadIdx.x < 32) {
        const uint32_t lane = threadIdx.x;
        if (tile != 0 && lane == 0) atomicExch(&state[tile], tile_word(epoch, kFlagAggregate, total));
        const unsigned long long want = epoch & 0x3FFFFFFFu;
        uint32_t prefix = 0;
        int hi = static_cast<int>(tile) - 1;  // nearest predecessor not yet added
        uint32_t spins = 0;
        while (hi >= 0) {
            const int j = hi - static_cast<int>(lane);
            uint32_t flag = kFlagPrefix, val = 0;  // lanes before tile 0: a zero prefix
            if (j >= 0) {
                const unsigned long long sv = *reinterpret_cast<volatile unsigned long long*>(&state[j]);
                flag = ((sv >> 34) == want) ? static_cast<uint32_t>(sv >> 32) & 3u : 0u;
                val = static_cast<uint32_t>(sv);
            }
            const unsigned not_ready = __ballot_sync(0xffffffffu, flag == 0u);
            const unsigned is_prefix = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
            // lanes up to the nearest prefix (lowest lane with one) count
            const uint32_t stop = is_prefix ? static_cast<uint32_t>(__ffs(is_prefix) - 1) : 31u;
            const unsigned needed = stop == 31u ? 0xffffffffu : ((2u << stop) - 1u);
            if (not_ready & needed) {
                if (++spins > kSpinLimit) {
                    if (lane == 0) set_status(sz, SEEDGB_TIMEOUT);
                    break;
                }
                __nanosleep(64);
                continue;
            }
            uint32_t part = lane <= stop ? val : 0u;
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
            prefix += part;
            if (is_prefix) break;
            hi -= 32;
        }
        if (lane == 0) {
            atomicExch(&state[tile], tile_word(epoch, kFlagPrefix, prefix + total));
            s_prefix = prefix;
            if (tile == n_tiles - 1u) {
                out[n] = prefix + total;
                if (total_dst) *total_dst = prefix + total;
            }
        }
    }
    __syncthreads();
    run += s_prefix;
    for (int j = 0; j < 4; ++j) {
        const uint32_t i = base + 4u * threadIdx.x + j;
        if (i < n) out[i] = run;
        run += v[j];
    }
}

// ---------------------------------------------------------------------------
// Nodes: gbts_count_spacepoints_by_layer, gbts_bin_spacepoints,
// gbts_sort_nodes, gbts_find_minmax_radius
// ---------------------------------------------------------------------------

// layer, eta bin, phi bin of every spacepoint
// (gbts_count_spacepoints_by_layer.ipp:32-113, gbts_bin_spacepoints.ipp:27-107)
__global__ void __launch_bounds__(kThreads)
k_classify(Tables T, seedgb_spacepoint_view sps, const uint64_t* link, const float* diam,
           uint32_t n_meas, Work w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sps.size) return;
    const seedgb_gbts_config& c = T.c;
    const float x = sps.global[3 * i], y = sps.global[3 * i + 1], z = sps.global[3 * i + 2];
    w.red[i] = make_float4(x, y, z, static_cast<float>(-CHAR_MAX - 1));
    w.sp_cell[i] = kInvalid;
    const uint32_t m = sps.measurement_index_1[i];
    if (m >= n_meas) {
        atomicAdd(&w.sz[S_BAD_INPUT], 1u);
        return;
    }
    const uint64_t lk = link[m];
    const uint32_t volume = static_cast<uint32_t>(field(lk, c.volume_shift, c.volume_bits));
    const int16_t begin_or_bin = (volume < T.n_volumes) ? T.vmap[volume] : SHRT_MAX;
    if (begin_or_bin == SHRT_MAX) return;
    uint32_t layer = 0u;
    if (begin_or_bin < 0) {
        const uint32_t sidx = static_cast<uint32_t>(field(lk, c.index_shift, c.index_bits));
        for (uint32_t s = static_cast<uint32_t>(-1 * (begin_or_bin + 1)); s < T.n_surfaces; s++) {
            if (T.smap[2 * s] == sidx) {
                layer = T.smap[2 * s + 1];
                break;
            }
        }
    } else {
        layer = static_cast<uint32_t>(begin_or_bin);
    }
    if (layer >= T.n_layers) return;
    float d = diam[m];
    const int type = static_cast<int>(T.layer_type[layer]);
    if (type == 1 && d > c.type1_max_width) return;
    d = (c.doTauCut && type != 0) ? static_cast<float>(-1 * type) : d;
    w.red[i].w = d;
    const uint32_t bin0 = T.eta_bin0[layer];
    const uint32_t nb = T.n_eta_l[layer];
    uint32_t eta_index;
    if (nb == 1u) {
        eta_index = bin0;
    } else {
        const float r = sqrtf(x * x + y * y);
        const float t1 = z / r;
        const float eta = -cr_logf(sqrtf(1.0f + t1 * t1) - t1);
        const uint32_t bi = static_cast<uint32_t>(
            smax(0.0f, smin((eta - T.min_eta[layer]) / T.eta_width[layer],
                            static_cast<float>(nb - 1u))));
        eta_index = bin0 + bi;
    }
    const float inv_slice = 1.0f / (kTwoPi / static_cast<float>(c.n_phi_bins));
    const float phi = cr_atan2f(y, x);
    uint32_t pb = static_cast<uint32_t>((phi + kPi) * inv_slice);
    if (pb >= c.n_phi_bins) pb -= c.n_phi_bins;
    const uint32_t cell = pb + c.n_phi_bins * eta_index;
    w.sp_phi[i] = phi;
    w.sp_cell[i] = cell;
    atomicAdd(&w.cell_cnt[cell], 1u);
}

__global__ void __launch_bounds__(kThreads) k_scatter(uint32_t n_sp, Work w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_sp) return;
    const uint32_t cell = w.sp_cell[i];
    if (cell == kInvalid) return;
    w.node_sp[w.cell_off[cell] + atomicAdd(&w.cell_cur[cell], 1u)] = i;
}

// the nodes of a cell in ascending spacepoint index (insertion sort per cell)
__global__ void __launch_bounds__(kThreads) k_sort_cells(uint32_t n_cells, Work w) {
    const uint32_t cidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (cidx >= n_cells) return;
    const uint32_t b = w.cell_off[cidx], e = w.cell_off[cidx + 1];
    for (uint32_t i = b + 1; i < e; ++i) {
        const uint32_t v = w.node_sp[i];
        uint32_t j = i;
        while (j > b && w.node_sp[j - 1] > v) {
            w.node_sp[j] = w.node_sp[j - 1];
            --j;
        }
        w.node_sp[j] = v;
    }
}

// gbts_sort_nodes.ipp:24-101: (tau_min, tau_max, r, z) and phi of each node
__global__ void __launch_bounds__(kThreads) k_node_params(Tables T, Work w) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w.sz[S_NODES]) return;
    const seedgb_gbts_config& ap = T.c;
    const uint32_t s = w.node_sp[k];
    const float4 sp = w.red[s];
    const float r = sqrtf(sp.x * sp.x + sp.y * sp.y);
    float min_tau = 0.0f;
    float max_tau = ap.maxTau;
    if (sp.w > 0) {
        if (ap.useTauLUT) {
            const int tau_bin = 5 * static_cast<int>(floorf(ap.tau_lut_inv_bin * sp.w) - 1.0f);
            if (tau_bin > -1 && tau_bin < static_cast<int>(ap.tauLutSize)) {
                min_tau = T.tau_lut[static_cast<uint32_t>(tau_bin) + 1u];
                max_tau = T.tau_lut[static_cast<uint32_t>(tau_bin) + 2u];
            }
            if (max_tau < 0.0f) max_tau = ap.maxTau;
            if (min_tau < 0.0f) min_tau = 0.0f;
        } else {
            min_tau = ap.tMin_slope * (sp.w - ap.offset);
            max_tau = ap.tMax_min + ap.tMax_correction / (sp.w + ap.offset) +
                      ap.tMax_slope * (sp.w - ap.offset);
        }
    }
    w.node_p[k] = make_float4(min_tau, max_tau, r, sp.z);
    w.node_phi[k] = w.sp_phi[s];
}

// node ranges of the eta bins and their radius range
// (gbts_find_minmax_radius.ipp:21-54); one warp per eta bin
__global__ void __launch_bounds__(kThreads) k_eta_bins(uint32_t n_eta, uint32_t n_phi, Work w) {
    const uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (e >= n_eta) return;
    const uint32_t b = w.cell_off[e * n_phi], en = w.cell_off[(e + 1) * n_phi];
    float mn = 1e8f, mx = -1e8f;
    for (uint32_t k = b + lane; k < en; k += 32) {
        const float r = w.node_p[k].z;
        mx = fmaxf(r, mx);
        mn = fminf(r, mn);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    if (lane == 0) {
        w.view[2 * e] = b;
        w.view[2 * e + 1] = en;
        w.rads[2 * e] = mn;
        w.rads[2 * e + 1] = mx;
    }
}

// ---------------------------------------------------------------------------
// Work items (gbts_seeding_algorithm.cpp:215-283): bin pairs with their phi
// window, bin 1 split into chunks of 128 nodes
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool pair_window(const Tables& T, const Work& w, uint32_t p,
                                            uint32_t& chunks, float& dphi) {
    const uint32_t bin1 = T.pairs[2 * p], bin2 = T.pairs[2 * p + 1];
    const uint32_t b1 = w.view[2 * bin1], e1 = w.view[2 * bin1 + 1];
    chunks = 0;
    if (b1 == e1 || w.view[2 * bin2] == w.view[2 * bin2 + 1]) return false;
    const float rb1 = w.rads[2 * bin1];
    const float rb2 = w.rads[2 * bin2 + 1];
    const float maxDeltaR = fabsf(rb2 - rb1);
    const seedgb_gbts_config& c = T.c;
    dphi = c.min_delta_phi + c.dphi_coeff * maxDeltaR;
    if (maxDeltaR < c.low_dr_threshold) dphi = c.min_delta_phi_low_dr + c.dphi_coeff_low_dr * maxDeltaR;
    chunks = (e1 - b1 + kNodeBuffer - 1u) / kNodeBuffer;
    return true;
}

__global__ void __launch_bounds__(kThreads) k_items_count(Tables T, Work w) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= T.n_pairs) return;
    uint32_t chunks;
    float dphi;
    pair_window(T, w, p, chunks, dphi);
    w.item_cnt[p] = chunks;
}

__global__ void __launch_bounds__(kThreads) k_items_fill(Tables T, Work w) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= T.n_pairs) return;
    uint32_t chunks;
    float dphi;
    if (!pair_window(T, w, p, chunks, dphi)) return;
    const uint32_t bin1 = T.pairs[2 * p], bin2 = T.pairs[2 * p + 1];
    const uint32_t b1 = w.view[2 * bin1], e1 = w.view[2 * bin1 + 1];
    const uint32_t o = w.item_off[p];
    // a node whose phi rounds into bin n_phi is wrapped to bin 0, ahead of
    // nodes of smaller phi: the window walk of such a chunk takes no short cut
    bool wrapped = false;
    const uint32_t c0 = bin1 * T.c.n_phi_bins;
    for (uint32_t k = w.cell_off[c0]; k < w.cell_off[c0 + 1] && !wrapped; ++k) wrapped = w.node_phi[k] > 0.0f;
    for (uint32_t j = 0; j < chunks; ++j) {
        const uint32_t b = b1 + j * kNodeBuffer;
        const uint32_t e = (e1 - b > kNodeBuffer) ? b + kNodeBuffer : e1;
        w.items[o + j] = make_uint4(b, e, w.view[2 * bin2], w.view[2 * bin2 + 1]);
        w.item_dphi[o + j] = dphi;
        w.item_eta[o + j] = bin1 | (wrapped ? 0x80000000u : 0u);
    }
}

// ---------------------------------------------------------------------------
// Edges (gbts_make_graph_edges.ipp:31-239)
// ---------------------------------------------------------------------------
// The cuts are a conjunction of tests on the same inputs, so their order does
// not change which edges pass: the phi-difference test (no division; the
// candidate window is wider than deltaPhi by a phi bin on each side) runs
// before the divisions.
__device__ __forceinline__ bool edge_test(float4 np1, float4 np2, float phi1, float phi2,
                                          float deltaPhi, const seedgb_gbts_config& ap,
                                          float4& out) {
    const float dr = np2.z - np1.z;
    if (dr < ap.minDeltaRadius) return false;
    const float dphi = wrap_phi(phi2 - phi1);
    if (fabsf(dphi) > deltaPhi) return false;
    const float dz = np2.w - np1.w;
    const float tau = dz / dr;
    const float ftau = fabsf(tau);
    if ((ftau < np2.x) || (ftau > np2.y)) return false;
    if ((ftau < np1.x) || (ftau > np1.y)) return false;
    const float z0 = np1.w - np1.z * tau;
    if ((z0 < ap.min_z0) || (z0 > ap.max_z0)) return false;
    const float zouter = z0 + ap.maxOuterRadius * tau;
    if (zouter < ap.cut_zMinU || zouter > ap.cut_zMaxU) return false;
    const float curv = dphi / dr;
    const float d0_for_max_curv = np1.z * np2.z * (fabsf(curv) - ap.max_Kappa);
    const float d0_max = (ftau < 4.0f) ? ap.low_Kappa_d0 : ap.high_Kappa_d0;
    if (d0_for_max_curv > d0_max) return false;
    out = make_float4(sqrtf(1.0f + tau * tau) - tau, curv, phi2 + curv * np2.z,
                      phi1 + curv * np1.z);
    return true;
}

struct ItemCtx {
    uint32_t b1, n1, b2;
    float dphi, phi0, phiN, pbw, brk;
    const uint32_t* bin_first;  // first node of each phi bin of the chunk's eta bin, or null
    float inv_slice;
    uint32_t n_phi;
};

// one outer node of a work item: the reference's window walk with the
// thread's sliding start (last_n1) and stop flag (done); counts the edges, and
// writes them from `pos` on when WRITE
template <bool WRITE>
__device__ __forceinline__ uint32_t walk(const ItemCtx& it, uint32_t n2Idx, uint32_t& last_n1,
                                         bool& done, const float* s_phi, const float4* s_np,
                                         const Work& w, const seedgb_gbts_config& c,
                                         uint64_t pos, uint64_t cap, uint32_t* s_cnt) {
    const uint32_t g2 = it.b2 + n2Idx;
    const float phi2 = w.node_phi[g2];
    uint32_t n1Idx = last_n1;
    float min_phi1 = phi2 - it.dphi;
    float max_phi1 = phi2 + it.dphi;
    if (min_phi1 < -kPi) min_phi1 += kTwoPi;
    if (max_phi1 > kPi) max_phi1 -= kTwoPi;
    const bool boundary = max_phi1 < min_phi1;
    max_phi1 += it.pbw;
    min_phi1 -= it.pbw;
    if (!boundary) {
        if (it.phi0 > max_phi1) return 0;
        if (it.phiN < min_phi1) {
            if (it.phi0 > it.brk) done = true;
            return 0;
        }
        // every node of a phi bin below the bin of min_phi1 has phi1 <
        // min_phi1 (the bin is a monotone function of phi), so the walk
        // would step over it: start at the first node of that bin
        const float x = (min_phi1 + kPi) * it.inv_slice;
        if (it.bin_first && x >= 1.0f) {
            const uint32_t pb = static_cast<uint32_t>(x);
            if (pb < it.n_phi) {
                const uint32_t f = it.bin_first[pb];
                const uint32_t jump = f > it.b1 ? (f - it.b1 < it.n1 ? f - it.b1 : it.n1) : 0u;
                if (jump > n1Idx) n1Idx = jump;
            }
        }
    } else {
        if (it.phi0 < max_phi1) {
            n1Idx = 0u;
        } else if (it.phiN < min_phi1) {
            return 0;
        }
    }
    const float4 np2 = w.node_p[g2];
    uint32_t cnt = 0;
    for (; n1Idx < it.n1; n1Idx++) {
        const float phi1 = s_phi[n1Idx];
        if (!boundary) {
            if (phi1 > max_phi1) break;
            if (phi1 < min_phi1) continue;
        } else if (phi1 > max_phi1 && phi1 < min_phi1) {
            continue;
        }
        last_n1 = n1Idx;
        float4 ep;
        if (edge_test(s_np[n1Idx], np2, phi1, phi2, it.dphi, c, ep)) {
            if (WRITE) {
                const uint64_t q = pos + cnt;
                if (q < cap) {
                    w.e_in[q] = it.b1 + n1Idx;
                    w.e_out[q] = g2;
                    w.e_p[q] = ep;
                    atomicAdd(&s_cnt[n1Idx], 1u);
                }
            }
            ++cnt;
        }
    }
    return cnt;
}

// The same walk recording which inner nodes pair with the outer node: bit
// n1Idx of (lo, hi) (the chunk has at most 128 nodes); the candidate loop
// only sets bits, so it runs without branches on the result.
__device__ __forceinline__ uint32_t walk_mask(const ItemCtx& it, uint32_t n2Idx, uint32_t& last_n1,
                                              bool& done, const float* s_phi, const float4* s_np,
                                              const Work& w, const seedgb_gbts_config& c,
                                              unsigned long long& lo, unsigned long long& hi) {
    lo = 0ull;
    hi = 0ull;
    const uint32_t g2 = it.b2 + n2Idx;
    const float phi2 = w.node_phi[g2];
    uint32_t n1Idx = last_n1;
    float min_phi1 = phi2 - it.dphi;
    float max_phi1 = phi2 + it.dphi;
    if (min_phi1 < -kPi) min_phi1 += kTwoPi;
    if (max_phi1 > kPi) max_phi1 -= kTwoPi;
    const bool boundary = max_phi1 < min_phi1;
    max_phi1 += it.pbw;
    min_phi1 -= it.pbw;
    if (!boundary) {
        if (it.phi0 > max_phi1) return 0;
        if (it.phiN < min_phi1) {
            if (it.phi0 > it.brk) done = true;
            return 0;
        }
        const float x = (min_phi1 + kPi) * it.inv_slice;
        if (it.bin_first && x >= 1.0f) {
            const uint32_t pb = static_cast<uint32_t>(x);
            if (pb < it.n_phi) {
                const uint32_t f = it.bin_first[pb];
                const uint32_t jump = f > it.b1 ? (f - it.b1 < it.n1 ? f - it.b1 : it.n1) : 0u;
                if (jump > n1Idx) n1Idx = jump;
            }
        }
    } else {
        if (it.phi0 < max_phi1) {
            n1Idx = 0u;
        } else if (it.phiN < min_phi1) {
            return 0;
        }
    }
    const float4 np2 = w.node_p[g2];
    for (; n1Idx < it.n1; n1Idx++) {
        const float phi1 = s_phi[n1Idx];
        if (!boundary) {
            if (phi1 > max_phi1) break;
            if (phi1 < min_phi1) continue;
        } else if (phi1 > max_phi1 && phi1 < min_phi1) {
            continue;
        }
        last_n1 = n1Idx;
        float4 ep;
        const bool pass = edge_test(s_np[n1Idx], np2, phi1, phi2, it.dphi, c, ep);
        const unsigned long long bit = pass ? (1ull << (n1Idx & 63u)) : 0ull;
        lo |= n1Idx < 64u ? bit : 0ull;
        hi |= n1Idx < 64u ? 0ull : bit;
    }
    return static_cast<uint32_t>(__popcll(lo) + __popcll(hi));
}

// The parameters of an edge that passed (exp(-eta), curvature, phi
// extrapolated at node 2 and at node 1), the same float operations as in
// edge_test, so a recomputation gives the same bits.
__device__ __forceinline__ float4 edge_params(float4 np1, float4 np2, float phi1, float phi2) {
    const float dr = np2.z - np1.z;
    const float tau = (np2.w - np1.w) / dr;
    const float curv = wrap_phi(phi2 - phi1) / dr;
    return make_float4(sqrtf(1.0f + tau * tau) - tau, curv, phi2 + curv * np2.z, phi1 + curv * np1.z);
}

// Edges of one work item, thread t (of 128) taking the outer nodes t,
// t + 128, ... with the reference's sliding-window state; an item's edges in
// thread order, then outer node, then inner node.  The four warps of a block
// work independently: a warp takes one quarter of an item (threads 32q ...
// 32q + 31, a "unit") and stages its own copy of the item's bin-1 chunk, so
// only warp barriers remain.  k_edge_masks walks once and keeps, per outer
// node with edges, a record (outer node, inner-node bit mask, the position of
// its first edge within the unit); after a scan over the units' edge counts,
// k_edge_expand writes one edge per set bit.  A unit with more than
// kRecStage records is walked again by k_edge_expand (count, then write).
// The walk's warps take units from a counter, so a costly unit late in the
// order holds up only its own warp.
constexpr int kEdgeWarps = kEdgeThreads / 32;
constexpr uint32_t kRecStage = 128;
constexpr uint32_t kUnitOverflow = 0xFFFFFFFFu;

__device__ __forceinline__ void setup_item(const Tables& T, const Work& w, uint32_t item, uint32_t lane,
                                           ItemCtx& it, uint32_t& n2, float* s_phi, float4* s_np,
                                           uint32_t* s_cnt) {
    const uint4 r = w.items[item];
    it.b1 = r.x;
    it.n1 = r.y - r.x;
    it.b2 = r.z;
    n2 = r.w - r.z;
    it.dphi = w.item_dphi[item];
    const uint32_t em = w.item_eta[item];
    it.bin_first = (em & 0x80000000u) ? nullptr : w.cell_off + (em & 0x7FFFFFFFu) * T.c.n_phi_bins;
    it.n_phi = T.c.n_phi_bins;
    it.inv_slice = 1.0f / (kTwoPi / static_cast<float>(T.c.n_phi_bins));
    __syncwarp();
    for (uint32_t k = lane; k < kNodeBuffer; k += 32) {
        if (k < it.n1) {
            s_np[k] = w.node_p[it.b1 + k];
            s_phi[k] = w.node_phi[it.b1 + k];
        }
        if (s_cnt) s_cnt[k] = 0;
    }
    __syncwarp();
    it.phi0 = s_phi[0];
    it.phiN = s_phi[it.n1 - 1u];
    it.pbw = kTwoPi / static_cast<float>(T.c.n_phi_bins);
    it.brk = it.dphi + it.pbw - kPi;
}

__device__ __forceinline__ uint32_t warp_exclusive(uint32_t v, uint32_t lane, uint32_t& total) {
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += x;
    }
    total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - v;
}

__global__ void __launch_bounds__(kEdgeThreads, 8) k_edge_masks(Tables T, Work w) {
    __shared__ float s_phi_all[kEdgeWarps][kNodeBuffer];
    __shared__ float4 s_np_all[kEdgeWarps][kNodeBuffer];
    __shared__ uint2 s_ra_all[kEdgeWarps][kRecStage];        // (lane << 27 | n2Idx, lane's edges before)
    __shared__ ulonglong2 s_rm_all[kEdgeWarps][kRecStage];   // the inner-node mask
    __shared__ uint32_t s_nrec_all[kEdgeWarps];
    __shared__ uint32_t s_excl_all[kEdgeWarps][32];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    float* s_phi = s_phi_all[wid];
    float4* s_np = s_np_all[wid];
    uint2* s_ra = s_ra_all[wid];
    ulonglong2* s_rm = s_rm_all[wid];
    uint32_t* s_excl = s_excl_all[wid];
    const uint32_t n_items = w.sz[S_ITEMS];
    if (blockIdx.x == 0 && threadIdx.x == 0) w.sz[S_UNITS] = n_items * kEdgeWarps;
    const uint32_t n_units = n_items * kEdgeWarps;
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(&w.sz[S_UNIT_NEXT], 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= n_units) break;
        ItemCtx it;
        uint32_t n2;
        setup_item(T, w, u / kEdgeWarps, lane, it, n2, s_phi, s_np, nullptr);
        if (lane == 0) s_nrec_all[wid] = 0;
        __syncwarp();
        const uint32_t t = 32u * (u % kEdgeWarps) + lane;
        uint32_t last_n1 = 0u, cnt = 0;
        bool done = false;
        for (uint32_t n2Idx = t; n2Idx < n2 && !done; n2Idx += kEdgeThreads) {
            unsigned long long lo, hi;
            const uint32_t k = walk_mask(it, n2Idx, last_n1, done, s_phi, s_np, w, T.c, lo, hi);
            if (k) {
                const uint32_t r = atomicAdd(&s_nrec_all[wid], 1u);
                if (r < kRecStage) {
                    s_ra[r] = make_uint2((lane << 27) | n2Idx, cnt);
                    s_rm[r] = make_ulonglong2(lo, hi);
                }
                cnt += k;
            }
        }
        __syncwarp();
        uint32_t total;
        s_excl[lane] = warp_exclusive(cnt, lane, total);
        const uint32_t nrec = s_nrec_all[wid];
        bool ok = nrec <= kRecStage && n2 < (1u << 27);
        uint32_t pos0 = 0;
        if (ok) {
            if (lane == 0) pos0 = atomicAdd(&w.sz[S_RECS], nrec);
            pos0 = __shfl_sync(0xffffffffu, pos0, 0);
            ok = static_cast<uint64_t>(pos0) + nrec <= w.ecap;
        }
        __syncwarp();
        if (ok)
            for (uint32_t r = lane; r < nrec; r += 32) {
                const uint2 a = s_ra[r];
                w.rec_a[pos0 + r] = make_uint2(a.x & ((1u << 27) - 1u), s_excl[a.x >> 27] + a.y);
                w.rec_m[pos0 + r] = s_rm[r];
            }
        if (lane == 0) {
            w.unit_cnt[u] = total;
            w.unit_pos[u] = ok ? pos0 : kUnitOverflow;
            w.unit_nrec[u] = nrec;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kEdgeThreads) k_edge_expand(Tables T, Work w) {
    __shared__ float s_phi_all[kEdgeWarps][kNodeBuffer];
    __shared__ float4 s_np_all[kEdgeWarps][kNodeBuffer];
    __shared__ uint32_t s_cnt_all[kEdgeWarps][kNodeBuffer];  // edges per inner node of the chunk
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    float* s_phi = s_phi_all[wid];
    float4* s_np = s_np_all[wid];
    uint32_t* s_cnt = s_cnt_all[wid];
    const uint64_t by_nodes = static_cast<uint64_t>(T.c.max_edges_factor) * w.sz[S_NODES];
    const uint64_t cap = by_nodes < w.ecap ? by_nodes : w.ecap;
    const uint32_t n_units = w.sz[S_UNITS];
    for (uint32_t u = blockIdx.x * kEdgeWarps + wid; u < n_units; u += gridDim.x * kEdgeWarps) {
        if (w.unit_cnt[u] == 0) continue;
        ItemCtx it;
        uint32_t n2;
        setup_item(T, w, u / kEdgeWarps, lane, it, n2, s_phi, s_np, s_cnt);
        const uint64_t off = w.unit_off[u];
        const uint32_t pos0 = w.unit_pos[u];
        if (pos0 != kUnitOverflow) {
            const uint32_t nrec = w.unit_nrec[u];
            for (uint32_t r = lane; r < nrec; r += 32) {
                const uint2 a = w.rec_a[pos0 + r];
                const ulonglong2 m = w.rec_m[pos0 + r];
                const uint32_t g2 = it.b2 + a.x;
                const float4 np2 = w.node_p[g2];
                const float phi2 = w.node_phi[g2];
                uint64_t q = off + a.y;
                for (int half = 0; half < 2; ++half) {
                    unsigned long long bits = half ? m.y : m.x;
                    while (bits) {
                        const uint32_t i1 = (half ? 64u : 0u) + static_cast<uint32_t>(__ffsll(bits) - 1);
                        bits &= bits - 1ull;
                        if (q < cap) {
                            w.e_in[q] = it.b1 + i1;
                            w.e_out[q] = g2;
                            w.e_p[q] = edge_params(s_np[i1], np2, s_phi[i1], phi2);
                            atomicAdd(&s_cnt[i1], 1u);
                        }
                        ++q;
                    }
                }
            }
        } else {
            // more records than the stage held: count per thread, then write
            const uint32_t t = 32u * (u % kEdgeWarps) + lane;
            uint32_t last_n1 = 0u, cnt = 0;
            bool done = false;
            for (uint32_t n2Idx = t; n2Idx < n2 && !done; n2Idx += kEdgeThreads)
                cnt += walk<false>(it, n2Idx, last_n1, done, s_phi, s_np, w, T.c, 0, 0, s_cnt);
            uint32_t total;
            const uint64_t pos = off + warp_exclusive(cnt, lane, total);
            const uint32_t want = cnt;
            last_n1 = 0u;
            done = false;
            cnt = 0;
            for (uint32_t n2Idx = t; n2Idx < n2 && !done && cnt < want; n2Idx += kEdgeThreads)
                cnt += walk<true>(it, n2Idx, last_n1, done, s_phi, s_np, w, T.c, pos + cnt, cap, s_cnt);
        }
        __syncwarp();
        for (uint32_t k = lane; k < it.n1; k += 32)
            if (s_cnt[k]) atomicAdd(&w.out_cnt[it.b1 + k], s_cnt[k]);
    }
}

// gbts_link_graph_edges.ipp:22-44: the edges leaving each node (by inner
// node), first in arrival order ...
// (the kept edges: min(made, max_edges_factor x nodes, capacity))
__global__ void k_edges_kept(Tables T, Work w) {
    const uint64_t by_nodes = static_cast<uint64_t>(T.c.max_edges_factor) * w.sz[S_NODES];
    uint64_t n = w.sz[S_EDGES_MADE];
    if (by_nodes < n) n = by_nodes;
    if (w.ecap < n) n = w.ecap;
    w.sz[S_EDGES] = static_cast<uint32_t>(n);
}

__global__ void __launch_bounds__(kThreads) k_link_fill(Work w) {
    GRID_STRIDE(e, w.sz[S_EDGES]) {
        const uint32_t n1 = w.e_in[e];
        w.links_tmp[w.lstart[n1] + atomicAdd(&w.lcur[n1], 1u)] = e;
        atomicAdd(&w.in_cnt[w.e_out[e]], 1u);
        w.kept[e] = 0u;
    }
}

// the edges entering each node, in any order (the matching of an edge does
// not depend on the other edges entering its outer node)
__global__ void __launch_bounds__(kThreads) k_in_fill(Work w) {
    GRID_STRIDE(e, w.sz[S_EDGES]) {
        const uint32_t n2 = w.e_out[e];
        w.in_list[w.instart[n2] + atomicAdd(&w.incur[n2], 1u)] = e;
    }
}

// ... then in ascending edge index: one warp per node, each edge placed at
// its rank (the edge indices of a list are distinct)
__global__ void __launch_bounds__(kThreads) k_link_sort(Work w) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t n = w.sz[S_NODES];
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n;
         k += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t b = w.lstart[k], L = w.lstart[k + 1] - b;
        const uint32_t* src = w.links_tmp + b;
        for (uint32_t i = lane; i < L; i += 32) {
            const uint32_t v = src[i];
            uint32_t r = 0;
            for (uint32_t j = 0; j < L; ++j) r += src[j] < v;
            w.links[b + r] = v;
        }
    }
}

// gbts_match_graph_edges.ipp:29-118: each edge keeps the first max_num_neighbours
// edges leaving its outer node (in link order) that pass the tau-ratio, phi
// and curvature cuts.  Done per node: one warp stages the node's outgoing
// edges (the candidates) in shared memory and its lanes match the edges
// entering the node against them; lists longer than the stage read the rest
// from global memory.  Every edge enters exactly one node, so every edge is
// matched once.
constexpr uint32_t kMatchStage = 128;
constexpr int kMatchWarps = kThreads / 32;

__global__ void __launch_bounds__(kThreads) k_match_nodes(Tables T, Work w) {
    __shared__ uint32_t s_e2_all[kMatchWarps][kMatchStage];
    __shared__ float4 s_p2_all[kMatchWarps][kMatchStage];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    uint32_t* s_e2 = s_e2_all[wid];
    float4* s_p2 = s_p2_all[wid];
    const seedgb_gbts_config& c = T.c;
    const uint32_t M = c.max_num_neighbours;
    const uint32_t n_nodes = w.sz[S_NODES];
    for (uint32_t n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; n < n_nodes;
         n += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t i0 = w.instart[n], ni = w.instart[n + 1] - i0;
        if (ni == 0) continue;
        const uint32_t link_begin = w.lstart[n];
        const uint32_t nLinks = w.lstart[n + 1] - link_begin;
        const uint32_t staged = nLinks < kMatchStage ? nLinks : kMatchStage;
        __syncwarp();
        for (uint32_t k = lane; k < staged; k += 32) {
            const uint32_t e2 = w.links[link_begin + k];
            s_e2[k] = e2;
            s_p2[k] = w.e_p[e2];
        }
        __syncwarp();
        for (uint32_t i = lane; i < ni; i += 32) {
            const uint32_t e = w.in_list[i0 + i];
            uint32_t num_nei = 0;
            if (nLinks != 0u) {
                const float4 p1 = w.e_p[e];
                const float uat_2 = 1.0f / p1.x;
                const float Phi2 = p1.z;
                const float curv2 = p1.y;
                for (uint32_t k = 0u; k < nLinks; k++) {
                    if (num_nei >= M) break;
                    const bool st = k < kMatchStage;
                    const uint32_t e2 = st ? s_e2[k] : w.links[link_begin + k];
                    const float4 p2 = st ? s_p2[k] : w.e_p[e2];
                    const float tau_ratio = p2.x * uat_2 - 1.0f;
                    if (fabsf(tau_ratio) > c.cut_tau_ratio_max) continue;
                    const float dPhi = wrap_phi(Phi2 - p2.w);
                    if (fabsf(dPhi) > c.cut_dphi_max) continue;
                    const float dcurv = curv2 - p2.y;
                    if (fabsf(dcurv) > c.cut_dcurv_max) continue;
                    w.nei[static_cast<uint64_t>(M) * e + num_nei] = e2;
                    w.kept[e2] = 1u;
                    ++num_nei;
                }
            }
            w.nnei[e] = static_cast<uint8_t>(num_nei);
            if (num_nei != 0) {
                w.kept[e] = 1u;
                atomicAdd(&w.sz[S_CONN], num_nei);
            }
        }
    }
}

// gbts_compress_graph.ipp:22-68: rows [outer sp, inner sp, nNei, neighbours]
__global__ void __launch_bounds__(kThreads) k_compress(Tables T, Work w) {
    GRID_STRIDE(e, w.sz[S_EDGES]) {
        if (!w.kept[e]) continue;
        const uint32_t M = T.c.max_num_neighbours;
        uint32_t* row = w.graph + static_cast<uint64_t>(3u + M) * w.kbase[e];
        row[0] = w.node_sp[w.e_out[e]];
        row[1] = w.node_sp[w.e_in[e]];
        const uint32_t nn = w.nnei[e];
        row[2] = nn;
        for (uint32_t k = 0; k < nn; ++k)
            row[3 + k] = w.kbase[w.nei[static_cast<uint64_t>(M) * e + k]];
    }
}

// ---------------------------------------------------------------------------
// Longest chains: gbts_run_cca_iteration.ipp:23-101 (one launch per iteration)
// ---------------------------------------------------------------------------
// returns whether this thread left an edge active for the next iteration
__device__ __forceinline__ bool cca_step(const Tables& T, const Work& w, uint32_t iter) {
    bool more = false;
    GRID_STRIDE(e, w.sz[S_CONNECTED]) {
    if (iter != 0 && w.active[e] != static_cast<int8_t>(iter)) continue;
    const uint32_t esz = 3u + T.c.max_num_neighbours;
    const uint32_t* row = w.graph + static_cast<uint64_t>(esz) * e;
    const uint32_t toggle = iter % 2;
    const uint8_t* lload = w.levels + toggle * w.ecap;
    uint8_t* lstore = w.levels + (1u - toggle) * w.ecap;
    const uint32_t nN = row[2];
    uint8_t next_level = lload[e];
    bool change = false;
    for (uint32_t k = 0; k < nN; k++) {
        const uint8_t f = lload[row[3 + k]];
        if (next_level == f) {
            next_level = static_cast<uint8_t>(f + 1);
            change = true;
            break;
        }
    }
    if (change) {
        if (iter == kMaxCca - 1) {
            w.opy[e] = -1;
            w.active[e] = -1;
        } else {
            w.active[e] = static_cast<int8_t>(iter + 1u);
            more = true;
        }
    } else {
        w.active[e] = -1;
        int64_t out_paths = 0;
        for (uint32_t k = 0; k < nN; ++k) {
            const uint32_t n = row[3 + k];
            if (next_level == 1 + w.levels[n]) out_paths += 1 + w.opx[n];
            w.opy[n] = -1;
        }
        if (out_paths > kPathCountLimit) {
            out_paths = kPathCountLimit;
            set_status(w.sz, SEEDGB_CAPACITY_OVERFLOW);
        }
        w.opx[e] = static_cast<int32_t>(out_paths);
        w.opy[e] = static_cast<int16_t>((next_level >= T.c.minLevel) - 1);
    }
    lstore[e] = next_level;
    }
    return more;
}

// the fifteen iterations in one cooperative launch, a grid barrier between them
// (an iteration that leaves no edge active ends the automaton: the
// remaining iterations would change nothing)
// 1024-thread blocks: full occupancy with a quarter of the blocks arriving at
// each grid barrier
constexpr int kCcaThreads = 1024;
__global__ void __launch_bounds__(kCcaThreads) k_cca_all(Tables T, Work w) {
    cg::grid_group g = cg::this_grid();
    for (uint32_t iter = 0; iter < kMaxCca; ++iter) {
        const bool more = cca_step(T, w, iter);
        if (__syncthreads_or(more) && threadIdx.x == 0) w.flags[iter] = 1u;
        g.sync();
        if (w.flags[iter] == 0u) break;
    }
}

// gbts_count_terminus_edges.ipp:22-46
__global__ void __launch_bounds__(kThreads) k_term_flags(Work w) {
    GRID_STRIDE(e, w.sz[S_CONNECTED]) {
        const bool t = w.opy[e] != -1;
        w.tflag[e] = t ? 1u : 0u;
        w.tpaths[e] = t ? static_cast<uint32_t>(w.opx[e]) : 0u;
    }
}

// gbts_add_terminus_to_path_store.ipp:21-44
__global__ void __launch_bounds__(kThreads) k_term_fill(Work w) {
    GRID_STRIDE(e, w.sz[S_CONNECTED]) {
        if (!w.tflag[e]) continue;
        const uint32_t ti = w.tidx[e];
        w.store[ti] = make_int2(static_cast<int>(e), -1);
        w.term_edge[ti] = e;
        w.term_pos[ti] = w.sz[S_TERMINUS] + w.pbase[e];
    }
}

// gbts_fill_path_store.ipp:24-163 as a depth-first pre-order walk below each
// terminus edge: the children of an entry are its neighbours one level down
__global__ void __launch_bounds__(kThreads) k_dfs(Tables T, Work w) {
    const uint32_t ti = blockIdx.x * blockDim.x + threadIdx.x;
    if (ti >= w.sz[S_TERMINUS]) return;
    const uint32_t esz = 3u + T.c.max_num_neighbours;
    const uint64_t end = static_cast<uint64_t>(w.sz[S_TERMINUS]) + w.sz[S_PATHS];
    uint32_t se[kMaxCca + 2], sk[kMaxCca + 2];
    int32_t si[kMaxCca + 2];
    uint64_t pos = w.term_pos[ti];
    int d = 0;
    se[0] = w.term_edge[ti];
    si[0] = static_cast<int32_t>(ti);
    sk[0] = 0;
    while (d >= 0) {
        const uint32_t e = se[d];
        const uint32_t* row = w.graph + static_cast<uint64_t>(esz) * e;
        if (sk[d] >= row[2]) {
            --d;
            continue;
        }
        const uint32_t n = row[3 + sk[d]++];
        if (w.levels[e] != w.levels[n] + 1) continue;
        if (pos >= end || d + 1 > static_cast<int>(kMaxCca)) {
            set_status(w.sz, SEEDGB_CAPACITY_OVERFLOW);
            break;
        }
        w.store[pos] = make_int2(static_cast<int>(n), si[d]);
        ++d;
        se[d] = n;
        si[d] = static_cast<int32_t>(pos);
        sk[d] = 0;
        ++pos;
    }
}

// ---------------------------------------------------------------------------
// Kalman fit of the paths (gbts_fit_segments.ipp:37-335)
// ---------------------------------------------------------------------------
struct EdgeState {
    float X[3], Y[2];
    float c, s, refX, refY;
    float J;
    bool head_type;
    float Cx[6];
    float Cy[3];
    __device__ __forceinline__ float& cx(int i, int j) { return Cx[i + j + 1 * (i != 0) * (j != 0)]; }
    __device__ __forceinline__ float cx(int i, int j) const { return Cx[i + j + 1 * (i != 0) * (j != 0)]; }
    __device__ __forceinline__ float& cy(int i, int j) { return Cy[i + j]; }
    __device__ __forceinline__ float cy(int i, int j) const { return Cy[i + j]; }
};

__device__ __forceinline__ void state_init(EdgeState& st, float4 n1, float4 n2) {
    st.J = 0.0f;
    st.head_type = (n1.w < 0);
    const float dx = n1.x - n2.x;
    const float dy = n1.y - n2.y;
    const float L = sqrtf(dx * dx + dy * dy);
    const float r1 = sqrtf(n1.x * n1.x + n1.y * n1.y);
    const float r2 = sqrtf(n2.x * n2.x + n2.y * n2.y);
    st.s = dy / L;
    st.c = dx / L;
    st.refX = n2.x * st.c + n2.y * st.s;
    st.refY = r2;
    st.X[0] = -n2.x * st.s + n2.y * st.c;
    st.X[1] = 0.0f;
    st.X[2] = 0.0f;
    st.Y[0] = n2.z;
    st.Y[1] = (n1.z - n2.z) / (r1 - r2);
    for (int i = 0; i < 6; ++i) st.Cx[i] = 0.0f;
    for (int i = 0; i < 3; ++i) st.Cy[i] = 0.0f;
    st.cx(0, 0) = 0.25f;
    st.cx(1, 1) = 0.001f;
    st.cx(2, 2) = 0.001f;
    st.cy(0, 0) = 1.5f;
    st.cy(1, 1) = 0.001f;
}

__device__ bool kalman_update(EdgeState& nt, const EdgeState& ts, float4 node,
                              const seedgb_gbts_config& p) {
    const float tau2 = ts.Y[1] * ts.Y[1];
    const float invSin2 = 1 + tau2;
    const float lenCorr = (node.w != -1) ? invSin2 : invSin2 / tau2;
    const float minPtFrac = fabsf(ts.X[2]) * p.inv_max_curvature;
    const float corrMS = p.sigmaMS * minPtFrac;
    const float sigma2 = p.radLen * lenCorr * corrMS * corrMS;
    const float m_Cx11 = ts.cx(1, 1) + sigma2;
    const float m_Cy11 = ts.cy(1, 1) + sigma2;
    const float r = sqrtf(node.x * node.x + node.y * node.y);
    nt.refX = node.x * ts.c + node.y * ts.s;
    const float mx = -node.x * ts.s + node.y * ts.c;
    nt.refY = r;
    const float my = node.z;
    const float A = nt.refX - ts.refX;
    const float B = (0.5f) * A * A;
    const float dr = nt.refY - ts.refY;
    nt.X[0] = ts.X[0] + ts.X[1] * A + ts.X[2] * B;
    nt.X[1] = ts.X[1] + ts.X[2] * A;
    nt.X[2] = ts.X[2];
    nt.cx(0, 0) = ts.cx(0, 0) + 2 * ts.cx(0, 1) * A + 2 * ts.cx(0, 2) * B + A * m_Cx11 * A +
                  2 * A * ts.cx(1, 2) * B + B * ts.cx(2, 2) * B;
    nt.cx(0, 1) = ts.cx(0, 1) + m_Cx11 * A + ts.cx(1, 2) * B + ts.cx(0, 2) * A +
                  A * ts.cx(1, 2) * A + A * ts.cx(2, 2) * B;
    nt.cx(0, 2) = ts.cx(0, 2) + ts.cx(1, 2) * A + ts.cx(2, 2) * B;
    nt.cx(1, 1) = m_Cx11 + 2 * A * ts.cx(1, 2) + A * ts.cx(2, 2) * A;
    nt.cx(1, 2) = ts.cx(1, 2) + ts.cx(2, 2) * A;
    nt.cx(2, 2) = ts.cx(2, 2);
    nt.Y[0] = ts.Y[0] + ts.Y[1] * dr;
    nt.Y[1] = ts.Y[1];
    nt.cy(0, 0) = ts.cy(0, 0) + 2 * ts.cy(0, 1) * dr + dr * m_Cy11 * dr;
    nt.cy(0, 1) = ts.cy(0, 1) + dr * m_Cy11;
    nt.cy(1, 1) = m_Cy11;
    const float resid_x = mx - nt.X[0];
    const float resid_y = my - nt.Y[0];
    float sigma_rz = 0;
    if (!ts.head_type) {
        sigma_rz = p.sigma_y;
    } else {
        sigma_rz = p.sigma_y * ts.Y[1];
    }
    const float inv_Dx = nt.cx(0, 0) + p.sigma_x * p.sigma_x;
    const float Dx = 1 / inv_Dx;
    const float Dy = 1 / (nt.cy(0, 0) + sigma_rz * sigma_rz);
    const float dchi2_x = resid_x * resid_x * Dx;
    const float dchi2_y = resid_y * resid_y * Dy;
    if (dchi2_x > p.maxDChi2_x || dchi2_y > p.maxDChi2_y) return false;
    nt.J = ts.J + (p.add_hit - dchi2_x * p.weight_x - dchi2_y * p.weight_y);
    for (int i = 0; i < 3; i++) nt.X[i] += Dx * nt.cx(0, i) * resid_x;
    if (fabsf(nt.X[2]) * p.inv_max_curvature > 1.0f) return false;
    for (int i = 0; i < 2; i++) nt.Y[i] += Dx * nt.cy(0, i) * resid_y;
    const float z0 = nt.Y[0] - nt.refY * ts.Y[1];
    if (fabsf(z0) > p.max_z0) return false;
    nt.cx(2, 2) = Dx * (nt.cx(2, 2) * inv_Dx - nt.cx(0, 2) * nt.cx(0, 2));
    nt.cx(1, 2) = Dx * (nt.cx(1, 2) * inv_Dx - nt.cx(0, 1) * nt.cx(0, 2));
    nt.cx(1, 1) = Dx * (nt.cx(1, 1) * inv_Dx - nt.cx(0, 1) * nt.cx(0, 1));
    nt.cx(0, 2) = Dx * (nt.cx(0, 2) * inv_Dx - nt.cx(0, 0) * nt.cx(0, 2));
    nt.cx(0, 1) = Dx * (nt.cx(0, 1) * inv_Dx - nt.cx(0, 0) * nt.cx(0, 1));
    nt.cx(0, 0) *= Dx * (p.sigma_x * p.sigma_x);
    nt.cy(1, 1) -= Dy * nt.cy(0, 1) * nt.cy(0, 1);
    nt.cy(0, 1) -= Dy * nt.cy(0, 0) * nt.cy(0, 1);
    nt.cy(0, 0) -= Dy * nt.cy(0, 0) * nt.cy(0, 0);
    nt.c = ts.c;
    nt.s = ts.s;
    nt.head_type = (node.w < 0);
    return true;
}

__global__ void __launch_bounds__(kThreads) k_fit(Tables T, Work w) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= w.sz[S_PATHS]) return;
    const seedgb_gbts_config& c = T.c;
    const uint32_t esz = 3u + c.max_num_neighbours;
    const uint32_t path_idx = w.sz[S_TERMINUS] + q;
    unsigned length = 1;
    bool toggle = false;
    EdgeState s1, s2;
    int2 path = w.store[path_idx];
    const uint32_t* row = w.graph + static_cast<uint64_t>(esz) * static_cast<uint32_t>(path.x);
    state_init(s1, w.red[row[1]], w.red[row[0]]);
    s2 = s1;
    while (path.y >= 0) {
        path = w.store[path.y];
        const float4 nd = w.red[w.graph[static_cast<uint64_t>(esz) * static_cast<uint32_t>(path.x) + 1]];
        if (toggle) {
            if (!kalman_update(s1, s2, nd, c)) {
                s1 = s2;
                break;
            }
        } else if (!kalman_update(s2, s1, nd, c)) {
            break;
        }
        toggle = !toggle;
        length++;
    }
    const bool ok = length >= c.minLevel;
    w.fflag[q] = ok ? 1u : 0u;
    w.fqual[q] = toggle ? static_cast<int>(c.qual_scale * s2.J) : static_cast<int>(c.qual_scale * s1.J);
}

__global__ void __launch_bounds__(kThreads) k_props(Work w) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= w.sz[S_PATHS] || !w.fflag[q]) return;
    const uint32_t P = w.fidx[q];
    w.props[P] = make_int2(w.fqual[q], static_cast<int>(w.sz[S_TERMINUS] + q));
    w.ambi[P] = 0;
    w.bidder[P] = 1;
}

// ---------------------------------------------------------------------------
// Bidding (gbts_create_seed_candidate.ipp:22-58, gbts_rebid_seeds_for_edges.
// ipp:23-62, gbts_reset_edge_bids.ipp:22-69).  Each round's bidders are fixed
// before the bids (value 2 = bidding this round); a bid phase only ever
// writes -1, so the outcome does not depend on the order of the atomics.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long bid_of(int2 prop, uint32_t P) {
    return (static_cast<unsigned long long>(static_cast<uint32_t>(prop.x)) << 32) |
           static_cast<unsigned long long>(P);
}

__device__ __forceinline__ void bid_step(const Work& w, int depth) {
    GRID_STRIDE(P, w.sz[S_PROPS]) {
        if (!w.bidder[P]) continue;
        const int2 prop = w.props[P];
        const unsigned long long seed_bid = bid_of(prop, P);
        int2 path = make_int2(0, prop.y);
        int d = depth;
        while (path.y >= 0 && d != 0) {
            path = w.store[path.y];
            d--;
            const unsigned long long comp = atomicMax(&w.ebid[path.x], seed_bid);
            if (comp > seed_bid) {
                w.ambi[P] = -1;
            } else if (comp != 0) {
                w.ambi[comp & 0xFFFFFFFFull] = -1;
            }
        }
    }
}

// who bids in this round: the first round every proposal still 0 (best on
// its outermost edge), later rounds the "maybe" ones (1); value 2 marks a
// bidder until its round's reset
__device__ __forceinline__ bool round_step(const Work& w, bool first) {
    bool any = false;
    GRID_STRIDE(P, w.sz[S_PROPS]) {
        const int8_t a = w.ambi[P];
        uint8_t b = 0;
        if (first) {
            if (a == 0) {
                w.ambi[P] = 2;
                b = 1;
            } else {
                w.ambi[P] = -2;
            }
        } else if (a == 1) {
            w.ambi[P] = 2;
            b = 1;
        }
        w.bidder[P] = b;
        any |= b != 0;
    }
    return any;
}

__device__ __forceinline__ void reset_step(const Work& w) {
    GRID_STRIDE(P, w.sz[S_PROPS]) {
        const int8_t a = w.ambi[P];
        if (a == 2) {
            w.ambi[P] = 0;
            continue;
        }
        if (a != -1) continue;
        bool good = true;
        int2 path = make_int2(0, w.props[P].y);
        while (path.y >= 0) {
            path = w.store[path.y];
            const int8_t best = w.ambi[w.ebid[path.x] & 0xFFFFFFFFull];
            if (best == 0 || best == 2) {
                good = false;
                break;
            }
        }
        w.ambi[P] = good ? 1 : -2;
    }
}

// gbts_bid_seeds_for_hits.ipp:23-70
__device__ __forceinline__ void hit_step(const Tables& T, const Work& w) {
    const uint32_t esz = 3u + T.c.max_num_neighbours;
    GRID_STRIDE(P, w.sz[S_PROPS]) {
        if (w.ambi[P] == -2) {
            atomicAdd(&w.sz[S_REJECTED], 1u);
            continue;
        }
        const int2 prop = w.props[P];
        const unsigned long long b = bid_of(prop, P);
        int2 path = make_int2(0, prop.y);
        while (path.y >= 0) {
            path = w.store[path.y];
            atomicMax(&w.hbid[w.graph[static_cast<uint64_t>(esz) * static_cast<uint32_t>(path.x)]], b);
        }
        atomicMax(&w.hbid[w.graph[static_cast<uint64_t>(esz) * static_cast<uint32_t>(path.x) + 1]], b);
    }
}

__device__ __forceinline__ void zero64(unsigned long long* p, uint64_t n) {
    for (uint64_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0ull;
}

// the fit's bids on each proposal's outermost edge, the rounds of edge
// bidding and the hit bids, in one cooperative launch.  Bids are indexed by
// connected edge (the path store's numbering), so only those entries are
// cleared each round.
__global__ void __launch_bounds__(kThreads)
k_bidding(Tables T, Work w, uint32_t n_sp, uint32_t rounds) {
    cg::grid_group g = cg::this_grid();
    const uint32_t n_conn = w.sz[S_CONNECTED];
    zero64(w.ebid, n_conn);
    zero64(w.hbid, n_sp);
    g.sync();
    bid_step(w, 1);
    g.sync();
    for (uint32_t r = 0; r < rounds; ++r) {
        zero64(w.ebid, n_conn);
        const bool any = round_step(w, r == 0);
        if (__syncthreads_or(any) && threadIdx.x == 0) w.flags[kMaxCca + r] = 1u;
        g.sync();
        // a round without bidders leaves nothing to bid on in any later round
        if (w.flags[kMaxCca + r] == 0u) break;
        bid_step(w, -1);
        g.sync();
        reset_step(w);
        g.sync();
    }
    hit_step(T, w);
}

// gbts_estimate_seed_params (gbts_convert_seeds.ipp:33-67)
__device__ __forceinline__ float2 estimate_seed_params(const float4 sps[3]) {
    float u[2], v[2];
    const float x0 = sps[1].x;
    const float y0 = sps[1].y;
    const float r0 = sqrtf(x0 * x0 + y0 * y0);
    const float cosA = x0 / r0;
    const float sinA = y0 / r0;
    for (unsigned k = 0; k < 2; k++) {
        const unsigned i = (k == 1) ? 2u : k;
        const float dx = sps[i].x - x0;
        const float dy = sps[i].y - y0;
        const float r2_inv = 1.0f / (dx * dx + dy * dy);
        const float xn = dx * cosA + dy * sinA;
        const float yn = -dx * sinA + dy * cosA;
        u[k] = xn * r2_inv;
        v[k] = yn * r2_inv;
    }
    const float du = u[0] - u[1];
    if (du == 0.0f) return make_float2(0.0f, 0.0f);
    const float A = (v[0] - v[1]) / du;
    const float B = v[1] - A * u[1];
    const float curv = 1000.0f * B / sqrtf(1 + A * A);
    const float cot_t = (sps[2].z - sps[1].z) / (sqrtf(sps[2].x * sps[2].x + sps[2].y * sps[2].y) - r0);
    return make_float2(curv, cot_t);
}

// gbts_convert_seeds.ipp:72-194: up to three seeds per surviving proposal
__global__ void __launch_bounds__(kThreads) k_convert(Tables T, Work w) {
    const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= w.sz[S_PROPS]) return;
    w.ecount[P] = 0;
    if (w.ambi[P] == -2) return;
    const seedgb_gbts_config& c = T.c;
    const uint32_t esz = 3u + c.max_num_neighbours;
    uint32_t nodes[kMaxCca + 1];
    int size = 0;
    signed char best_for_hit = 0;
    const int2 prop = w.props[P];
    int2 path = make_int2(0, prop.y);
    while (path.y >= 0 && size < static_cast<int>(kMaxCca)) {
        path = w.store[path.y];
        nodes[size++] = w.graph[static_cast<uint64_t>(esz) * static_cast<uint32_t>(path.x)];
        best_for_hit = static_cast<signed char>(best_for_hit + (P == (w.hbid[nodes[size - 1]] & 0xFFFFFFFFull)));
    }
    nodes[size++] = w.graph[static_cast<uint64_t>(esz) * static_cast<uint32_t>(path.x) + 1];
    best_for_hit = static_cast<signed char>(best_for_hit + (P == (w.hbid[nodes[size - 1]] & 0xFFFFFFFFull)));
    if (best_for_hit < c.best_hit_frac * static_cast<float>(size)) return;
    int diff_code = 0;
    bool force_dropout = false;
    if (c.use_dropout) {
        float4 sps[3] = {w.red[nodes[size - 1]], w.red[nodes[(size - 1) / 2 + 1]], w.red[nodes[0]]};
        const float2 c1 = estimate_seed_params(sps);
        sps[1] = w.red[nodes[(size - 1) / 2]];
        const float2 c2 = estimate_seed_params(sps);
        sps[0] = w.red[nodes[size - 2]];
        const float2 c3 = estimate_seed_params(sps);
        if ((best_for_hit < size - 1) & (fabsf(c1.y + c2.y + c3.y) < 3.0f * c.tight_bid_cot_threshold) &
            (size < 5))
            return;
        const float d0 = fabsf(c1.x - c2.x), d1 = fabsf(c2.x - c3.x), d2 = fabsf(c1.x - c3.x);
        diff_code = 4 * (d0 < c.dropout_dcurv_m) + 2 * (d1 < c.dropout_dcurv_m) + (d2 < c.dropout_dcurv_m);
        force_dropout = fabsf(c1.x + c2.x + c3.x) < 3.0f * c.force_dropout_max_curv_m;
        force_dropout |= (fabsf(c1.y + c2.y + c3.y) < 3.0f * c.tight_bid_cot_threshold) & (diff_code == 0);
    }
    const uint32_t qbits = __float_as_uint(static_cast<float>(prop.x));
    uint32_t ne = 0;
    uint4* o = w.seeds3 + 3ull * P;
    if (((diff_code != 3) & (diff_code != 6)) | force_dropout)
        o[ne++] = make_uint4(nodes[size - 1], nodes[(size - 1) / 2 + 1], nodes[0], qbits);
    if ((diff_code == 1) | (diff_code == 6))
        o[ne++] = make_uint4(nodes[size - 1], nodes[(size - 1) / 2], nodes[0], qbits);
    if ((diff_code == 2) | (diff_code == 3) | (diff_code == 4) | force_dropout)
        o[ne++] = make_uint4(nodes[size - 2], nodes[(size - 1) / 2], nodes[0], qbits);
    w.ecount[P] = ne;
}

__global__ void __launch_bounds__(kThreads) k_seeds_out(Work w, seedgb_seed_buffer out) {
    const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = w.sz[S_PROPS];
    if (P == 0) {
        const uint32_t tot = w.sz[S_SEEDS];
        *out.size = tot < out.capacity ? tot : out.capacity;
        if (tot > out.capacity) set_status(w.sz, SEEDGB_CAPACITY_OVERFLOW);
    }
    if (P >= n) return;
    const uint32_t ne = w.ecount[P];
    const uint32_t o = w.eoff[P];
    for (uint32_t k = 0; k < ne; ++k) {
        if (o + k >= out.capacity) break;
        const uint4 s = w.seeds3[3ull * P + k];
        out.bottom_index[o + k] = s.x;
        out.middle_index[o + k] = s.y;
        out.top_index[o + k] = s.z;
        out.quality[o + k] = __uint_as_float(s.w);
    }
}

__global__ void k_empty_out(seedgb_seed_buffer out) { *out.size = 0; }

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
uint64_t field_h(uint64_t v, uint32_t shift, uint32_t bits) {
    const uint64_t m = bits >= 64 ? ~0ull : ((1ull << bits) - 1ull);
    return shift >= 64 ? 0 : ((v >> shift) & m);
}

struct DevBlock {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBlock() {
        if (p) cudaFree(p);
    }
    bool ensure(size_t need) {
        if (need <= bytes) return true;
        if (p) {
            cudaDeviceSynchronize();
            cudaFree(p);
            p = nullptr;
            bytes = 0;
        }
        if (cudaMalloc(&p, need) != cudaSuccess) return false;
        bytes = need;
        return true;
    }
};

struct Carver {
    char* base;
    size_t off = 0;
    template <class T>
    T* take(uint64_t n) {
        off = (off + 255) & ~size_t(255);
        T* r = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += sizeof(T) * static_cast<size_t>(n ? n : 1);
        return r;
    }
};

}  // namespace

namespace {

// One event in flight: its work arenas, sizes and scan ticket.  A single call
// uses slot 0; a batch alternates its events over two slots on the caller's
// stream and enqueues event e + 1's kernels before it waits for event e's
// path-store size, so the GPU has work queued while the host waits (the
// events' kernels stay in stream order: no two cooperative launches can be
// resident at once).
constexpr uint32_t kMaxSlots = 2;

struct Slot {
    DevBlock arena_a, arena_b;
    uint32_t* d_sz = nullptr;
    uint32_t* h_sz = nullptr;  // pinned
    Work w{};
    uint64_t a_sp = 0, a_e = 0;
    // single-pass scans: running tile ticket and scan epoch
    unsigned long long* d_ticket = nullptr;
    unsigned long long ticket_base = 0;
    uint32_t epoch = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ready = nullptr;    // sizes copied to h_sz
    // the event in flight: its tail runs after the path store's size is known
    bool pending = false;
    seedgb_seed_buffer out{};
    uint32_t n_sp = 0;
};

}  // namespace

struct seedgb_gbts {
    seedgb_gbts_config cfg;
    uint32_t n_layers = 0, n_eta = 0, n_pairs = 0, n_volumes = 0, n_surfaces = 0, n_tau = 0;
    uint32_t max_first_degree = 0;
    // device tables
    int8_t* d_type = nullptr;
    uint32_t *d_bin0 = nullptr, *d_neta = nullptr, *d_pairs = nullptr, *d_smap = nullptr;
    float *d_min_eta = nullptr, *d_width = nullptr, *d_lut = nullptr;
    int16_t* d_vmap = nullptr;
    Slot slot[kMaxSlots];
    uint32_t used = 1;       // slots the last call used
    uint32_t last_slot = 0;  // slot of the last event
    // cooperative launches: blocks that can be co-resident
    uint32_t coop_cca = 0, coop_bid = 0, walk_blocks = 0;
};

namespace {

Tables tables_of(const seedgb_gbts* h) {
    Tables T;
    T.c = h->cfg;
    T.n_layers = h->n_layers;
    T.n_eta = h->n_eta;
    T.n_pairs = h->n_pairs;
    T.n_volumes = h->n_volumes;
    T.n_surfaces = h->n_surfaces;
    T.n_tau_lut = h->n_tau;
    T.layer_type = h->d_type;
    T.eta_bin0 = h->d_bin0;
    T.n_eta_l = h->d_neta;
    T.min_eta = h->d_min_eta;
    T.eta_width = h->d_width;
    T.pairs = h->d_pairs;
    T.vmap = h->d_vmap;
    T.smap = h->d_smap;
    T.tau_lut = h->d_lut;
    return T;
}

uint32_t blocks(uint64_t n, int threads = kThreads) {
    return static_cast<uint32_t>(std::max<uint64_t>(1, (n + threads - 1) / threads));
}

// exclusive scan of n values (n_dev + add on the device, else n_host) into
// out[0, n], the total also to *total_dst; one launch sized for `cap`
void scan(Slot& sl, const uint32_t* in, uint32_t* out, const uint32_t* n_dev, uint32_t n_host,
          uint32_t add, uint64_t cap, unsigned long long* state, uint32_t* total_dst) {
    const uint32_t tiles = static_cast<uint32_t>(std::max<uint64_t>(1, (cap + kScanTile - 1) / kScanTile));
    if (++sl.epoch >= (1u << 30)) sl.epoch = 1;
    k_scan<<<tiles, kScanThreads, 0, sl.stream>>>(in, out, n_dev, n_host, add, state, sl.d_ticket,
                                                  sl.ticket_base, sl.epoch, total_dst, sl.d_sz);
    sl.ticket_base += tiles;
}

// carve the spacepoint-sized arena (base == nullptr: measure only)
size_t carve_a(seedgb_gbts* h, char* base, uint64_t n_sp, uint64_t items_cap, Work& w) {
    const uint64_t N = std::max<uint64_t>(n_sp, 1);
    const uint64_t E = std::max<uint64_t>(1, static_cast<uint64_t>(h->cfg.max_edges_factor) * N);
    const uint64_t M = h->cfg.max_num_neighbours;
    const uint64_t cells = static_cast<uint64_t>(h->n_eta) * h->cfg.n_phi_bins;
    const uint64_t scan_cap =
        std::max<uint64_t>({E + 1, N + 1, cells + 1, items_cap * kEdgeWarps + 1, h->n_pairs + 1ull});
    Carver cv{base};
    w.red = cv.take<float4>(N);
    w.sp_phi = cv.take<float>(N);
    w.sp_cell = cv.take<uint32_t>(N);
    w.cell_cnt = cv.take<uint32_t>(cells + 1);
    w.cell_off = cv.take<uint32_t>(cells + 1);
    w.cell_cur = cv.take<uint32_t>(cells + 1);
    w.node_sp = cv.take<uint32_t>(N);
    w.node_p = cv.take<float4>(N);
    w.node_phi = cv.take<float>(N);
    w.view = cv.take<uint32_t>(2ull * h->n_eta);
    w.rads = cv.take<float>(2ull * h->n_eta);
    w.item_cnt = cv.take<uint32_t>(h->n_pairs + 1ull);
    w.item_off = cv.take<uint32_t>(h->n_pairs + 1ull);
    w.items = cv.take<uint4>(items_cap);
    w.item_dphi = cv.take<float>(items_cap);
    w.item_eta = cv.take<uint32_t>(items_cap);
    w.unit_cnt = cv.take<uint32_t>(items_cap * kEdgeWarps + 1);
    w.unit_off = cv.take<uint32_t>(items_cap * kEdgeWarps + 1);
    w.unit_pos = cv.take<uint32_t>(items_cap * kEdgeWarps + 1);
    w.unit_nrec = cv.take<uint32_t>(items_cap * kEdgeWarps + 1);
    w.rec_a = cv.take<uint2>(E);
    w.rec_m = cv.take<ulonglong2>(E);
    w.e_in = cv.take<uint32_t>(E);
    w.e_out = cv.take<uint32_t>(E);
    w.e_p = cv.take<float4>(E);
    w.out_cnt = cv.take<uint32_t>(N + 1);
    w.lstart = cv.take<uint32_t>(N + 1);
    w.lcur = cv.take<uint32_t>(N + 1);
    w.links = cv.take<uint32_t>(E);
    w.links_tmp = cv.take<uint32_t>(E);
    w.in_cnt = cv.take<uint32_t>(N + 1);
    w.instart = cv.take<uint32_t>(N + 1);
    w.incur = cv.take<uint32_t>(N + 1);
    w.in_list = cv.take<uint32_t>(E);
    w.nnei = cv.take<uint8_t>(E);
    w.nei = cv.take<uint32_t>(M * E);
    w.kept = cv.take<uint32_t>(E);
    w.kbase = cv.take<uint32_t>(E + 1);
    w.graph = cv.take<uint32_t>((3 + M) * E);
    w.levels = cv.take<uint8_t>(2 * E);
    w.active = cv.take<int8_t>(E);
    w.opx = cv.take<int32_t>(E);
    w.opy = cv.take<int16_t>(E);
    w.tflag = cv.take<uint32_t>(E);
    w.tidx = cv.take<uint32_t>(E + 1);
    w.tpaths = cv.take<uint32_t>(E);
    w.pbase = cv.take<uint32_t>(E + 1);
    w.ebid = cv.take<unsigned long long>(E);
    w.hbid = cv.take<unsigned long long>(N);
    w.tstate = cv.take<unsigned long long>(scan_cap / kScanTile + 4);
    w.flags = cv.take<uint32_t>(kFlagSlots);
    w.ecap = E;
    return cv.off + 256;
}

size_t carve_b(char* base, uint64_t n_term, uint64_t n_paths, Work& w) {
    const uint64_t S = std::max<uint64_t>(1, n_term + n_paths);
    const uint64_t P = std::max<uint64_t>(1, n_paths);
    Carver cv{base};
    w.store = cv.take<int2>(S);
    w.term_edge = cv.take<uint32_t>(std::max<uint64_t>(1, n_term));
    w.term_pos = cv.take<uint32_t>(std::max<uint64_t>(1, n_term));
    w.fflag = cv.take<uint32_t>(P);
    w.fidx = cv.take<uint32_t>(P + 1);
    w.fqual = cv.take<int32_t>(P);
    w.props = cv.take<int2>(P);
    w.ambi = cv.take<int8_t>(P);
    w.bidder = cv.take<uint8_t>(P);
    w.ecount = cv.take<uint32_t>(P);
    w.eoff = cv.take<uint32_t>(P + 1);
    w.seeds3 = cv.take<uint4>(3 * P);
    w.tstate_b = cv.take<unsigned long long>((P + 1) / kScanTile + 4);
    w.pcap = S;
    return cv.off + 256;
}

// gbts_seedfinder_config::setLinkingScheme (core/src/gbts_seeding/
// gbts_seeding_config.cpp:19-142): descending barcodes; one volume -> one
// layer, or -(first surface-map entry + 1) when its surfaces lie on several
// layers; a (UINT_MAX, -1) sentinel ends the walk; the volume map is
// (largest volume + 1) zeros followed by as many SHRT_MAX entries.
bool linking(seedgb_gbts_config& c, float minPt, const seedgb_gbts_geoid* geoids, uint32_t n,
             std::vector<int16_t>& vmap, std::vector<uint32_t>& smap) {
    if (n == 0) return false;
    std::vector<std::pair<uint64_t, int16_t>> g(n);
    for (uint32_t i = 0; i < n; ++i) g[i] = {geoids[i].barcode, static_cast<int16_t>(geoids[i].layer)};
    std::stable_sort(g.begin(), g.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    const uint32_t largest = static_cast<uint32_t>(field_h(g[0].first, c.volume_shift, c.volume_bits));
    if (largest >= SHRT_MAX) return false;
    int16_t current_volume = static_cast<int16_t>(largest);
    bool layer_change = false;
    int16_t current_layer = g[0].second;
    g.emplace_back(static_cast<uint64_t>(UINT_MAX), static_cast<int16_t>(-1));
    std::vector<std::pair<int16_t, uint32_t>> vol_bins;
    std::vector<std::pair<uint32_t, uint32_t>> in_volume;
    smap.clear();
    for (const auto& gp : g) {
        const int16_t vol = static_cast<int16_t>(field_h(gp.first, c.volume_shift, c.volume_bits));
        if (current_volume != vol) {
            int16_t bin = current_layer;
            if (layer_change) {
                bin = static_cast<int16_t>(-1 * static_cast<int16_t>(smap.size() / 2 + 1));
                for (const auto& s : in_volume) {
                    smap.push_back(s.first);
                    smap.push_back(s.second);
                }
            }
            vol_bins.emplace_back(bin, static_cast<uint32_t>(static_cast<uint16_t>(current_volume)));
            current_volume = vol;
            current_layer = gp.second;
            layer_change = false;
            in_volume.clear();
        }
        layer_change |= (current_layer != gp.second);
        in_volume.emplace_back(static_cast<uint32_t>(field_h(gp.first, c.index_shift, c.index_bits)),
                               static_cast<uint32_t>(static_cast<int32_t>(gp.second)));
    }
    vmap.assign(largest + 1, 0);
    vmap.insert(vmap.end(), largest + 1, static_cast<int16_t>(SHRT_MAX));
    for (const auto& vb : vol_bins)
        if (vb.second < vmap.size()) vmap[vb.second] = vb.first;
    if (smap.size() / 2 > SHRT_MAX) return false;
    const float ptScale = 900.0f / minPt;
    c.min_delta_phi *= ptScale;
    c.dphi_coeff *= ptScale;
    c.min_delta_phi_low_dr *= ptScale;
    c.dphi_coeff_low_dr *= ptScale;
    c.max_Kappa *= ptScale;
    return true;
}

template <class T>
bool upload(T** dst, const T* src, size_t n) {
    if (cudaMalloc(reinterpret_cast<void**>(dst), sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess)
        return false;
    if (n && cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) return false;
    return true;
}

void free_tables(seedgb_gbts* h) {
    cudaFree(h->d_type);
    cudaFree(h->d_bin0);
    cudaFree(h->d_neta);
    cudaFree(h->d_pairs);
    cudaFree(h->d_smap);
    cudaFree(h->d_min_eta);
    cudaFree(h->d_width);
    cudaFree(h->d_lut);
    cudaFree(h->d_vmap);
    for (Slot& sl : h->slot) {
        cudaFree(sl.d_sz);
        cudaFree(sl.d_ticket);
        if (sl.h_sz) cudaFreeHost(sl.h_sz);
        if (sl.ready) cudaEventDestroy(sl.ready);
    }
}

bool slot_init(Slot& sl) {
    if (sl.d_sz) return true;
    if (cudaMalloc(reinterpret_cast<void**>(&sl.d_sz), sizeof(uint32_t) * S_COUNT) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void**>(&sl.h_sz), sizeof(uint32_t) * S_COUNT) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&sl.d_ticket), sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(sl.d_ticket, 0, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(sl.d_sz, 0, sizeof(uint32_t) * S_COUNT) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming) != cudaSuccess)
        return false;
    std::memset(sl.h_sz, 0, sizeof(uint32_t) * S_COUNT);
    return true;
}

}  // namespace

extern "C" void seedgb_gbts_config_default(seedgb_gbts_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->tMin_slope = 6.7f;
    c->offset = 0.2f;
    c->tMax_min = 1.6f;
    c->tMax_correction = 0.15f;
    c->tMax_slope = 6.1f;
    c->maxTau = 36.0f;
    c->minDeltaRadius = 2.0f;
    c->min_z0 = -160.0f;
    c->max_z0 = 160.0f;
    c->maxOuterRadius = 350.0f;
    c->tau_roi = 45.0f;
    c->cut_zMinU = c->min_z0 - c->maxOuterRadius * c->tau_roi;
    c->cut_zMaxU = c->max_z0 + c->maxOuterRadius * c->tau_roi;
    c->max_Kappa = 3.75e-4f;
    c->cut_dphi_max = 0.012f;
    c->cut_dcurv_max = 0.001f;
    c->cut_tau_ratio_max = 0.01f;
    c->min_delta_phi = 0.015f;
    c->dphi_coeff = 2.2e-4f;
    c->min_delta_phi_low_dr = 0.002f;
    c->dphi_coeff_low_dr = 4.33e-4f;
    c->low_dr_threshold = 60.0f;
    c->type1_max_width = 0.2f;
    c->doTauCut = 1;
    c->sigmaMS = 0.016f;
    c->radLen = 0.025f;
    c->sigma_x = 0.08f;
    c->sigma_y = 0.25f;
    c->weight_x = 0.5f;
    c->weight_y = 0.5f;
    c->maxDChi2_x = 5.0f;
    c->maxDChi2_y = 6.0f;
    c->add_hit = 14.0f;
    c->qual_scale = 0.01f * static_cast<float>(INT_MAX) / (c->add_hit * static_cast<float>(kMaxCca));
    c->inv_max_curvature = 900.0f;
    c->use_dropout = 1;
    c->dropout_dcurv_m = 0.007f;
    c->force_dropout_max_curv_m = 0.03f;
    c->best_hit_frac = 0.49f;
    c->tight_bid_cot_threshold = 1.0f;
    c->n_phi_bins = 128;
    c->max_num_neighbours = 10;
    c->minLevel = 3;
    c->max_edges_factor = 10;
    c->edge_bidding_rounds = 5;
    c->volume_shift = 52;
    c->volume_bits = 12;
    c->index_shift = 27;
    c->index_bits = 21;
}

extern "C" seedgb_status seedgb_gbts_create(const seedgb_gbts_config* config,
                                            const seedgb_gbts_layer* layers, uint32_t n_layers,
                                            const uint32_t* bin_pairs, uint32_t n_pairs,
                                            const seedgb_gbts_geoid* geoids, uint32_t n_geoids,
                                            float min_pt, const float* tau_lut, uint32_t n_tau_lut,
                                            seedgb_gbts** out) {
    if (!config || !out || (n_layers && !layers) || (n_pairs && !bin_pairs) ||
        (n_geoids && !geoids))
        return SEEDGB_INVALID_ARGUMENT;
    *out = nullptr;
    seedgb_gbts_config c = *config;
    if (n_layers == 0 || c.n_phi_bins == 0 || c.max_num_neighbours == 0 ||
        c.max_num_neighbours > 255 || c.max_edges_factor == 0 || !(min_pt > 0.0f) ||
        c.edge_bidding_rounds > kFlagSlots - kMaxCca)
        return SEEDGB_BAD_CONFIG;
    if (c.useTauLUT && (!tau_lut || n_tau_lut % 5 != 0 || c.tauLutSize > n_tau_lut))
        return SEEDGB_BAD_CONFIG;
    std::vector<int16_t> vmap;
    std::vector<uint32_t> smap;
    if (!linking(c, min_pt, geoids, n_geoids, vmap, smap)) return SEEDGB_BAD_CONFIG;
    for (uint32_t i = 0; i < n_geoids; ++i)
        if (geoids[i].layer < 0 || static_cast<uint32_t>(geoids[i].layer) >= n_layers)
            return SEEDGB_BAD_CONFIG;
    uint32_t n_eta = 0;
    std::vector<int8_t> type(n_layers);
    std::vector<uint32_t> bin0(n_layers), neta(n_layers);
    std::vector<float> mine(n_layers), width(n_layers);
    for (uint32_t l = 0; l < n_layers; ++l) {
        if (layers[l].n_eta_bins == 0) return SEEDGB_BAD_CONFIG;
        type[l] = static_cast<int8_t>(layers[l].type);
        bin0[l] = layers[l].eta_bin0;
        neta[l] = layers[l].n_eta_bins;
        mine[l] = layers[l].min_eta;
        width[l] = layers[l].eta_bin_width;
        n_eta = std::max(n_eta, layers[l].eta_bin0 + layers[l].n_eta_bins);
    }
    if (static_cast<uint64_t>(n_eta) * c.n_phi_bins >= 0xFFFFFFF0ull) return SEEDGB_BAD_CONFIG;
    std::vector<uint32_t> deg(n_eta, 0);
    for (uint32_t p = 0; p < n_pairs; ++p) {
        if (bin_pairs[2 * p] >= n_eta || bin_pairs[2 * p + 1] >= n_eta) return SEEDGB_BAD_CONFIG;
        deg[bin_pairs[2 * p]]++;
    }
    auto* h = new seedgb_gbts();
    h->cfg = c;
    h->n_layers = n_layers;
    h->n_eta = n_eta;
    h->n_pairs = n_pairs;
    h->n_volumes = static_cast<uint32_t>(vmap.size());
    h->n_surfaces = static_cast<uint32_t>(smap.size() / 2);
    h->n_tau = c.useTauLUT ? n_tau_lut : 0;
    h->max_first_degree = n_eta ? *std::max_element(deg.begin(), deg.end()) : 0;
    std::vector<float> lut(tau_lut && c.useTauLUT ? tau_lut : nullptr,
                           tau_lut && c.useTauLUT ? tau_lut + n_tau_lut : nullptr);
    const bool ok = upload(&h->d_type, type.data(), type.size()) &&
                    upload(&h->d_bin0, bin0.data(), bin0.size()) &&
                    upload(&h->d_neta, neta.data(), neta.size()) &&
                    upload(&h->d_min_eta, mine.data(), mine.size()) &&
                    upload(&h->d_width, width.data(), width.size()) &&
                    upload(&h->d_pairs, bin_pairs, 2ull * n_pairs) &&
                    upload(&h->d_vmap, vmap.data(), vmap.size()) &&
                    upload(&h->d_smap, smap.data(), smap.size()) &&
                    upload(&h->d_lut, lut.data(), lut.size()) && slot_init(h->slot[0]);
    if (!ok) {
        free_tables(h);
        delete h;
        return SEEDGB_CUDA_ERROR;
    }
    int dev = 0, sms = 0, coop = 0, nb_cca = 0, nb_bid = 0, nb_walk = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_cca, k_cca_all, kCcaThreads, 0) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_bid, k_bidding, kThreads, 0) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_walk, k_edge_masks, kEdgeThreads, 0) !=
            cudaSuccess) {
        free_tables(h);
        delete h;
        return SEEDGB_CUDA_ERROR;
    }
    if (!coop || nb_cca < 1 || nb_bid < 1) {
        free_tables(h);
        delete h;
        return SEEDGB_UNSUPPORTED;
    }
    // the automaton at full occupancy; the bidding at two blocks per SM (few
    // arrivals per grid barrier)
    h->coop_cca = static_cast<uint32_t>(nb_cca * sms);
    h->coop_bid = static_cast<uint32_t>(std::min(nb_bid, 2) * sms);
    // the edge walk: every block resident, units handed out by a counter
    h->walk_blocks = static_cast<uint32_t>(std::max(nb_walk, 1) * sms);
    *out = h;
    return SEEDGB_OK;
}

extern "C" seedgb_status seedgb_gbts_destroy(seedgb_gbts* h) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    cudaDeviceSynchronize();
    free_tables(h);
    delete h;
    return SEEDGB_OK;
}

extern "C" seedgb_status seedgb_gbts_get_config(const seedgb_gbts* h, seedgb_gbts_config* config,
                                                uint32_t* n_eta_bins, uint32_t* n_volumes,
                                                uint32_t* n_surfaces) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    if (config) *config = h->cfg;
    if (n_eta_bins) *n_eta_bins = h->n_eta;
    if (n_volumes) *n_volumes = h->n_volumes;
    if (n_surfaces) *n_surfaces = h->n_surfaces;
    return SEEDGB_OK;
}

namespace {

seedgb_status check_event(const seedgb_spacepoint_view* sps, const uint64_t* surface_link,
                          const float* diameter, uint32_t n_meas, const seedgb_seed_buffer* out) {
    if (!sps || !out || !out->size || (sps->size && (!sps->global || !sps->measurement_index_1)) ||
        (n_meas && (!surface_link || !diameter)) ||
        (out->capacity && (!out->bottom_index || !out->middle_index || !out->top_index || !out->quality)))
        return SEEDGB_INVALID_ARGUMENT;
    return SEEDGB_OK;
}

// the event's kernels up to the path store's size, whose copy to the host
// the slot's `ready` event marks; the status words of the call stay
seedgb_status front(seedgb_gbts* h, Slot& sl, const seedgb_spacepoint_view* sps,
                    const uint64_t* surface_link, const float* diameter, uint32_t n_meas,
                    const seedgb_seed_buffer* out) {
    if (cudaMemsetAsync(sl.d_sz, 0, sizeof(uint32_t) * S_STATUS, sl.stream) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    sl.pending = false;
    const uint32_t n_sp = sps->size;
    if (n_sp == 0) {
        k_empty_out<<<1, 1, 0, sl.stream>>>(*out);
        return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
    }
    const uint64_t items_cap = static_cast<uint64_t>(h->n_pairs) +
                               static_cast<uint64_t>(h->max_first_degree) * ((n_sp + kNodeBuffer - 1) / kNodeBuffer);
    if (n_sp > sl.a_sp || items_cap > sl.a_e) {
        Work tmp{};
        const size_t need = carve_a(h, nullptr, n_sp, items_cap, tmp);
        if (!sl.arena_a.ensure(need)) return SEEDGB_CUDA_ERROR;
        sl.a_sp = n_sp;
        sl.a_e = items_cap;
    }
    Work& w = sl.w;
    carve_a(h, static_cast<char*>(sl.arena_a.p), sl.a_sp, sl.a_e, w);
    w.sz = sl.d_sz;
    const Tables T = tables_of(h);
    const uint64_t N = n_sp;
    const uint64_t E = w.ecap;  // edge capacity: max_edges_factor x arena spacepoints
    const uint32_t cells = h->n_eta * h->cfg.n_phi_bins;
    unsigned long long* st = w.tstate;
    const uint64_t scan_tiles = (std::max<uint64_t>({E + 1, N + 1, cells + 1ull, sl.a_e * kEdgeWarps + 1,
                                                    h->n_pairs + 1ull}) / kScanTile) + 4;
    cudaMemsetAsync(st, 0, sizeof(unsigned long long) * scan_tiles, sl.stream);
    cudaMemsetAsync(w.flags, 0, sizeof(uint32_t) * kFlagSlots, sl.stream);
    // nodes
    cudaMemsetAsync(w.cell_cnt, 0, sizeof(uint32_t) * (cells + 1ull), sl.stream);
    cudaMemsetAsync(w.cell_cur, 0, sizeof(uint32_t) * (cells + 1ull), sl.stream);
    k_classify<<<blocks(N), kThreads, 0, sl.stream>>>(T, *sps, surface_link, diameter, n_meas, w);
    scan(sl, w.cell_cnt, w.cell_off, nullptr, cells, 0, cells + 1ull, st, sl.d_sz + S_NODES);
    k_scatter<<<blocks(N), kThreads, 0, sl.stream>>>(n_sp, w);
    k_sort_cells<<<blocks(cells), kThreads, 0, sl.stream>>>(cells, w);
    k_node_params<<<blocks(N), kThreads, 0, sl.stream>>>(T, w);
    k_eta_bins<<<blocks(32ull * h->n_eta), kThreads, 0, sl.stream>>>(h->n_eta, h->cfg.n_phi_bins, w);
    // work items
    k_items_count<<<blocks(h->n_pairs), kThreads, 0, sl.stream>>>(T, w);
    scan(sl, w.item_cnt, w.item_off, nullptr, h->n_pairs, 0, h->n_pairs + 1ull, st, sl.d_sz + S_ITEMS);
    k_items_fill<<<blocks(h->n_pairs), kThreads, 0, sl.stream>>>(T, w);
    // edges: one walk per (item, quarter) keeping inner-node masks, a scan
    // over the units' edge counts, one edge record per set bit
    const uint32_t edge_grid = 152u * 16u;
    k_edge_masks<<<h->walk_blocks, kEdgeThreads, 0, sl.stream>>>(T, w);
    scan(sl, w.unit_cnt, w.unit_off, sl.d_sz + S_UNITS, 0, 0, sl.a_e * kEdgeWarps + 1, st,
         sl.d_sz + S_EDGES_MADE);
    cudaMemsetAsync(w.out_cnt, 0, sizeof(uint32_t) * (N + 1), sl.stream);
    k_edge_expand<<<edge_grid, kEdgeThreads, 0, sl.stream>>>(T, w);
    // the edges leaving each node: offsets by inner node, lists in ascending
    // edge index; every kernel from here to the path store reads its size
    // from device memory (grid-stride launches), so nothing waits on the host
    scan(sl, w.out_cnt, w.lstart, sl.d_sz + S_NODES, 0, 0, N + 1, st, nullptr);
    cudaMemsetAsync(w.lcur, 0, sizeof(uint32_t) * (N + 1), sl.stream);
    cudaMemsetAsync(w.in_cnt, 0, sizeof(uint32_t) * (N + 1), sl.stream);
    cudaMemsetAsync(w.incur, 0, sizeof(uint32_t) * (N + 1), sl.stream);
    k_edges_kept<<<1, 1, 0, sl.stream>>>(T, w);
    k_link_fill<<<blocks(E), kThreads, 0, sl.stream>>>(w);
    k_link_sort<<<kGrid, kThreads, 0, sl.stream>>>(w);
    scan(sl, w.in_cnt, w.instart, sl.d_sz + S_NODES, 0, 0, N + 1, st, nullptr);
    k_in_fill<<<blocks(E), kThreads, 0, sl.stream>>>(w);
    k_match_nodes<<<kGrid, kThreads, 0, sl.stream>>>(T, w);
    scan(sl, w.kept, w.kbase, sl.d_sz + S_EDGES, 0, 0, E + 1, st, sl.d_sz + S_CONNECTED);
    k_compress<<<blocks(E), kThreads, 0, sl.stream>>>(T, w);
    // automaton over the connected edges
    cudaMemsetAsync(w.levels, 1, static_cast<size_t>(2 * E), sl.stream);
    {
        Tables Tc = T;
        Work wc = w;
        void* args[] = {&Tc, &wc};
        if (cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_cca_all), dim3(h->coop_cca),
                                        dim3(kCcaThreads), args, 0, sl.stream) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
    }
    k_term_flags<<<kGrid, kThreads, 0, sl.stream>>>(w);
    scan(sl, w.tflag, w.tidx, sl.d_sz + S_CONNECTED, 0, 0, E + 1, st, sl.d_sz + S_TERMINUS);
    scan(sl, w.tpaths, w.pbase, sl.d_sz + S_CONNECTED, 0, 0, E + 1, st, sl.d_sz + S_PATHS);
    if (cudaMemcpyAsync(sl.h_sz, sl.d_sz, sizeof(uint32_t) * S_COUNT, cudaMemcpyDeviceToHost,
                        sl.stream) != cudaSuccess ||
        cudaEventRecord(sl.ready, sl.stream) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    sl.pending = true;
    sl.out = *out;
    sl.n_sp = n_sp;
    return SEEDGB_OK;
}

// the rest of the event once its path store's size is on the host
seedgb_status finish(seedgb_gbts* h, Slot& sl) {
    if (!sl.pending) return SEEDGB_OK;
    sl.pending = false;
    if (cudaEventSynchronize(sl.ready) != cudaSuccess) return SEEDGB_CUDA_ERROR;
    const seedgb_seed_buffer* out = &sl.out;
    const uint32_t n_sp = sl.n_sp;
    Work& w = sl.w;
    const Tables T = tables_of(h);
    const uint64_t n_term = sl.h_sz[S_TERMINUS], n_paths = sl.h_sz[S_PATHS];
    if (n_term == 0 || n_paths == 0) {
        k_empty_out<<<1, 1, 0, sl.stream>>>(*out);
        return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
    }
    {
        Work tmp{};
        const size_t need = carve_b(nullptr, n_term, n_paths, tmp);
        if (!sl.arena_b.ensure(need)) return SEEDGB_CUDA_ERROR;
        carve_b(static_cast<char*>(sl.arena_b.p), n_term, n_paths, w);
        cudaMemsetAsync(w.tstate_b, 0, sizeof(unsigned long long) * ((n_paths + 1) / kScanTile + 4), sl.stream);
    }
    k_term_fill<<<kGrid, kThreads, 0, sl.stream>>>(w);
    k_dfs<<<blocks(n_term), kThreads, 0, sl.stream>>>(T, w);
    k_fit<<<blocks(n_paths), kThreads, 0, sl.stream>>>(T, w);
    scan(sl, w.fflag, w.fidx, sl.d_sz + S_PATHS, 0, 0, n_paths + 1, w.tstate_b, sl.d_sz + S_PROPS);
    k_props<<<blocks(n_paths), kThreads, 0, sl.stream>>>(w);
    // bidding: the fit's one-edge bids, the rounds, the hit bids
    {
        Tables Tc = T;
        Work wc = w;
        uint32_t nsp = n_sp, rounds = h->cfg.edge_bidding_rounds;
        void* args[] = {&Tc, &wc, &nsp, &rounds};
        if (cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_bidding), dim3(h->coop_bid),
                                        dim3(kThreads), args, 0, sl.stream) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
    }
    k_convert<<<blocks(n_paths), kThreads, 0, sl.stream>>>(T, w);
    scan(sl, w.ecount, w.eoff, sl.d_sz + S_PROPS, 0, 0, n_paths + 1, w.tstate_b, sl.d_sz + S_SEEDS);
    k_seeds_out<<<blocks(n_paths), kThreads, 0, sl.stream>>>(w, *out);
    return cudaGetLastError() == cudaSuccess ? SEEDGB_OK : SEEDGB_CUDA_ERROR;
}

}  // namespace

extern "C" seedgb_status seedgb_gbts_run(seedgb_gbts* h, const seedgb_spacepoint_view* sps,
                                         const uint64_t* surface_link, const float* diameter,
                                         uint32_t n_meas, seedgb_seed_buffer* out, void* stream) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    const seedgb_status chk = check_event(sps, surface_link, diameter, n_meas, out);
    if (chk != SEEDGB_OK) return chk;
    Slot& sl = h->slot[0];
    sl.stream = static_cast<cudaStream_t>(stream);
    h->used = 1;
    h->last_slot = 0;
    if (cudaMemsetAsync(sl.d_sz + S_STATUS, 0, sizeof(uint32_t) * (S_COUNT - S_STATUS), sl.stream) !=
        cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    const seedgb_status st = front(h, sl, sps, surface_link, diameter, n_meas, out);
    if (st != SEEDGB_OK) return st;
    return finish(h, sl);
}

extern "C" seedgb_status seedgb_gbts_run_batch(seedgb_gbts* h, const seedgb_spacepoint_view* events,
                                               const uint64_t* const* surface_links,
                                               const float* const* diameters, const uint32_t* n_meas,
                                               uint32_t n_events, seedgb_seed_buffer* outs,
                                               void* stream) {
    if (!h || (n_events && (!events || !surface_links || !diameters || !n_meas || !outs)))
        return SEEDGB_INVALID_ARGUMENT;
    for (uint32_t e = 0; e < n_events; ++e) {
        const seedgb_status chk =
            check_event(&events[e], surface_links[e], diameters[e], n_meas[e], &outs[e]);
        if (chk != SEEDGB_OK) return chk;
    }
    if (n_events == 0) return SEEDGB_OK;
    const uint32_t S = std::min<uint32_t>(kMaxSlots, n_events);
    for (uint32_t k = 0; k < S; ++k) {
        Slot& sl = h->slot[k];
        if (!slot_init(sl)) return SEEDGB_CUDA_ERROR;
        sl.stream = static_cast<cudaStream_t>(stream);
        if (cudaMemsetAsync(sl.d_sz + S_STATUS, 0, sizeof(uint32_t) * (S_COUNT - S_STATUS),
                            sl.stream) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
    }
    h->used = S;
    seedgb_status st = SEEDGB_OK;
    for (uint32_t e = 0; e < n_events && st == SEEDGB_OK; ++e) {
        // the slot's previous event (e - S) gets its tail after event e - 1's
        // front is queued; then event e's front
        Slot& sl = h->slot[e % S];
        st = finish(h, sl);
        if (st == SEEDGB_OK)
            st = front(h, sl, &events[e], surface_links[e], diameters[e], n_meas[e], &outs[e]);
        h->last_slot = e % S;
    }
    for (uint32_t k = 0; k < S; ++k) {
        const uint32_t e = (h->last_slot + 1 + k) % S;  // the older pending event first
        const seedgb_status f = finish(h, h->slot[e]);
        if (st == SEEDGB_OK) st = f;
    }
    return st;
}

extern "C" seedgb_status seedgb_gbts_last_status(seedgb_gbts* h, void* stream) {
    if (!h) return SEEDGB_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    uint32_t worst = SEEDGB_OK;
    bool bad_input = false;
    for (uint32_t k = 0; k < h->used; ++k) {
        Slot& sl = h->slot[k];
        if (cudaMemcpyAsync(sl.h_sz, sl.d_sz, sizeof(uint32_t) * S_COUNT, cudaMemcpyDeviceToHost,
                            sl.stream) != cudaSuccess ||
            cudaStreamSynchronize(sl.stream) != cudaSuccess)
            return SEEDGB_CUDA_ERROR;
        worst = std::max(worst, sl.h_sz[S_STATUS]);
        bad_input |= sl.h_sz[S_BAD_INPUT] != 0;
    }
    if (bad_input) return SEEDGB_INVALID_ARGUMENT;
    return static_cast<seedgb_status>(worst);
}

extern "C" seedgb_status seedgb_gbts_counters(seedgb_gbts* h, uint64_t* counters) {
    if (!h || !counters) return SEEDGB_INVALID_ARGUMENT;
    Slot& sl = h->slot[h->last_slot];
    if (cudaMemcpyAsync(sl.h_sz, sl.d_sz, sizeof(uint32_t) * S_COUNT, cudaMemcpyDeviceToHost,
                        sl.stream) != cudaSuccess ||
        cudaStreamSynchronize(sl.stream) != cudaSuccess)
        return SEEDGB_CUDA_ERROR;
    const uint32_t* z = sl.h_sz;
    counters[0] = z[S_NODES];
    counters[1] = z[S_EDGES_MADE];
    counters[2] = z[S_CONN];
    counters[3] = z[S_CONNECTED];
    counters[4] = z[S_TERMINUS];
    counters[5] = z[S_PATHS];
    counters[6] = z[S_PROPS];
    counters[7] = z[S_REJECTED];
    counters[8] = z[S_SEEDS];
    return SEEDGB_OK;
}
