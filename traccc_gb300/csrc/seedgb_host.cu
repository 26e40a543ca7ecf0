// Host-side drivers over the C ABI, for C++ callers: the launch-shape
// autotuner of the batched seeding launch, and training and calibration of
// the learned doublet filter.  No counterpart in the reference (the
// benchmark's batching and learned-filter additions).  Everything here calls
// the library's public entry points (seedgb.h) plus two small gather kernels;
// the network's arithmetic is seedgb_mlp_grad / seedgb_mlp_adam.
//
// Determinism: the doublet dump appends records in the order the GPU finds
// them, so the records are put in (event, role, middle, other) order before
// anything depends on their order; negatives are sampled by a hash of
// (seed, event, middle, other), and shuffles use a seeded mt19937_64.  The
// same events, configuration and seed give the same network bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "seedgb.h"

namespace {

// ---------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DevBuf() { cudaFree(p); }
    bool alloc(size_t count) {
        if (count <= n && p) return true;
        cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(1, count)) != cudaSuccess) return false;
        n = count;
        return true;
    }
};

#define SEEDGB_TRY(x)                               \
    do {                                            \
        const seedgb_status st_ = (x);              \
        if (st_ != SEEDGB_OK) return st_;           \
    } while (0)
#define SEEDGB_CUDA(x)                                         \
    do {                                                       \
        if ((x) != cudaSuccess) return SEEDGB_CUDA_ERROR;      \
    } while (0)

uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// One doublet-dump record (48 bytes, seedgb_seeding_set_doublet_dump).
struct DumpRec {
    uint32_t middle, other, role_event;
    float feat[8];
    float logit;
};
static_assert(sizeof(DumpRec) == 48, "doublet record");

constexpr uint32_t kParams = 8 * 32 + 32 + 32 * 32 + 32 + 32 + 1;  // 1377
// Middles with more middle-top doublets than this are kept unscored by the
// gate a training run returns (seedgb_doublet_filter.gate_max_tops).
constexpr uint32_t kDefaultGateMaxTops = 32;

// Per-event seed buffers sized like the seeding path's maximum.
struct SeedSet {
    std::vector<DevBuf<uint32_t>> cols;  // 3 index columns per event
    std::vector<DevBuf<float>> qual;
    DevBuf<uint32_t> sizes;
    std::vector<seedgb_seed_buffer> bufs;
    bool make(const seedgb_spacepoint_view* ev, uint32_t n, uint32_t per_sp) {
        cols = std::vector<DevBuf<uint32_t>>(3 * n);
        qual = std::vector<DevBuf<float>>(n);
        bufs.assign(n, seedgb_seed_buffer{});
        if (!sizes.alloc(n)) return false;
        for (uint32_t e = 0; e < n; ++e) {
            const uint32_t cap = std::max<uint32_t>(1, per_sp * ev[e].size);
            for (int k = 0; k < 3; ++k)
                if (!cols[3 * e + k].alloc(cap)) return false;
            if (!qual[e].alloc(cap)) return false;
            bufs[e] = seedgb_seed_buffer{cols[3 * e].p, cols[3 * e + 1].p, cols[3 * e + 2].p,
                                         qual[e].p, cap, sizes.p + e};
        }
        return true;
    }
};

// Scored plain seeding of events [e0, e1): the top-doublet records (in the
// order the GPU found them) and, per event, the set of plain seeds'
// (middle, top) keys.
struct Scored {
    std::vector<DumpRec> tops;                       // role 1 only
    std::vector<std::unordered_set<uint64_t>> seeds;  // per event of the pass
    std::vector<std::unordered_map<uint32_t, uint32_t>> seeds_per_middle;
};

uint64_t mt_key(uint32_t middle, uint32_t top) {
    return (static_cast<uint64_t>(middle) << 32) | top;
}

seedgb_status scored_pass(seedgb_seeding* h, const seedgb_doublet_filter& scoring,
                          const seedgb_spacepoint_view* ev, uint32_t n, uint32_t per_sp,
                          DevBuf<DumpRec>& rec, Scored& out, cudaStream_t s) {
    SeedSet ss;
    if (!ss.make(ev, n, per_sp)) return SEEDGB_CUDA_ERROR;
    uint64_t total_sp = 0;
    for (uint32_t e = 0; e < n; ++e) total_sp += ev[e].size;
    if (!rec.p && !rec.alloc(80 * total_sp + 1024)) return SEEDGB_CUDA_ERROR;
    uint64_t n_rec = 0;
    for (int attempt = 0; attempt < 3; ++attempt) {
        SEEDGB_TRY(seedgb_seeding_set_filter(h, &scoring));
        SEEDGB_TRY(seedgb_seeding_set_doublet_dump(h, rec.p, rec.n));
        SEEDGB_TRY(seedgb_seeding_run_batch(h, ev, n, ss.bufs.data(), s));
        uint64_t n_trip = 0;
        SEEDGB_TRY(seedgb_seeding_filter_stats(h, n, nullptr, nullptr, &n_rec, &n_trip, s));
        if (n_rec <= rec.n) break;
        SEEDGB_TRY(seedgb_seeding_set_doublet_dump(h, nullptr, 0));
        if (!rec.alloc(n_rec + n_rec / 10 + 1024)) return SEEDGB_CUDA_ERROR;
    }
    SEEDGB_TRY(seedgb_seeding_set_doublet_dump(h, nullptr, 0));
    SEEDGB_TRY(seedgb_seeding_set_filter(h, nullptr));
    const seedgb_status st = seedgb_seeding_last_status(h, s);
    if (st != SEEDGB_OK) return st;
    if (n_rec > rec.n) return SEEDGB_CAPACITY_OVERFLOW;
    std::vector<DumpRec> all(n_rec);
    SEEDGB_CUDA(cudaMemcpy(all.data(), rec.p, sizeof(DumpRec) * n_rec, cudaMemcpyDeviceToHost));
    out.tops.clear();
    for (const DumpRec& r : all)
        if (r.role_event & 1u) out.tops.push_back(r);
    std::vector<uint32_t> sizes(n);
    SEEDGB_CUDA(cudaMemcpy(sizes.data(), ss.sizes.p, 4 * n, cudaMemcpyDeviceToHost));
    out.seeds.assign(n, {});
    out.seeds_per_middle.assign(n, {});
    for (uint32_t e = 0; e < n; ++e) {
        const uint32_t k = std::min(sizes[e], ss.bufs[e].capacity);
        std::vector<uint32_t> mid(k), top(k);
        SEEDGB_CUDA(cudaMemcpy(mid.data(), ss.bufs[e].middle_index, 4ull * k,
                               cudaMemcpyDeviceToHost));
        SEEDGB_CUDA(cudaMemcpy(top.data(), ss.bufs[e].top_index, 4ull * k,
                               cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < k; ++i) {
            out.seeds[e].insert(mt_key(mid[i], top[i]));
            ++out.seeds_per_middle[e][mid[i]];
        }
    }
    return SEEDGB_OK;
}

__global__ void k_gather_rows(const float4* __restrict__ x, const float* __restrict__ y,
                              const uint32_t* __restrict__ perm, uint32_t n,
                              float4* __restrict__ xo, float* __restrict__ yo) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j = perm[i];
        xo[2 * i] = x[2 * j];
        xo[2 * i + 1] = x[2 * j + 1];
        yo[i] = y[j];
    }
}

void scoring_filter(const float* params, const float norm[16], const float* edges,
                    uint32_t n_edges, seedgb_doublet_filter& f) {
    std::memset(&f, 0, sizeof f);
    for (int i = 0; i < 8; ++i) {
        f.mu[i] = norm[i];
        f.isd[i] = norm[8 + i];
    }
    std::memcpy(f.w1, params, sizeof f.w1);
    std::memcpy(f.b1, params + 256, sizeof f.b1);
    std::memcpy(f.w2, params + 288, sizeof f.w2);
    std::memcpy(f.b2, params + 1312, sizeof f.b2);
    std::memcpy(f.w3, params + 1344, sizeof f.w3);
    f.b3 = params[1376];
    f.threshold[0] = f.threshold[1] = -INFINITY;
    f.n_edges = n_edges;
    for (uint32_t i = 0; i < n_edges && i < 15; ++i) f.edges[i] = edges[i];
    f.prune_bottom = f.prune_top = SEEDGB_FILTER_KEEP;
    f.band[0] = 0.f;
    f.band[1] = 1.f;
}

}  // namespace

extern "C" {

seedgb_status seedgb_seeding_autotune(seedgb_seeding* h, const seedgb_spacepoint_view* events,
                                      uint32_t n_events, seedgb_seed_buffer* outs,
                                      const seedgb_tune* candidates, uint32_t n_candidates,
                                      uint32_t reps, seedgb_tune* best, float* times_ms,
                                      void* stream) {
    if (!h || !events || !outs || !n_events || !best || (n_candidates && !candidates))
        return SEEDGB_INVALID_ARGUMENT;
    std::vector<seedgb_tune> grid;
    if (candidates) {
        grid.assign(candidates, candidates + n_candidates);
    } else {
        for (int w : {8, 12, 16})
            for (int m : {64, 256, 384, 512, 1024})
                for (int nb : {1536, 2048, 2560, 3072})
                    for (int c : {1, 2}) grid.push_back(seedgb_tune{w, m, nb, c});
    }
    reps = std::max(1u, reps);
    uint64_t total = 0;
    for (uint32_t e = 0; e < n_events; ++e) total += events[e].size;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaEvent_t t0, t1;
    SEEDGB_CUDA(cudaEventCreate(&t0));
    if (cudaEventCreate(&t1) != cudaSuccess) {
        cudaEventDestroy(t0);
        return SEEDGB_CUDA_ERROR;
    }
    std::vector<seedgb_tune> measured;
    float best_ms = INFINITY;
    seedgb_status st = SEEDGB_OK;
    for (size_t i = 0; i < grid.size() && st == SEEDGB_OK; ++i) {
        if (times_ms) times_ms[i] = -1.f;
        if (seedgb_seeding_set_tune(h, &grid[i]) != SEEDGB_OK) continue;  // does not fit
        seedgb_tune eff;
        if ((st = seedgb_seeding_get_tune(h, &eff)) != SEEDGB_OK) break;
        bool seen = false;
        for (const seedgb_tune& m : measured)
            seen |= std::memcmp(&m, &eff, sizeof eff) == 0;
        if (seen) continue;  // clamped to a shape already measured
        measured.push_back(eff);
        if ((st = seedgb_seeding_graph_create(h, n_events, total)) != SEEDGB_OK) break;
        if ((st = seedgb_seeding_graph_launch(h, events, n_events, outs, stream)) != SEEDGB_OK)
            break;
        std::vector<float> t(reps);
        for (uint32_t r = 0; r < reps && st == SEEDGB_OK; ++r) {
            if (cudaEventRecord(t0, s) != cudaSuccess) st = SEEDGB_CUDA_ERROR;
            if (st == SEEDGB_OK)
                st = seedgb_seeding_graph_launch(h, events, n_events, outs, stream);
            if (st == SEEDGB_OK && (cudaEventRecord(t1, s) != cudaSuccess ||
                                    cudaEventSynchronize(t1) != cudaSuccess ||
                                    cudaEventElapsedTime(&t[r], t0, t1) != cudaSuccess))
                st = SEEDGB_CUDA_ERROR;
        }
        if (st != SEEDGB_OK) break;
        if ((st = seedgb_seeding_last_status(h, stream)) != SEEDGB_OK) break;
        std::sort(t.begin(), t.end());
        const float ms = t[t.size() / 2];
        if (times_ms) times_ms[i] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            *best = eff;
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (st != SEEDGB_OK) return st;
    if (!(best_ms < INFINITY)) return SEEDGB_UNSUPPORTED;  // no shape fits this device
    SEEDGB_TRY(seedgb_seeding_set_tune(h, best));
    return seedgb_seeding_graph_create(h, n_events, total);
}

seedgb_status seedgb_filter_train(seedgb_seeding* h, const seedgb_spacepoint_view* events,
                                  uint32_t n_events, const float* band_edges, uint32_t n_edges,
                                  const seedgb_filter_train_config* cfg,
                                  seedgb_doublet_filter* out, float* loss_per_epoch,
                                  void* stream) {
    if (!h || !events || !n_events || !cfg || !out || n_edges > 15 || (n_edges && !band_edges) ||
        !cfg->epochs || !cfg->batch || !(cfg->neg_keep >= 0.f && cfg->neg_keep <= 1.f))
        return SEEDGB_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t per_pass = std::max(1u, cfg->events_per_pass);
    // labels from plain seeding (the network does not affect the dump's
    // features or the seeds: a scoring filter prunes nothing)
    std::vector<float> p0(kParams, 0.f), norm0(16, 0.f);
    for (int i = 0; i < 8; ++i) norm0[8 + i] = 1.f;
    seedgb_doublet_filter scoring;
    scoring_filter(p0.data(), norm0.data(), band_edges, n_edges, scoring);
    std::vector<float> feats;
    std::vector<float> labels;
    uint64_t n_pos = 0;
    DevBuf<DumpRec> rec;
    for (uint32_t e0 = 0; e0 < n_events; e0 += per_pass) {
        const uint32_t n = std::min(per_pass, n_events - e0);
        Scored sc;
        SEEDGB_TRY(scored_pass(h, scoring, events + e0, n, 8, rec, sc, s));
        // keep the positives and a hashed share of the negatives, then put
        // the kept samples in (event, middle, partner) order
        std::vector<std::pair<const DumpRec*, bool>> kept;
        for (const DumpRec& r : sc.tops) {
            const uint32_t e = r.role_event >> 1;
            const bool pos = sc.seeds[e].count(mt_key(r.middle, r.other)) != 0;
            const uint64_t hsh = splitmix64(cfg->seed ^ splitmix64(
                (static_cast<uint64_t>(e0 + e) << 42) ^ (static_cast<uint64_t>(r.middle) << 21) ^
                r.other));
            const double u = static_cast<double>(hsh >> 11) * 0x1p-53;
            if (pos || u < cfg->neg_keep) kept.emplace_back(&r, pos);
        }
        std::sort(kept.begin(), kept.end(), [](const auto& a, const auto& b) {
            if (a.first->role_event != b.first->role_event)
                return a.first->role_event < b.first->role_event;
            if (a.first->middle != b.first->middle) return a.first->middle < b.first->middle;
            return a.first->other < b.first->other;
        });
        for (const auto& k : kept) {
            feats.insert(feats.end(), k.first->feat, k.first->feat + 8);
            labels.push_back(k.second ? 1.f : 0.f);
            n_pos += k.second;
        }
    }
    const uint64_t n64 = labels.size();
    if (n64 == 0 || n_pos == 0) return SEEDGB_EMPTY;
    if (n64 > 0xffffffffull) return SEEDGB_SIZE_LIMIT;
    const uint32_t n = static_cast<uint32_t>(n64);
    // input standardisation over the training samples
    float norm[16];
    for (int k = 0; k < 8; ++k) {
        double m = 0, q = 0;
        for (uint32_t i = 0; i < n; ++i) m += feats[8ull * i + k];
        m /= n;
        for (uint32_t i = 0; i < n; ++i) {
            const double d = feats[8ull * i + k] - m;
            q += d * d;
        }
        const double sd = std::max(std::sqrt(q / std::max(1u, n - 1)), 1e-6);
        norm[k] = static_cast<float>(m);
        norm[8 + k] = static_cast<float>(1.0 / sd);
    }
    // He-uniform weights, zero biases
    std::mt19937_64 rng(cfg->seed);
    std::vector<float> P(kParams, 0.f);
    auto fill = [&](uint32_t off, uint32_t cnt, double lim) {
        std::uniform_real_distribution<double> d(-lim, lim);
        for (uint32_t i = 0; i < cnt; ++i) P[off + i] = static_cast<float>(d(rng));
    };
    fill(0, 256, std::sqrt(6.0 / 8));
    fill(288, 1024, std::sqrt(6.0 / 32));
    fill(1344, 32, std::sqrt(3.0 / 32));
    const float pos_weight =
        static_cast<float>(std::max(1.0, static_cast<double>(n - n_pos) / n_pos));
    DevBuf<float> dX, dY, dXs, dYs, dP, dG, dM, dV, dN, dL;
    DevBuf<uint32_t> dPerm;
    const uint32_t nb = (n + cfg->batch - 1) / cfg->batch;
    if (!dX.alloc(8ull * n) || !dY.alloc(n) || !dXs.alloc(8ull * n) || !dYs.alloc(n) ||
        !dP.alloc(kParams) || !dG.alloc(kParams) || !dM.alloc(kParams) || !dV.alloc(kParams) ||
        !dN.alloc(16) || !dL.alloc(nb) || !dPerm.alloc(n))
        return SEEDGB_CUDA_ERROR;
    SEEDGB_CUDA(cudaMemcpy(dX.p, feats.data(), 32ull * n, cudaMemcpyHostToDevice));
    SEEDGB_CUDA(cudaMemcpy(dY.p, labels.data(), 4ull * n, cudaMemcpyHostToDevice));
    SEEDGB_CUDA(cudaMemcpy(dP.p, P.data(), 4ull * kParams, cudaMemcpyHostToDevice));
    SEEDGB_CUDA(cudaMemcpy(dN.p, norm, sizeof norm, cudaMemcpyHostToDevice));
    SEEDGB_CUDA(cudaMemsetAsync(dM.p, 0, 4ull * kParams, s));
    SEEDGB_CUDA(cudaMemsetAsync(dV.p, 0, 4ull * kParams, s));
    std::vector<uint32_t> perm(n);
    std::vector<float> losses(nb);
    uint32_t step = 0;
    for (uint32_t ep = 0; ep < cfg->epochs; ++ep) {
        for (uint32_t i = 0; i < n; ++i) perm[i] = i;
        std::mt19937_64 sh(cfg->seed * 1000003ull + ep + 1);
        for (uint32_t i = n - 1; i > 0; --i) {
            const uint32_t j = static_cast<uint32_t>(sh() % (static_cast<uint64_t>(i) + 1));
            std::swap(perm[i], perm[j]);
        }
        SEEDGB_CUDA(cudaMemcpyAsync(dPerm.p, perm.data(), 4ull * n, cudaMemcpyHostToDevice, s));
        k_gather_rows<<<1024, 256, 0, s>>>(reinterpret_cast<const float4*>(dX.p), dY.p, dPerm.p,
                                           n, reinterpret_cast<float4*>(dXs.p), dYs.p);
        SEEDGB_CUDA(cudaGetLastError());
        for (uint32_t b = 0; b < nb; ++b) {
            const uint32_t i0 = b * cfg->batch, cnt = std::min(cfg->batch, n - i0);
            SEEDGB_TRY(seedgb_mlp_grad(dP.p, dN.p, dXs.p + 8ull * i0, dYs.p + i0, cnt, pos_weight,
                                       dG.p, dL.p + b, stream));
            SEEDGB_TRY(seedgb_mlp_adam(dP.p, dG.p, dM.p, dV.p, kParams, ++step,
                                       cfg->learning_rate, 0.9f, 0.999f, 1e-8f, stream));
        }
        SEEDGB_CUDA(cudaMemcpyAsync(losses.data(), dL.p, 4ull * nb, cudaMemcpyDeviceToHost, s));
        SEEDGB_CUDA(cudaStreamSynchronize(s));
        if (loss_per_epoch) {
            double acc = 0;
            for (float l : losses) acc += l;
            loss_per_epoch[ep] = static_cast<float>(acc / nb);
        }
    }
    SEEDGB_CUDA(cudaMemcpy(P.data(), dP.p, 4ull * kParams, cudaMemcpyDeviceToHost));
    scoring_filter(P.data(), norm, band_edges, n_edges, *out);
    out->prune_top = SEEDGB_FILTER_GATE_MIDDLE;
    out->gate_max_tops = kDefaultGateMaxTops;
    return SEEDGB_OK;
}

seedgb_status seedgb_filter_calibrate_gate(seedgb_seeding* h, const seedgb_spacepoint_view* events,
                                           uint32_t n_events, const uint32_t* class_max,
                                           uint32_t n_classes, float target, float min_event,
                                           float margin, seedgb_doublet_filter* f,
                                           float* recall_out, float* pruned_out, void* stream) {
    if (!h || !events || !n_events || !f || n_classes > 8 || (n_classes && !class_max))
        return SEEDGB_INVALID_ARGUMENT;
    for (uint32_t k = 1; k < n_classes; ++k)
        if (!(class_max[k - 1] <= class_max[k])) return SEEDGB_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    seedgb_doublet_filter scoring = *f;
    scoring.prune_bottom = scoring.prune_top = SEEDGB_FILTER_KEEP;
    scoring.threshold[0] = scoring.threshold[1] = -INFINITY;
    scoring.band[0] = 0.f;
    scoring.band[1] = 1.f;
    scoring.n_size_classes = 0;
    // per middle with both roles: event, best middle-top logit, plain seeds,
    // middle-top doublets
    struct Mid {
        uint32_t ev;
        float best;
        uint32_t seeds, n_mt;
    };
    std::vector<Mid> mids;
    DevBuf<DumpRec> rec;
    const uint32_t per_pass = 8;
    for (uint32_t e0 = 0; e0 < n_events; e0 += per_pass) {
        const uint32_t n = std::min(per_pass, n_events - e0);
        Scored sc;
        SEEDGB_TRY(scored_pass(h, scoring, events + e0, n, 8, rec, sc, s));
        // group by (event, middle); the result does not depend on the order
        std::unordered_map<uint64_t, Mid> by_mid;
        by_mid.reserve(sc.tops.size() / 16 + 16);
        for (const DumpRec& r : sc.tops) {
            const uint32_t e = r.role_event >> 1;
            auto ins = by_mid.emplace(mt_key(e, r.middle), Mid{e0 + e, -INFINITY, 0, 0});
            Mid& m = ins.first->second;
            if (ins.second) {
                const auto it = sc.seeds_per_middle[e].find(r.middle);
                m.seeds = it == sc.seeds_per_middle[e].end() ? 0u : it->second;
            }
            m.best = std::max(m.best, r.logit);
            ++m.n_mt;
        }
        for (const auto& kv : by_mid) mids.push_back(kv.second);
    }
    const uint32_t nc = std::max(1u, n_classes);
    auto class_of = [&](uint32_t e) {
        for (uint32_t k = 0; k + 1 < nc; ++k)
            if (events[e].size <= class_max[k]) return k;
        return nc - 1;
    };
    // exact recall and gated share per event at threshold thr (class k)
    std::vector<double> tot(n_events), keep(n_events), mt(n_events), gated(n_events);
    const uint32_t max_tops = f->gate_max_tops;
    const auto gateable = [&](const Mid& m) { return max_tops == 0 || m.n_mt <= max_tops; };
    auto evaluate = [&](uint32_t k, float thr) {
        std::fill(tot.begin(), tot.end(), 0.0);
        std::fill(keep.begin(), keep.end(), 0.0);
        std::fill(mt.begin(), mt.end(), 0.0);
        std::fill(gated.begin(), gated.end(), 0.0);
        for (const Mid& m : mids) {
            if (class_of(m.ev) != k) continue;
            const bool kept = !gateable(m) || m.best >= thr;
            tot[m.ev] += m.seeds;
            keep[m.ev] += kept ? m.seeds : 0;
            mt[m.ev] += m.n_mt;
            gated[m.ev] += kept ? 0 : m.n_mt;
        }
    };
    seedgb_doublet_filter res = *f;
    res.prune_bottom = SEEDGB_FILTER_KEEP;
    res.prune_top = SEEDGB_FILTER_GATE_MIDDLE;
    res.n_size_classes = n_classes;
    for (uint32_t k = 0; k < nc; ++k) {
        std::vector<float> cand;
        for (const Mid& m : mids)
            if (class_of(m.ev) == k && m.seeds > 0 && gateable(m)) cand.push_back(m.best);
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        float chosen = -INFINITY;
        auto passes = [&](float thr) {
            evaluate(k, thr);
            double T = 0, K = 0, mn = 1.0;
            bool any = false;
            for (uint32_t e = 0; e < n_events; ++e) {
                if (class_of(e) != k || tot[e] == 0) continue;
                any = true;
                T += tot[e];
                K += keep[e];
                mn = std::min(mn, keep[e] / tot[e]);
            }
            return !any || (K / T >= target && mn >= min_event);
        };
        int64_t lo = 0, hi = static_cast<int64_t>(cand.size()) - 1;
        while (lo <= hi) {  // recall is non-increasing in the threshold
            const int64_t mid = (lo + hi) / 2;
            if (passes(cand[mid])) {
                chosen = cand[mid];
                lo = mid + 1;
            } else {
                hi = mid - 1;
            }
        }
        evaluate(k, chosen);
        double fmin = 1.0, fmax = 0.0;
        bool any = false;
        for (uint32_t e = 0; e < n_events; ++e) {
            if (class_of(e) != k) continue;
            const double fr = mt[e] > 0 ? gated[e] / mt[e] : 0.0;
            if (recall_out) recall_out[e] = tot[e] > 0 ? static_cast<float>(keep[e] / tot[e]) : 1.f;
            if (pruned_out) pruned_out[e] = static_cast<float>(fr);
            fmin = std::min(fmin, fr);
            fmax = std::max(fmax, fr);
            any = true;
        }
        if (!any) fmin = 0.0, fmax = 1.0;
        const float blo = static_cast<float>(std::max(0.0, fmin - margin));
        const float bhi = static_cast<float>(std::min(1.0, fmax + margin));
        if (k < 8 && n_classes) {
            res.size_class_max[k] = class_max[k];
            res.size_class_threshold[k][0] = -INFINITY;
            res.size_class_threshold[k][1] = chosen;
            res.size_class_band[k][0] = blo;
            res.size_class_band[k][1] = bhi;
        }
        if (k == nc - 1) {
            res.threshold[0] = -INFINITY;
            res.threshold[1] = chosen;
            res.band[0] = blo;
            res.band[1] = bhi;
        }
    }
    *f = res;
    return SEEDGB_OK;
}

}  // extern "C"
