/* CPU oracle of traccc's GBTS seeding -- TEST INFRASTRUCTURE ONLY.
 *
 * A sequential restatement of the reference's GBTS kernels
 * (the .ipp files of device/common/include/traccc/gbts_seeding/device/impl) in the order
 * device/common/src/gbts_seeding/gbts_seeding_algorithm.cpp runs them, with
 * one canonical order wherever the reference's output depends on the order
 * in which its atomics land:
 *   - nodes of one (eta, phi) cell in ascending spacepoint index;
 *   - edges by (work item, thread, outer node, inner node): work items in
 *     bin-table order, each bin-1 chunk of at most 128 nodes its own work
 *     item; 128 threads per item, thread t taking outer nodes t, t + 128, ...;
 *   - the edges leaving a node in ascending edge index; the first
 *     max_num_neighbours matches kept;
 *   - connected edges numbered in ascending edge index;
 *   - terminus edges in ascending connected-edge index, the path store as a
 *     depth-first pre-order walk below each terminus edge in turn;
 *   - seed proposals in ascending path-store index, output seeds by proposal.
 * Everything else -- the cuts, the CCA, the Kalman fit, the bidding -- is the
 * reference's arithmetic in its expression order (compile without FMA
 * contraction).  Transcendental functions are correctly rounded: atan2 and
 * log in double, rounded to float (the GPU library does the same), where the
 * reference calls the float functions of its platform.
 */
#include "gbts_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAX_CCA_ITER 15u   /* gbts_consts::max_cca_iter */
#define NODE_BUFFER 128u   /* gbts_consts::node_buffer_length */
#define EDGE_THREADS 128u  /* threads per work item of gbts_make_graph_edges */

static const float PI_F = 3.14159265358979323846f;
#define TWO_PI_F (2.0f * PI_F)

/* std::min / std::max as the reference calls them (comparison based) */
static float smin(float a, float b) { return (b < a) ? b : a; }
static float smax(float a, float b) { return (a < b) ? b : a; }

static float cr_atan2f(float y, float x) { return (float)atan2((double)y, (double)x); }
static float cr_logf(float x) { return (float)log((double)x); }

/* traccc::detail::wrap_phi (core/include/traccc/utils/trigonometric_helpers.hpp:18-38) */
static float wrap_phi(float phi) {
    const float diff = phi - (-PI_F);
    return ((0 <= diff) && (diff < TWO_PI_F)) ? phi : (phi - TWO_PI_F * floorf(diff / TWO_PI_F));
}

void or_gbts_config_default(or_gbts_config* c) {
    memset(c, 0, sizeof(*c));
    c->tMin_slope = 6.7f;
    c->offset = 0.2f;
    c->tMax_min = 1.6f;
    c->tMax_correction = 0.15f;
    c->tMax_slope = 6.1f;
    c->maxTau = 36.0f;
    c->useTauLUT = 0;
    c->tau_lut_inv_bin = 0.0f;
    c->tauLutSize = 0;
    c->minDeltaRadius = 2.0f;
    c->min_z0 = -160.0f;
    c->max_z0 = 160.0f;
    c->maxOuterRadius = 350.0f;
    c->tau_roi = 45.0f;
    c->cut_zMinU = c->min_z0 - c->maxOuterRadius * c->tau_roi;
    c->cut_zMaxU = c->max_z0 + c->maxOuterRadius * c->tau_roi;
    c->max_Kappa = 3.75e-4f;
    c->low_Kappa_d0 = 0.0f;
    c->high_Kappa_d0 = 0.0f;
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
    c->qual_scale = 0.01f * (float)INT_MAX / (c->add_hit * (float)MAX_CCA_ITER);
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

static uint64_t field(uint64_t v, uint32_t shift, uint32_t bits) {
    const uint64_t m = bits >= 64 ? ~0ull : ((1ull << bits) - 1ull);
    return shift >= 64 ? 0 : ((v >> shift) & m);
}

typedef struct {
    uint64_t id;
    int16_t layer;
} geo_pair;

static int geo_desc(const void* a, const void* b) {
    const uint64_t x = ((const geo_pair*)a)->id, y = ((const geo_pair*)b)->id;
    return (x > y) ? -1 : (x < y) ? 1 : 0;
}

/* gbts_seedfinder_config::setLinkingScheme (gbts_seeding_config.cpp:19-142):
 * pairs sorted by descending barcode; a volume whose surfaces all lie on one
 * layer maps to that layer, a volume split over layers to -(its first entry in
 * the surface map + 1); the walk ends with a (UINT_MAX, -1) sentinel.  The
 * volume map is resized to (largest volume + 1) zeros and then as many
 * SHRT_MAX entries appended, the way the reference builds it (volumes below
 * the largest that are missing from the binning therefore map to layer 0). */
int or_gbts_linking(or_gbts_config* c, float minPt, const uint64_t* geoid,
                    const int16_t* geoid_layer, uint32_t n, int16_t* volume_map,
                    uint32_t volume_cap, uint32_t* n_volumes, uint32_t* surface_map,
                    uint32_t surface_cap, uint32_t* n_surfaces) {
    if (n == 0) return -1;
    geo_pair* g = (geo_pair*)malloc(sizeof(geo_pair) * (n + 1));
    for (uint32_t i = 0; i < n; ++i) {
        g[i].id = geoid[i];
        g[i].layer = geoid_layer[i];
    }
    qsort(g, n, sizeof(geo_pair), geo_desc);
    const uint32_t largest = (uint32_t)field(g[0].id, c->volume_shift, c->volume_bits);
    if (largest >= SHRT_MAX) {
        free(g);
        return -1;
    }
    int16_t current_volume = (int16_t)largest;
    int layer_change = 0;
    int16_t current_layer = g[0].layer;
    g[n].id = UINT_MAX;
    g[n].layer = -1;
    /* (bin, volume) pairs in the order the reference records them */
    int16_t* vb = (int16_t*)malloc(sizeof(int16_t) * (n + 1));
    uint32_t* vv = (uint32_t*)malloc(sizeof(uint32_t) * (n + 1));
    uint32_t nv = 0, ns = 0;
    uint32_t* sv = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (n + 1));
    uint32_t nsv = 0;
    for (uint32_t i = 0; i <= n; ++i) {
        const int16_t vol = (int16_t)field(g[i].id, c->volume_shift, c->volume_bits);
        if (current_volume != vol) {
            int16_t bin = current_layer;
            if (layer_change) {
                bin = (int16_t)(-1 * (int16_t)(ns + 1));
                for (uint32_t k = 0; k < nsv; ++k) {
                    if (ns >= surface_cap) {
                        free(g); free(vb); free(vv); free(sv);
                        return -1;
                    }
                    surface_map[2 * ns] = sv[2 * k];
                    surface_map[2 * ns + 1] = sv[2 * k + 1];
                    ++ns;
                }
            }
            vb[nv] = bin;
            vv[nv] = (uint32_t)(uint16_t)current_volume;
            ++nv;
            current_volume = vol;
            current_layer = g[i].layer;
            layer_change = 0;
            nsv = 0;
        }
        layer_change |= (current_layer != g[i].layer);
        sv[2 * nsv] = (uint32_t)field(g[i].id, c->index_shift, c->index_bits);
        sv[2 * nsv + 1] = (uint32_t)(int32_t)g[i].layer;
        ++nsv;
    }
    const uint32_t nvol = 2 * (largest + 1);
    int rc = 0;
    if (nvol > volume_cap) {
        rc = -1;
    } else {
        for (uint32_t i = 0; i <= largest; ++i) volume_map[i] = 0;
        for (uint32_t i = largest + 1; i < nvol; ++i) volume_map[i] = SHRT_MAX;
        for (uint32_t k = 0; k < nv; ++k)
            if (vv[k] < nvol) volume_map[vv[k]] = vb[k];
        *n_volumes = nvol;
        *n_surfaces = ns;
        if (ns > SHRT_MAX) rc = -1;
    }
    free(g); free(vb); free(vv); free(sv);
    if (rc != 0) return rc;
    const float ptScale = 900.0f / minPt;
    c->min_delta_phi *= ptScale;
    c->dphi_coeff *= ptScale;
    c->min_delta_phi_low_dr *= ptScale;
    c->dphi_coeff_low_dr *= ptScale;
    c->max_Kappa *= ptScale;
    return 0;
}

typedef struct { float x, y, z, w; } f4;

/* ---------------------------------------------------------------------------
 * Kalman fit of a path (gbts_fit_segments.ipp:37-251)
 * ------------------------------------------------------------------------- */
typedef struct {
    float X[3], Y[2];
    float c, s, refX, refY;
    float J;
    int head_type;
    float Cx[6];
    float Cy[3];
} edge_state;

#define CX(st, i, j) ((st)->Cx[(i) + (j) + 1 * ((i) != 0) * ((j) != 0)])
#define CY(st, i, j) ((st)->Cy[(i) + (j)])

static void state_init(edge_state* st, f4 n1, f4 n2) {
    st->J = 0.0f;
    st->head_type = (n1.w < 0);
    const float dx = n1.x - n2.x;
    const float dy = n1.y - n2.y;
    const float L = sqrtf(dx * dx + dy * dy);
    const float r1 = sqrtf(n1.x * n1.x + n1.y * n1.y);
    const float r2 = sqrtf(n2.x * n2.x + n2.y * n2.y);
    st->s = dy / L;
    st->c = dx / L;
    st->refX = n2.x * st->c + n2.y * st->s;
    st->refY = r2;
    st->X[0] = -n2.x * st->s + n2.y * st->c;
    st->X[1] = 0.0f;
    st->X[2] = 0.0f;
    st->Y[0] = n2.z;
    st->Y[1] = (n1.z - n2.z) / (r1 - r2);
    memset(st->Cx, 0, sizeof(st->Cx));
    memset(st->Cy, 0, sizeof(st->Cy));
    CX(st, 0, 0) = 0.25f;
    CX(st, 1, 1) = 0.001f;
    CX(st, 2, 2) = 0.001f;
    CY(st, 0, 0) = 1.5f;
    CY(st, 1, 1) = 0.001f;
}

static int kalman_update(edge_state* nt, const edge_state* ts, f4 node,
                         const or_gbts_config* p, float max_z0) {
    const float tau2 = ts->Y[1] * ts->Y[1];
    const float invSin2 = 1 + tau2;
    const float lenCorr = (node.w != -1) ? invSin2 : invSin2 / tau2;
    const float minPtFrac = fabsf(ts->X[2]) * p->inv_max_curvature;
    const float corrMS = p->sigmaMS * minPtFrac;
    const float sigma2 = p->radLen * lenCorr * corrMS * corrMS;
    const float m_Cx11 = CX(ts, 1, 1) + sigma2;
    const float m_Cy11 = CY(ts, 1, 1) + sigma2;
    const float r = sqrtf(node.x * node.x + node.y * node.y);
    nt->refX = node.x * ts->c + node.y * ts->s;
    const float mx = -node.x * ts->s + node.y * ts->c;
    nt->refY = r;
    const float my = node.z;
    const float A = nt->refX - ts->refX;
    const float B = (0.5f) * A * A;
    const float dr = nt->refY - ts->refY;
    nt->X[0] = ts->X[0] + ts->X[1] * A + ts->X[2] * B;
    nt->X[1] = ts->X[1] + ts->X[2] * A;
    nt->X[2] = ts->X[2];
    CX(nt, 0, 0) = CX(ts, 0, 0) + 2 * CX(ts, 0, 1) * A + 2 * CX(ts, 0, 2) * B + A * m_Cx11 * A +
                   2 * A * CX(ts, 1, 2) * B + B * CX(ts, 2, 2) * B;
    CX(nt, 0, 1) = CX(ts, 0, 1) + m_Cx11 * A + CX(ts, 1, 2) * B + CX(ts, 0, 2) * A +
                   A * CX(ts, 1, 2) * A + A * CX(ts, 2, 2) * B;
    CX(nt, 0, 2) = CX(ts, 0, 2) + CX(ts, 1, 2) * A + CX(ts, 2, 2) * B;
    CX(nt, 1, 1) = m_Cx11 + 2 * A * CX(ts, 1, 2) + A * CX(ts, 2, 2) * A;
    CX(nt, 1, 2) = CX(ts, 1, 2) + CX(ts, 2, 2) * A;
    CX(nt, 2, 2) = CX(ts, 2, 2);
    nt->Y[0] = ts->Y[0] + ts->Y[1] * dr;
    nt->Y[1] = ts->Y[1];
    CY(nt, 0, 0) = CY(ts, 0, 0) + 2 * CY(ts, 0, 1) * dr + dr * m_Cy11 * dr;
    CY(nt, 0, 1) = CY(ts, 0, 1) + dr * m_Cy11;
    CY(nt, 1, 1) = m_Cy11;
    const float resid_x = mx - nt->X[0];
    const float resid_y = my - nt->Y[0];
    float sigma_rz = 0;
    if (!ts->head_type) {
        sigma_rz = p->sigma_y;
    } else {
        sigma_rz = p->sigma_y * ts->Y[1];
    }
    const float inv_Dx = CX(nt, 0, 0) + p->sigma_x * p->sigma_x;
    const float Dx = 1 / inv_Dx;
    const float Dy = 1 / (CY(nt, 0, 0) + sigma_rz * sigma_rz);
    const float dchi2_x = resid_x * resid_x * Dx;
    const float dchi2_y = resid_y * resid_y * Dy;
    if (dchi2_x > p->maxDChi2_x || dchi2_y > p->maxDChi2_y) return 0;
    nt->J = ts->J + (p->add_hit - dchi2_x * p->weight_x - dchi2_y * p->weight_y);
    for (int i = 0; i < 3; i++) nt->X[i] += Dx * CX(nt, 0, i) * resid_x;
    if (fabsf(nt->X[2]) * p->inv_max_curvature > 1.0f) return 0;
    for (int i = 0; i < 2; i++) nt->Y[i] += Dx * CY(nt, 0, i) * resid_y;
    const float z0 = nt->Y[0] - nt->refY * ts->Y[1];
    if (fabsf(z0) > max_z0) return 0;
    CX(nt, 2, 2) = Dx * (CX(nt, 2, 2) * inv_Dx - CX(nt, 0, 2) * CX(nt, 0, 2));
    CX(nt, 1, 2) = Dx * (CX(nt, 1, 2) * inv_Dx - CX(nt, 0, 1) * CX(nt, 0, 2));
    CX(nt, 1, 1) = Dx * (CX(nt, 1, 1) * inv_Dx - CX(nt, 0, 1) * CX(nt, 0, 1));
    CX(nt, 0, 2) = Dx * (CX(nt, 0, 2) * inv_Dx - CX(nt, 0, 0) * CX(nt, 0, 2));
    CX(nt, 0, 1) = Dx * (CX(nt, 0, 1) * inv_Dx - CX(nt, 0, 0) * CX(nt, 0, 1));
    CX(nt, 0, 0) *= Dx * (p->sigma_x * p->sigma_x);
    CY(nt, 1, 1) -= Dy * CY(nt, 0, 1) * CY(nt, 0, 1);
    CY(nt, 0, 1) -= Dy * CY(nt, 0, 0) * CY(nt, 0, 1);
    CY(nt, 0, 0) -= Dy * CY(nt, 0, 0) * CY(nt, 0, 0);
    nt->c = ts->c;
    nt->s = ts->s;
    nt->head_type = (node.w < 0);
    return 1;
}

/* gbts_estimate_seed_params (gbts_convert_seeds.ipp:33-67) */
static void estimate_seed_params(const f4 sps[3], float* curv_out, float* cot_out) {
    float u[2], v[2];
    const float x0 = sps[1].x;
    const float y0 = sps[1].y;
    const float r0 = sqrtf(x0 * x0 + y0 * y0);
    const float cosA = x0 / r0;
    const float sinA = y0 / r0;
    for (unsigned k = 0; k < 2; k++) {
        const unsigned sp_idx = (k == 1) ? 2u : k;
        const float dx = sps[sp_idx].x - x0;
        const float dy = sps[sp_idx].y - y0;
        const float r2_inv = 1.0f / (dx * dx + dy * dy);
        const float xn = dx * cosA + dy * sinA;
        const float yn = -dx * sinA + dy * cosA;
        u[k] = xn * r2_inv;
        v[k] = yn * r2_inv;
    }
    const float du = u[0] - u[1];
    if (du == 0.0f) {
        *curv_out = 0.0f;
        *cot_out = 0.0f;
        return;
    }
    const float A = (v[0] - v[1]) / du;
    const float B = v[1] - A * u[1];
    *curv_out = 1000.0f * B / sqrtf(1 + A * A);
    *cot_out = (sps[2].z - sps[1].z) / (sqrtf(sps[2].x * sps[2].x + sps[2].y * sps[2].y) - r0);
}

typedef struct {
    uint32_t sp;
    uint32_t cell;
} node_key;

static int node_cmp(const void* a, const void* b) {
    const node_key* x = (const node_key*)a;
    const node_key* y = (const node_key*)b;
    if (x->cell != y->cell) return x->cell < y->cell ? -1 : 1;
    return (x->sp < y->sp) ? -1 : (x->sp > y->sp) ? 1 : 0;
}

typedef struct { int32_t x, y; } i2;

/* the edge test of gbts_make_graph_edges.ipp:31-99; returns 1 and the edge's
 * parameters when (n1 -> n2) passes */
static int edge_candidate(f4 np1, f4 np2, float phi1, float phi2, float deltaPhi,
                          const or_gbts_config* ap, float out[4]) {
    const float tau_min1 = np1.x, tau_max1 = np1.y, r1 = np1.z, z1 = np1.w;
    const float tau_min2 = np2.x, tau_max2 = np2.y, r2 = np2.z, z2 = np2.w;
    const float dr = r2 - r1;
    if (dr < ap->minDeltaRadius) return 0;
    const float dz = z2 - z1;
    const float tau = dz / dr;
    const float ftau = fabsf(tau);
    if ((ftau < tau_min2) || (ftau > tau_max2)) return 0;
    if ((ftau < tau_min1) || (ftau > tau_max1)) return 0;
    const float z0 = z1 - r1 * tau;
    if ((z0 < ap->min_z0) || (z0 > ap->max_z0)) return 0;
    const float zouter = z0 + ap->maxOuterRadius * tau;
    if (zouter < ap->cut_zMinU || zouter > ap->cut_zMaxU) return 0;
    const float dphi = wrap_phi(phi2 - phi1);
    if (fabsf(dphi) > deltaPhi) return 0;
    const float curv = dphi / dr;
    const float d0_for_max_curv = r1 * r2 * (fabsf(curv) - ap->max_Kappa);
    const float d0_max = (ftau < 4.0f) ? ap->low_Kappa_d0 : ap->high_Kappa_d0;
    if (d0_for_max_curv > d0_max) return 0;
    out[0] = sqrtf(1.0f + tau * tau) - tau;
    out[1] = curv;
    out[2] = phi2 + curv * r2;
    out[3] = phi1 + curv * r1;
    return 1;
}

typedef struct {
    uint32_t* data;
    size_t n, cap;
} u32vec;

static void push(u32vec* v, uint32_t x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 1024;
        v->data = (uint32_t*)realloc(v->data, v->cap * sizeof(uint32_t));
    }
    v->data[v->n++] = x;
}

/* one work item of gbts_make_graph_edges (gbts_make_graph_edges.ipp:104-239):
 * 128 threads, thread t taking the outer nodes t, t + 128, ... with its own
 * sliding-window start; edges in thread order, then outer node, then inner
 * node (the order the thread finds them in) */
static void make_edges_item(const or_gbts_config* c, const f4* np, const float* nphi,
                            uint32_t b1, uint32_t e1, uint32_t b2, uint32_t e2, float deltaPhi,
                            u32vec* en1, u32vec* en2, u32vec* ep) {
    const uint32_t n1 = e1 - b1, n2 = e2 - b2;
    const float phi0 = nphi[b1];
    const float phiN = nphi[b1 + n1 - 1u];
    const float phi_bin_width = TWO_PI_F / (float)c->n_phi_bins;
    const float break_threshold = deltaPhi + phi_bin_width - PI_F;
    for (uint32_t t = 0; t < EDGE_THREADS; ++t) {
        uint32_t last_n1 = 0u;
        for (uint32_t n2Idx = t; n2Idx < n2; n2Idx += EDGE_THREADS) {
            const uint32_t g2 = b2 + n2Idx;
            const float phi2 = nphi[g2];
            uint32_t n1Idx = last_n1;
            float min_phi1 = phi2 - deltaPhi;
            float max_phi1 = phi2 + deltaPhi;
            if (min_phi1 < -PI_F) min_phi1 += TWO_PI_F;
            if (max_phi1 > PI_F) max_phi1 -= TWO_PI_F;
            const int boundary = max_phi1 < min_phi1;
            max_phi1 += phi_bin_width;
            min_phi1 -= phi_bin_width;
            if (!boundary) {
                if (phi0 > max_phi1) continue;
                if (phiN < min_phi1) {
                    if (phi0 > break_threshold) break;
                    continue;
                }
            } else {
                if (phi0 < max_phi1) {
                    n1Idx = 0u;
                } else if (phiN < min_phi1) {
                    continue;
                }
            }
            const f4 np2 = np[g2];
            for (; n1Idx < n1; n1Idx++) {
                const float phi1 = nphi[b1 + n1Idx];
                if (!boundary) {
                    if (phi1 > max_phi1) break;
                    if (phi1 < min_phi1) continue;
                } else if (phi1 > max_phi1 && phi1 < min_phi1) {
                    continue;
                }
                last_n1 = n1Idx;
                float e[4];
                if (edge_candidate(np[b1 + n1Idx], np2, phi1, phi2, deltaPhi, c, e)) {
                    push(en1, b1 + n1Idx);
                    push(en2, g2);
                    for (int q = 0; q < 4; ++q) {
                        uint32_t bits;
                        memcpy(&bits, &e[q], 4);
                        push(ep, bits);
                    }
                }
            }
        }
    }
}

int or_gbts_run(const or_gbts_config* c, const or_gbts_tables* t, uint32_t n_sp,
                const float* xyz, const uint32_t* meas_idx, uint32_t n_meas,
                const uint64_t* surface_link, const float* diameter, or_gbts_seed* out,
                uint64_t cap, uint64_t* n_out, uint64_t* counters) {
    int rc = 0;
    memset(counters, 0, sizeof(uint64_t) * OR_GBTS_N_COUNTERS);
    *n_out = 0;
    const uint32_t nPhi = c->n_phi_bins;
    const uint32_t nEta = t->n_eta_bins;
    const uint32_t nMaxNei = c->max_num_neighbours;
    /* -- gbts_count_spacepoints_by_layer (gbts_count_spacepoints_by_layer.ipp:32-113) */
    f4* reduced = (f4*)malloc(sizeof(f4) * (n_sp ? n_sp : 1));
    int32_t* sp_layer = (int32_t*)malloc(sizeof(int32_t) * (n_sp ? n_sp : 1));
    for (uint32_t i = 0; i < n_sp; ++i) {
        sp_layer[i] = -1;
        reduced[i].x = xyz[3 * i];
        reduced[i].y = xyz[3 * i + 1];
        reduced[i].z = xyz[3 * i + 2];
        reduced[i].w = -CHAR_MAX - 1;
        const uint32_t m = meas_idx[i];
        if (m >= n_meas) {
            rc = 2;
            continue;
        }
        const uint64_t link = surface_link[m];
        const uint32_t volume = (uint32_t)field(link, c->volume_shift, c->volume_bits);
        const int16_t begin_or_bin = (volume < t->n_volumes) ? t->volume_map[volume] : SHRT_MAX;
        if (begin_or_bin == SHRT_MAX) continue;
        uint32_t layerIdx = 0u;
        if (begin_or_bin < 0) {
            const uint32_t surface_index = (uint32_t)field(link, c->index_shift, c->index_bits);
            for (uint32_t s = (uint32_t)(-1 * (begin_or_bin + 1)); s < t->n_surfaces; s++) {
                if (t->surface_map[2 * s] == surface_index) {
                    layerIdx = t->surface_map[2 * s + 1];
                    break;
                }
            }
        } else {
            layerIdx = (uint32_t)begin_or_bin;
        }
        if (layerIdx >= t->n_layers) continue; /* malformed tables */
        float cluster_diameter = diameter[m];
        const int type = (int)t->layer_type[layerIdx];
        if (type == 1 && cluster_diameter > c->type1_max_width) continue;
        cluster_diameter = (c->doTauCut && type != 0) ? (float)(-1 * type) : cluster_diameter;
        sp_layer[i] = (int32_t)layerIdx;
        reduced[i].w = cluster_diameter;
    }
    /* -- gbts_bin_spacepoints (gbts_bin_spacepoints.ipp:27-107): eta bin, phi bin */
    node_key* keys = (node_key*)malloc(sizeof(node_key) * (n_sp ? n_sp : 1));
    uint32_t nNodes = 0;
    const float inv_phiSliceWidth = 1.0f / (TWO_PI_F / (float)nPhi);
    for (uint32_t i = 0; i < n_sp; ++i) {
        if (sp_layer[i] < 0) continue;
        const f4 sp = reduced[i];
        const uint32_t L = (uint32_t)sp_layer[i];
        const uint32_t bin0 = t->eta_bin0[L];
        const uint32_t num_eta_bins = t->n_eta[L];
        uint32_t eta_index;
        if (num_eta_bins == 1u) {
            eta_index = bin0;
        } else {
            const float r = sqrtf(sp.x * sp.x + sp.y * sp.y);
            const float t1 = sp.z / r;
            const float eta = -cr_logf(sqrtf(1.0f + t1 * t1) - t1);
            const uint32_t binIdx = (uint32_t)smax(
                0.0f, smin((eta - t->min_eta[L]) / t->eta_width[L], (float)(num_eta_bins - 1u)));
            eta_index = bin0 + binIdx;
        }
        const float Phi = cr_atan2f(sp.y, sp.x);
        uint32_t phiIdx = (uint32_t)((Phi + PI_F) * inv_phiSliceWidth);
        if (phiIdx >= nPhi) phiIdx -= nPhi;
        keys[nNodes].sp = i;
        keys[nNodes].cell = phiIdx + nPhi * eta_index;
        ++nNodes;
    }
    counters[OR_GBTS_NODES] = nNodes;
    /* -- gbts_sort_nodes (gbts_sort_nodes.ipp:24-101): nodes by (eta, phi)
     * cell, ascending spacepoint index inside a cell */
    qsort(keys, nNodes, sizeof(node_key), node_cmp);
    f4* np = (f4*)malloc(sizeof(f4) * (nNodes ? nNodes : 1));
    float* nphi = (float*)malloc(sizeof(float) * (nNodes ? nNodes : 1));
    uint32_t* nidx = (uint32_t*)malloc(sizeof(uint32_t) * (nNodes ? nNodes : 1));
    for (uint32_t k = 0; k < nNodes; ++k) {
        const f4 sp = reduced[keys[k].sp];
        const float Phi = cr_atan2f(sp.y, sp.x);
        const float r = sqrtf(sp.x * sp.x + sp.y * sp.y);
        float min_tau = 0.0f;
        float max_tau = c->maxTau;
        if (sp.w > 0) {
            if (c->useTauLUT) {
                const int tau_bin = 5 * (int)(floorf(c->tau_lut_inv_bin * sp.w) - 1.0f);
                if (tau_bin > -1 && tau_bin < (int)c->tauLutSize) {
                    min_tau = t->tau_lut[(uint32_t)tau_bin + 1u];
                    max_tau = t->tau_lut[(uint32_t)tau_bin + 2u];
                }
                if (max_tau < 0.0f) max_tau = c->maxTau;
                if (min_tau < 0.0f) min_tau = 0.0f;
            } else {
                min_tau = c->tMin_slope * (sp.w - c->offset);
                max_tau = c->tMax_min + c->tMax_correction / (sp.w + c->offset) +
                          c->tMax_slope * (sp.w - c->offset);
            }
        }
        np[k].x = min_tau;
        np[k].y = max_tau;
        np[k].z = r;
        np[k].w = sp.z;
        nphi[k] = Phi;
        nidx[k] = keys[k].sp;
    }
    /* eta bin views and gbts_find_minmax_radius (gbts_find_minmax_radius.ipp:21-54) */
    uint32_t* view = (uint32_t*)calloc(2 * (size_t)(nEta ? nEta : 1), sizeof(uint32_t));
    float* bin_rads = (float*)malloc(sizeof(float) * 2 * (nEta ? nEta : 1));
    {
        uint32_t k = 0;
        for (uint32_t e = 0; e < nEta; ++e) {
            view[2 * e] = k;
            while (k < nNodes && keys[k].cell / nPhi == e) ++k;
            view[2 * e + 1] = k;
            float min_r = 1e8f, max_r = -1e8f;
            for (uint32_t j = view[2 * e]; j < k; ++j) {
                max_r = fmaxf(np[j].z, max_r);
                min_r = fminf(np[j].z, min_r);
            }
            bin_rads[2 * e] = min_r;
            bin_rads[2 * e + 1] = max_r;
        }
    }
    /* -- work items (gbts_seeding_algorithm.cpp:215-283) and
     * gbts_make_graph_edges */
    u32vec en1 = {0}, en2 = {0}, ep = {0};
    for (uint32_t p = 0; p < t->n_pairs; ++p) {
        const uint32_t bin1 = t->pairs[2 * p], bin2 = t->pairs[2 * p + 1];
        if (bin1 >= nEta || bin2 >= nEta) continue;
        const float rb1 = bin_rads[2 * bin1];
        const uint32_t begin_bin1 = view[2 * bin1], end_bin1 = view[2 * bin1 + 1];
        if (begin_bin1 == end_bin1) continue;
        if (view[2 * bin2] == view[2 * bin2 + 1]) continue;
        const float rb2 = bin_rads[2 * bin2 + 1];
        const float maxDeltaR = fabsf(rb2 - rb1);
        float deltaPhi = c->min_delta_phi + c->dphi_coeff * maxDeltaR;
        if (maxDeltaR < c->low_dr_threshold)
            deltaPhi = c->min_delta_phi_low_dr + c->dphi_coeff_low_dr * maxDeltaR;
        for (uint32_t b = begin_bin1; b < end_bin1; b += NODE_BUFFER) {
            const uint32_t e = (end_bin1 - b > NODE_BUFFER) ? b + NODE_BUFFER : end_bin1;
            make_edges_item(c, np, nphi, b, e, view[2 * bin2], view[2 * bin2 + 1], deltaPhi, &en1,
                            &en2, &ep);
        }
    }
    const uint64_t nMaxEdges = (uint64_t)c->max_edges_factor * nNodes;
    counters[OR_GBTS_EDGES] = en1.n;
    const uint32_t nEdges = (uint32_t)(en1.n < nMaxEdges ? en1.n : nMaxEdges);
    /* -- gbts_link_graph_edges: the edges leaving each node (by inner node) */
    uint32_t* lstart = (uint32_t*)calloc((size_t)nNodes + 1, sizeof(uint32_t));
    for (uint32_t e = 0; e < nEdges; ++e) lstart[en1.data[e] + 1]++;
    for (uint32_t k = 0; k < nNodes; ++k) lstart[k + 1] += lstart[k];
    uint32_t* links = (uint32_t*)malloc(sizeof(uint32_t) * (nEdges ? nEdges : 1));
    {
        uint32_t* cur = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)nNodes + 1));
        memcpy(cur, lstart, sizeof(uint32_t) * ((size_t)nNodes + 1));
        for (uint32_t e = 0; e < nEdges; ++e) links[cur[en1.data[e]]++] = e;
        free(cur);
    }
    /* -- gbts_match_graph_edges (gbts_match_graph_edges.ipp:29-118) */
    uint8_t* nnei = (uint8_t*)calloc(nEdges ? nEdges : 1, 1);
    uint32_t* nei = (uint32_t*)calloc((size_t)nMaxNei * (nEdges ? nEdges : 1), sizeof(uint32_t));
    uint8_t* kept = (uint8_t*)calloc(nEdges ? nEdges : 1, 1);
    uint64_t nConnections = 0;
    for (uint32_t e = 0; e < nEdges; ++e) {
        const uint32_t sharedNode = en2.data[e];
        const uint32_t link_begin = lstart[sharedNode];
        const uint32_t nLinks = lstart[sharedNode + 1] - link_begin;
        if (nLinks == 0u) continue;
        const float* p1 = (const float*)&ep.data[4 * (size_t)e];
        const float uat_2 = 1.0f / p1[0];
        const float Phi2 = p1[2];
        const float curv2 = p1[1];
        unsigned num_nei = 0;
        for (uint32_t k = 0; k < nLinks; k++) {
            if (num_nei >= nMaxNei) break;
            const uint32_t e2 = links[link_begin + k];
            const float* p2 = (const float*)&ep.data[4 * (size_t)e2];
            const float tau_ratio = p2[0] * uat_2 - 1.0f;
            if (fabsf(tau_ratio) > c->cut_tau_ratio_max) continue;
            const float dPhi = wrap_phi(Phi2 - p2[3]);
            if (fabsf(dPhi) > c->cut_dphi_max) continue;
            const float dcurv = curv2 - p2[1];
            if (fabsf(dcurv) > c->cut_dcurv_max) continue;
            nei[(size_t)nMaxNei * e + num_nei] = e2;
            kept[e2] = 1;
            ++num_nei;
        }
        nnei[e] = (uint8_t)num_nei;
        if (num_nei != 0) {
            kept[e] = 1;
            nConnections += num_nei;
        }
    }
    counters[OR_GBTS_CONNECTIONS] = nConnections;
    /* -- gbts_reindex_edges, gbts_compress_graph */
    int32_t* reidx = (int32_t*)malloc(sizeof(int32_t) * (nEdges ? nEdges : 1));
    uint32_t nC = 0;
    for (uint32_t e = 0; e < nEdges; ++e) reidx[e] = kept[e] ? (int32_t)nC++ : -1;
    counters[OR_GBTS_CONNECTED_EDGES] = nC;
    const uint32_t esz = 3u + nMaxNei;
    uint32_t* graph = (uint32_t*)calloc((size_t)esz * (nC ? nC : 1), sizeof(uint32_t));
    for (uint32_t e = 0; e < nEdges; ++e) {
        if (reidx[e] < 0) continue;
        uint32_t* row = graph + (size_t)esz * (uint32_t)reidx[e];
        row[0] = nidx[en2.data[e]];
        row[1] = nidx[en1.data[e]];
        row[2] = nnei[e];
        for (uint32_t k = 0; k < nnei[e]; ++k)
            row[3 + k] = (uint32_t)reidx[nei[(size_t)nMaxNei * e + k]];
    }
    /* -- gbts_run_cca_iteration x 15 (gbts_run_cca_iteration.ipp:23-101) */
    uint8_t* levels = (uint8_t*)malloc(2 * (size_t)(nC ? nC : 1));
    memset(levels, 1, 2 * (size_t)(nC ? nC : 1));
    int8_t* active = (int8_t*)calloc(nC ? nC : 1, 1);
    int32_t* opx = (int32_t*)calloc(nC ? nC : 1, sizeof(int32_t));
    int16_t* opy = (int16_t*)calloc(nC ? nC : 1, sizeof(int16_t));
    for (uint32_t iter = 0; iter < MAX_CCA_ITER; ++iter) {
        const uint32_t toggle = iter % 2;
        const uint8_t* lload = levels + (size_t)toggle * nC;
        uint8_t* lstore = levels + (size_t)(1 - toggle) * nC;
        for (uint32_t e = 0; e < nC; ++e) {
            if (iter != 0 && active[e] != (int8_t)iter) continue;
            const uint32_t* row = graph + (size_t)esz * e;
            const uint32_t nN = row[2];
            uint8_t next_level = lload[e];
            int localChange = 0;
            for (uint32_t k = 0; k < nN; k++) {
                const uint8_t forward_level = lload[row[3 + k]];
                if (next_level == forward_level) {
                    next_level = (uint8_t)(forward_level + 1);
                    localChange = 1;
                    break;
                }
            }
            if (localChange) {
                if (iter == MAX_CCA_ITER - 1) {
                    opy[e] = -1;
                    active[e] = -1;
                } else {
                    active[e] = (int8_t)(iter + 1u);
                }
            } else {
                active[e] = -1;
                int32_t out_paths = 0;
                for (uint32_t k = 0; k < nN; ++k) {
                    const uint32_t n = row[3 + k];
                    if (next_level == 1 + levels[n]) out_paths += 1 + opx[n];
                    opy[n] = -1;
                }
                opx[e] = out_paths;
                opy[e] = (int16_t)((next_level >= c->minLevel) - 1);
            }
            lstore[e] = next_level;
        }
    }
    /* -- gbts_count_terminus_edges, gbts_add_terminus_to_path_store */
    uint32_t nT = 0;
    uint64_t nPaths = 0;
    for (uint32_t e = 0; e < nC; ++e)
        if (opy[e] != -1) {
            ++nT;
            nPaths += (uint64_t)opx[e];
        }
    counters[OR_GBTS_TERMINUS] = nT;
    counters[OR_GBTS_PATHS] = nPaths;
    const uint64_t nStore = nT + nPaths;
    i2* store = (i2*)malloc(sizeof(i2) * (nStore ? nStore : 1));
    {
        uint32_t k = 0;
        for (uint32_t e = 0; e < nC; ++e)
            if (opy[e] != -1) {
                store[k].x = (int32_t)e;
                store[k].y = -1;
                ++k;
            }
    }
    /* -- gbts_fill_path_store: depth-first pre-order below each terminus edge;
     * the children of an entry are its neighbours one level down, in
     * neighbour order */
    {
        uint64_t pos = nT;
        uint32_t stk_e[MAX_CCA_ITER + 2], stk_k[MAX_CCA_ITER + 2];
        int64_t stk_i[MAX_CCA_ITER + 2];
        for (uint32_t ti = 0; ti < nT; ++ti) {
            int d = 0;
            stk_e[0] = (uint32_t)store[ti].x;
            stk_i[0] = ti;
            stk_k[0] = 0;
            while (d >= 0) {
                const uint32_t e = stk_e[d];
                const uint32_t* row = graph + (size_t)esz * e;
                if (stk_k[d] >= row[2]) {
                    --d;
                    continue;
                }
                const uint32_t n = row[3 + stk_k[d]++];
                if (levels[e] != levels[n] + 1) continue;
                if (pos >= nStore) break;
                store[pos].x = (int32_t)n;
                store[pos].y = (int32_t)stk_i[d];
                ++d;
                stk_e[d] = n;
                stk_i[d] = (int64_t)pos;
                stk_k[d] = 0;
                ++pos;
            }
        }
    }
    /* -- gbts_fit_segments (gbts_fit_segments.ipp:256-335) */
    i2* props = (i2*)malloc(sizeof(i2) * (nPaths ? nPaths : 1));
    uint32_t nProps = 0;
    for (uint64_t path_idx = nT; path_idx < nStore; ++path_idx) {
        unsigned length = 1;
        int toggle = 0;
        edge_state s1, s2;
        memset(&s1, 0, sizeof(s1));
        memset(&s2, 0, sizeof(s2));
        i2 path = store[path_idx];
        const uint32_t* row = graph + (size_t)esz * (uint32_t)path.x;
        const f4 node1 = reduced[row[0]];
        const f4 node2 = reduced[row[1]];
        state_init(&s1, node2, node1);
        while (path.y >= 0) {
            path = store[path.y];
            const f4 nd = reduced[graph[(size_t)esz * (uint32_t)path.x + 1]];
            if (toggle) {
                if (!kalman_update(&s1, &s2, nd, c, c->max_z0)) {
                    s1 = s2;
                    break;
                }
            } else if (!kalman_update(&s2, &s1, nd, c, c->max_z0)) {
                break;
            }
            toggle = !toggle;
            length++;
        }
        if (length < c->minLevel) continue;
        const int qual = toggle ? (int)(c->qual_scale * s2.J) : (int)(c->qual_scale * s1.J);
        props[nProps].x = qual;
        props[nProps].y = (int32_t)path_idx;
        ++nProps;
    }
    counters[OR_GBTS_PROPS] = nProps;
    /* -- bidding: gbts_create_seed_candidate (gbts_create_seed_candidate.ipp:
     * 22-58), gbts_rebid_seeds_for_edges, gbts_reset_edge_bids */
    int8_t* ambi = (int8_t*)calloc(nProps ? nProps : 1, 1);
    uint64_t* ebid = (uint64_t*)calloc(nC ? nC : 1, sizeof(uint64_t));
    uint64_t nRejected = 0;
#define BID(P) ((((uint64_t)(uint32_t)props[P].x) << 32) | (uint64_t)(P))
#define CANDIDATE(P, DEPTH)                                                  \
    do {                                                                     \
        ambi[P] = 0;                                                         \
        const uint64_t seed_bid = BID(P);                                    \
        i2 pth = {0, props[P].y};                                            \
        int depth = (DEPTH);                                                 \
        while (pth.y >= 0 && depth != 0) {                                   \
            pth = store[pth.y];                                              \
            depth--;                                                         \
            const uint64_t comp = ebid[pth.x];                               \
            if (seed_bid > comp) ebid[pth.x] = seed_bid;                     \
            if (comp > seed_bid) {                                           \
                ambi[P] = -1;                                                \
            } else if (comp != 0) {                                          \
                ambi[comp & 0xFFFFFFFFull] = -1;                             \
            }                                                                \
        }                                                                    \
    } while (0)
    for (uint32_t P = 0; P < nProps; ++P) CANDIDATE(P, 1);
    for (uint32_t round = 0; round < c->edge_bidding_rounds; ++round) {
        memset(ebid, 0, sizeof(uint64_t) * (nC ? nC : 1));
        const int first = round == 0u;
        for (uint32_t P = 0; P < nProps; ++P) {
            const int8_t a = ambi[P];
            if (first) {
                if (a == 0) {
                    ambi[P] = 1;
                } else {
                    ambi[P] = -2;
                    ++nRejected;
                    continue;
                }
            } else if ((a == -2) | (a == 0)) {
                continue;
            }
            CANDIDATE(P, -1);
        }
        for (uint32_t P = 0; P < nProps; ++P) {
            const int8_t a = ambi[P];
            if ((a == -2) | (a == 0)) continue;
            int isgood = 1;
            i2 pth = {0, props[P].y};
            while (pth.y >= 0) {
                pth = store[pth.y];
                const uint64_t best = ebid[pth.x];
                if (ambi[best & 0xFFFFFFFFull] == 0) {
                    isgood = 0;
                    break;
                }
            }
            if (isgood) {
                ambi[P] = 1;
            } else {
                ambi[P] = -2;
                ++nRejected;
            }
        }
    }
#undef CANDIDATE
    counters[OR_GBTS_REJECTED] = nRejected;
    /* -- gbts_bid_seeds_for_hits (gbts_bid_seeds_for_hits.ipp:23-70) */
    uint64_t* hbid = (uint64_t*)calloc(n_sp ? n_sp : 1, sizeof(uint64_t));
    for (uint32_t P = 0; P < nProps; ++P) {
        if (ambi[P] == -2) continue;
        const uint64_t b = BID(P);
        i2 pth = {0, props[P].y};
        while (pth.y >= 0) {
            pth = store[pth.y];
            const uint32_t sp = graph[(size_t)esz * (uint32_t)pth.x];
            if (b > hbid[sp]) hbid[sp] = b;
        }
        const uint32_t sp = graph[(size_t)esz * (uint32_t)pth.x + 1];
        if (b > hbid[sp]) hbid[sp] = b;
    }
#undef BID
    /* -- gbts_convert_seeds (gbts_convert_seeds.ipp:72-194) */
    uint64_t nOut = 0;
    for (uint32_t P = 0; P < nProps; ++P) {
        if (ambi[P] == -2) continue;
        signed char best_for_hit = 0;
        uint32_t nodes[MAX_CCA_ITER + 1];
        int size = 0;
        i2 pth = {0, props[P].y};
        while (pth.y >= 0) {
            pth = store[pth.y];
            nodes[size++] = graph[(size_t)esz * (uint32_t)pth.x];
            best_for_hit = (signed char)(best_for_hit + (P == (hbid[nodes[size - 1]] & 0xFFFFFFFFull)));
        }
        nodes[size++] = graph[(size_t)esz * (uint32_t)pth.x + 1];
        best_for_hit = (signed char)(best_for_hit + (P == (hbid[nodes[size - 1]] & 0xFFFFFFFFull)));
        if (best_for_hit < c->best_hit_frac * (float)size) continue;
        int diff_code = 0;
        int force_dropout = 0;
        if (c->use_dropout) {
            f4 sps[3] = {reduced[nodes[size - 1]], reduced[nodes[(size - 1) / 2 + 1]],
                         reduced[nodes[0]]};
            float c1x, c1y, c2x, c2y, c3x, c3y;
            estimate_seed_params(sps, &c1x, &c1y);
            sps[1] = reduced[nodes[(size - 1) / 2]];
            estimate_seed_params(sps, &c2x, &c2y);
            sps[0] = reduced[nodes[size - 2]];
            estimate_seed_params(sps, &c3x, &c3y);
            if ((best_for_hit < size - 1) &
                (fabsf(c1y + c2y + c3y) < 3.0f * c->tight_bid_cot_threshold) & (size < 5))
                continue;
            const float d0 = fabsf(c1x - c2x), d1 = fabsf(c2x - c3x), d2 = fabsf(c1x - c3x);
            diff_code = 4 * (d0 < c->dropout_dcurv_m) + 2 * (d1 < c->dropout_dcurv_m) +
                        (d2 < c->dropout_dcurv_m);
            force_dropout = fabsf(c1x + c2x + c3x) < 3.0f * c->force_dropout_max_curv_m;
            force_dropout |=
                (fabsf(c1y + c2y + c3y) < 3.0f * c->tight_bid_cot_threshold) & (diff_code == 0);
        }
        const float quality = (float)props[P].x;
        uint32_t emit[3][3];
        int ne = 0;
        if (((diff_code != 3) & (diff_code != 6)) | force_dropout) {
            emit[ne][0] = nodes[size - 1];
            emit[ne][1] = nodes[(size - 1) / 2 + 1];
            emit[ne][2] = nodes[0];
            ++ne;
        }
        if ((diff_code == 1) | (diff_code == 6)) {
            emit[ne][0] = nodes[size - 1];
            emit[ne][1] = nodes[(size - 1) / 2];
            emit[ne][2] = nodes[0];
            ++ne;
        }
        if ((diff_code == 2) | (diff_code == 3) | (diff_code == 4) | force_dropout) {
            emit[ne][0] = nodes[size - 2];
            emit[ne][1] = nodes[(size - 1) / 2];
            emit[ne][2] = nodes[0];
            ++ne;
        }
        for (int k = 0; k < ne; ++k) {
            if (nOut < cap) {
                out[nOut].bottom = emit[k][0];
                out[nOut].middle = emit[k][1];
                out[nOut].top = emit[k][2];
                out[nOut].quality = quality;
            }
            ++nOut;
        }
    }
    counters[OR_GBTS_SEEDS] = nOut;
    *n_out = nOut;
    if (nOut > cap && rc == 0) rc = 1;
    free(reduced); free(sp_layer); free(keys); free(np); free(nphi); free(nidx); free(view);
    free(bin_rads); free(en1.data); free(en2.data); free(ep.data); free(lstart); free(links);
    free(nnei); free(nei); free(kept); free(reidx); free(graph); free(levels); free(active);
    free(opx); free(opy); free(store); free(props); free(ambi); free(ebid); free(hbid);
    return rc;
}
