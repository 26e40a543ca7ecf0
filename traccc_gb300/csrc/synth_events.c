/*
 * synth_events.c -- seeded synthetic helix events for the seeding path.
 *
 * The reference measures seeding on ODD ttbar / traccc data files that are
 * not available here; these events stand in for them with the detector,
 * field, smearing and track distributions of the benchmark configurations:
 *
 *   barrel of 10 cylinders r = 32,72,116,172,260,360,500,600,700,820 mm,
 *   |z| <= 1000 mm, uniform field B along z; helices from a vertex offset by
 *   d0 ~ N(0, sigma_d0) (transverse) and z0 ~ N(0, sigma_z0); one spacepoint
 *   per first crossing of each layer, smeared in r*phi and z; uniform noise
 *   spacepoints on random layers.  Spacepoints are shuffled (the seeding
 *   result depends on the input order only through exact ties).
 *
 * One measurement per spacepoint: local = (r*phi, z), surface_link = the
 * layer number + 1.  Double-precision arithmetic with a project-owned
 * xoshiro256** generator, so an event is a pure function of its config.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct {
    uint32_t n_tracks;
    int32_t pt_dist;    /* 0 uniform(a,b), 1 log-uniform(a,b), 2 exp(mean a) >= b */
    double pt_a, pt_b;  /* GeV */
    double eta_max;
    double noise_frac;  /* noise spacepoints per track spacepoint */
    double z0_sigma, d0_sigma;      /* mm */
    double smear_rphi, smear_z;     /* mm */
    double bz_tesla;
    uint64_t seed;
} synth_config;

typedef struct {
    float* global;             /* 3 per spacepoint, xyz interleaved */
    uint32_t* measurement_index_1;
    uint32_t* measurement_index_2;
    float* z_variance;
    float* radius_variance;
    uint32_t* layer;           /* 0..9 */
    int32_t* particle;         /* track number, -1 for noise */
    float* local_position;     /* 2 per measurement */
    uint64_t* surface_link;
    uint32_t capacity;
} synth_output;

static const double k_layers[10] = {32., 72., 116., 172., 260.,
                                    360., 500., 600., 700., 820.};

typedef struct {
    uint64_t s[4];
} rng_t;

static uint64_t splitmix(uint64_t* x) {
    uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static void rng_seed(rng_t* r, uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) r->s[i] = splitmix(&x);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t rng_next(rng_t* r) {
    uint64_t* s = r->s;
    uint64_t res = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return res;
}
/* uniform in [0, 1) */
static double rng_u(rng_t* r) { return (double)(rng_next(r) >> 11) * 0x1.0p-53; }
static double rng_normal(rng_t* r) {
    double u1 = rng_u(r), u2 = rng_u(r);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

static double draw_pt(const synth_config* c, rng_t* r) {
    switch (c->pt_dist) {
        case 0: return c->pt_a + (c->pt_b - c->pt_a) * rng_u(r);
        case 1: return exp(log(c->pt_a) + (log(c->pt_b) - log(c->pt_a)) * rng_u(r));
        default: {
            /* exponential of mean pt_a, truncated below at pt_b: memoryless,
             * so shift the exponential to start at the cut */
            double u = rng_u(r);
            return c->pt_b - c->pt_a * log(1.0 - u);
        }
    }
}

static void emit(const synth_config* c, synth_output* o, uint32_t* n,
                 double x, double y, double z, uint32_t layer, int32_t particle) {
    (void)c;
    if (*n >= o->capacity) { (*n)++; return; }
    uint32_t i = *n;
    o->global[3 * i] = (float)x;
    o->global[3 * i + 1] = (float)y;
    o->global[3 * i + 2] = (float)z;
    o->layer[i] = layer;
    o->particle[i] = particle;
    (*n)++;
}

/* Returns the number of spacepoints; if it exceeds capacity, nothing past
 * capacity was written and the caller retries with a larger buffer. */
uint32_t synth_event(const synth_config* c, synth_output* o) {
    rng_t r;
    rng_seed(&r, c->seed * 0x2545F4914F6CDD1DULL + 12345u);
    uint32_t n = 0;
    const double kappa = 0.299792458e-3 * c->bz_tesla; /* GeV per mm of radius */
    for (uint32_t t = 0; t < c->n_tracks; ++t) {
        double q = (rng_u(&r) < 0.5) ? -1.0 : 1.0;
        double pt = draw_pt(c, &r);
        double eta = (2.0 * rng_u(&r) - 1.0) * c->eta_max;
        double phi0 = (2.0 * rng_u(&r) - 1.0) * M_PI;
        double z0 = rng_normal(&r) * c->z0_sigma;
        double d0 = rng_normal(&r) * c->d0_sigma;
        double cot = sinh(eta);
        double R = pt / kappa;
        double h = -q; /* +1: counter-clockwise in the xy plane */
        double nx = -sin(phi0), ny = cos(phi0);
        double px = d0 * nx, py = d0 * ny;
        double cx = px + h * R * nx, cy = py + h * R * ny;
        double D = sqrt(cx * cx + cy * cy);
        double gam = atan2(cy, cx);
        double beta0 = atan2(py - cy, px - cx);
        for (uint32_t l = 0; l < 10; ++l) {
            double rl = k_layers[l];
            double K = (rl * rl - D * D - R * R) / (2.0 * R);
            if (D <= 0.0 || fabs(K / D) > 1.0) break;
            double dacos = acos(K / D);
            double best = 1e30;
            for (int s = -1; s <= 1; s += 2) {
                double beta = gam + s * dacos;
                double a = h * (beta - beta0);
                a = fmod(a, 2.0 * M_PI);
                if (a < 0) a += 2.0 * M_PI;
                if (a < best) best = a;
            }
            if (best > M_PI) break;
            double beta = beta0 + h * best;
            double x = cx + R * cos(beta), y = cy + R * sin(beta);
            double z = z0 + R * best * cot;
            if (fabs(z) > 1000.0) continue;
            /* smear along the layer in r*phi and in z */
            double dphi = rng_normal(&r) * c->smear_rphi / rl;
            double ph = atan2(y, x) + dphi;
            z += rng_normal(&r) * c->smear_z;
            emit(c, o, &n, rl * cos(ph), rl * sin(ph), z, l, (int32_t)t);
        }
    }
    uint32_t n_track_sp = n;
    uint32_t n_noise = (uint32_t)llround(c->noise_frac * (double)n_track_sp);
    for (uint32_t k = 0; k < n_noise; ++k) {
        uint32_t l = (uint32_t)(rng_u(&r) * 10.0);
        if (l > 9) l = 9;
        double ph = (2.0 * rng_u(&r) - 1.0) * M_PI;
        double z = (2.0 * rng_u(&r) - 1.0) * 1000.0;
        emit(c, o, &n, k_layers[l] * cos(ph), k_layers[l] * sin(ph), z, l, -1);
    }
    if (n > o->capacity) return n;
    /* Fisher-Yates shuffle of the spacepoints */
    for (uint32_t i = n; i > 1; --i) {
        uint32_t j = (uint32_t)(rng_u(&r) * (double)i);
        if (j >= i) j = i - 1;
        uint32_t a = i - 1;
        float g[3];
        memcpy(g, &o->global[3 * a], sizeof g);
        memcpy(&o->global[3 * a], &o->global[3 * j], sizeof g);
        memcpy(&o->global[3 * j], g, sizeof g);
        uint32_t lt = o->layer[a]; o->layer[a] = o->layer[j]; o->layer[j] = lt;
        int32_t pt = o->particle[a]; o->particle[a] = o->particle[j]; o->particle[j] = pt;
    }
    for (uint32_t i = 0; i < n; ++i) {
        double x = o->global[3 * i], y = o->global[3 * i + 1];
        double rr = sqrt(x * x + y * y);
        o->measurement_index_1[i] = i;
        o->measurement_index_2[i] = 0xFFFFFFFFu;
        o->z_variance[i] = 0.f;
        o->radius_variance[i] = 0.f;
        o->local_position[2 * i] = (float)(rr * atan2(y, x));
        o->local_position[2 * i + 1] = o->global[3 * i + 2];
        o->surface_link[i] = (uint64_t)o->layer[i] + 1u;
    }
    return n;
}
