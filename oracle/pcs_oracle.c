/*
 * pcs_oracle.c -- CPU restatement of the reference's ABC-PMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see pcs_oracle.h).  Build with
 * -ffp-contract=off: each float expression below is evaluated as the listed
 * sequence of IEEE round-to-nearest operations.
 */
#include "pcs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Philox4x32-10                                                       */
/* ------------------------------------------------------------------ */

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += PHILOX_W0;
        k1 += PHILOX_W1;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

void orc_replay_draws(uint64_t seed, uint64_t n_particles, uint32_t stride, float* uniforms,
                      float* normals, float* sigmas, float base_sigma)
{
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const double s24 = 1.0 / 16777216.0;
    for (uint64_t n = 0; n < n_particles; ++n) {
        uint32_t ctr[4] = {(uint32_t)n, 0u, (uint32_t)(n >> 32), 0xA5A5A5A5u}, r[4];
        orc_philox4x32_10(ctr, key, r);
        for (int i = 0; i < 4; ++i) uniforms[4 * n + i] = (float)((double)(r[i] >> 8) * s24);
        if (sigmas) {
            ctr[1] = 0xFFFFFFFFu;
            orc_philox4x32_10(ctr, key, r);
            float u = (float)((double)(r[0] >> 8) * s24);
            sigmas[n] = base_sigma * (0.5f + u);
        }
        for (uint32_t s = 0; s < stride; ++s)
            for (uint32_t a = 0; a < 3; ++a) {
                ctr[1] = 1u + 3u * s + a;
                orc_philox4x32_10(ctr, key, r);
                double sum = 0.0;
                for (int i = 0; i < 4; ++i) sum += (double)(r[i] >> 8) * s24;
                normals[(n * stride + s) * 3 + a] = (float)((sum - 2.0) * 1.7320508075688772);
            }
    }
}

/* ------------------------------------------------------------------ */
/* Forward model, GPU conventions                                      */
/* ------------------------------------------------------------------ */

/* periodic_bounds_ (kernel-simulate.inl:95-103): one wrap. */
static float periodic_bounds(float v, float m)
{
    if (fabsf(v) > m) {
        float two_m = 2.0f * copysignf(m, v);
        v = v - two_m;
    }
    return v;
}

/* float -> uint32 as the GPU converts it (cvt.rzi.u32.f32: NaN -> 0,
 * saturating), which is the reference recorder's tCount(aDE / mDDE). */
static uint32_t f32_to_u32_rz_sat(float x)
{
    if (x != x) return 0u;
    if (x <= 0.0f) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}

/* HistogramRecorder::record (histogram2d.inl:313-321). */
static void record(const orc_setup* s, uint32_t* hist, uint32_t k, float de,
                   orc_track_counts* counts)
{
    /* de / ((detectionCount-1) * fourDeltaT): the count is unsigned, so k-1
     * wraps for k == 0 and converts to float before the multiply. */
    float km1 = (float)(uint32_t)(k - 1u);
    float denom = km1 * s->four_delta_t;
    float DE = de / denom;
    float q = DE / s->dde;
    uint32_t bin = f32_to_u32_rz_sat(q);
    counts->closed++;
    if (bin < s->de_bins) {
        uint64_t idx = (uint64_t)k * s->de_bins + bin;
        if (idx < (uint64_t)s->rows * s->de_bins) {
            hist[idx] += 1u;
        }
        counts->recorded++;
    }
}

/* wrand_index (utility.inl:8-57).  C == 2 compares with >=, C > 2 searches
 * for the first cumulative probability greater than the draw. */
static uint32_t wrand_index(float value, uint32_t C, const float* pre)
{
    if (C == 2) return (pre[0] >= value) ? 0u : 1u;
    uint32_t bot = 0, top = C;
    while (bot != top) {
        uint32_t mid = (top + bot) / 2;
        if (pre[mid] <= value)
            bot = mid + 1;
        else
            top = mid;
    }
    return bot;
}

/* detected (utility.inl:102-153). */
static int detected(float x, float y, float z, float half_az, const orc_setup* s)
{
    return fabsf(z) <= half_az && fabsf(x) <= s->half_ax && fabsf(y) <= s->half_ay;
}

int orc_simulate_replay(const orc_setup* s, const orc_run* r, const orc_replay* rp,
                        uint32_t* hist, orc_track_counts* counts)
{
    orc_track_counts local = {0, 0};
    if (!counts) counts = &local;
    if (s->component_count < 1 || s->component_count > ORC_MAX_COMPONENTS) return -1;
    uint64_t n = 0;
    for (uint32_t v = 0; v < s->video_count; ++v) {
        uint32_t frames = r->frames[v];
        if (frames >= 1 && frames - 1 > rp->normal_stride) return -2;
        for (uint32_t p = 0; p < r->particles[v]; ++p, ++n) {
            const float* u = rp->uniforms + 4 * n;
            /* make_particle (utility.inl:60-99) */
            float x = s->half_lx * (2.0f * u[0] - 1.0f);
            float y = s->half_ly * (2.0f * u[1] - 1.0f);
            float z = s->half_lz * (2.0f * u[2] - 1.0f);
            uint32_t idx = 0;
            if (s->component_count > 1) idx = wrand_index(u[3], s->component_count, r->pre_comp_prob);
            if (idx >= s->component_count) return -3; /* pre_comp_prob must end above 1 */

            /* one depth for the fixed-depth and lognormal models, one per component otherwise */
            float half_az = (s->model == ORC_MODEL_DISCRETE_VARIABLE_Z) ? r->half_az[idx] : r->half_az[0];
            float rwsd;
            if (s->model == ORC_MODEL_LOGNORMAL) {
                if (!rp->sigmas) return -4;
                rwsd = rp->sigmas[n];
            } else {
                rwsd = r->rand_walk_stddev[idx];
            }

            float de = 0.0f;
            uint32_t k = detected(x, y, z, half_az, s) ? 1u : 0u;
            const float* nrm = rp->normals + (uint64_t)n * rp->normal_stride * 3;
            for (uint32_t frame = 1; frame < frames; ++frame) {
                const float* nn = nrm + (uint64_t)(frame - 1) * 3;
                float dx = rwsd * nn[0];
                x = periodic_bounds(x + dx, s->half_lx);
                float dy = rwsd * nn[1];
                y = periodic_bounds(y + dy, s->half_ly);
                float dz = rwsd * nn[2];
                z = periodic_bounds(z + dz, s->half_lz);
                if (detected(x, y, z, half_az, s)) {
                    ++k;
                    if (k >= 2u) {
                        float dx2 = dx * dx;
                        float dy2 = dy * dy;
                        float sum = dx2 + dy2;
                        de = de + sum;
                    }
                } else {
                    if (k >= s->kmin) record(s, hist, k, de, counts);
                    k = 0;
                    de = 0.0f;
                }
            }
            if (k >= s->kmin) record(s, hist, k, de, counts);
        }
    }
    return 0;
}

static void bm_pair(uint32_t ra, uint32_t rb, float* n0, float* n1)
{
    float u = fmaf((float)ra, 2.3283064365386963e-10f, 1.1641532182693481e-10f);
    double x = -2.0 * log((double)u);
    double rad = sqrt(x);
    float t = fmaf((float)rb, 1.4629180792671596e-09f, -3.14159265358979f);
    *n0 = (float)(rad * sin((double)t));
    *n1 = (float)(rad * cos((double)t));
}

/* Track bookkeeping of one step (kernel-simulate.inl:70-93). */
static void track_step(const orc_setup* s, uint32_t* hist, orc_track_counts* counts, int det, float de_step,
                       uint32_t* k, float* de)
{
    if (det) {
        ++*k;
        if (*k >= 2u) *de = *de + de_step;
    } else {
        if (*k >= s->kmin) record(s, hist, *k, *de, counts);
        *k = 0;
        *de = 0.0f;
    }
}

/* The slab-split walk of one particle (steps 1..frames-1): the same model as
 * the per-step walk with fewer draws.  Steps go in groups of four (m <= 4 in
 * the last group); per group:
 *   z: four normals from one Philox block, z walked step by step exactly;
 *   x, y: the group's summed displacement drawn at once, S = sd sqrt(m) n,
 *     applied with one wrap;
 *   if any z of the group lies in the detection slab, the group's x, y steps
 *     are drawn conditionally on their sum (Gaussian bridge:
 *     d_i = S/m + sd (n_i - mean n), exactly i.i.d. N(0, sd^2) again), walked
 *     from the group's start and checked for detection; otherwise nothing in
 *     the group is detected.
 * Blocks per group pair h (groups 2h, 2h+1): 2+8h z(2h), 3+8h z(2h+1),
 * 4+8h the sums of both groups, 5+8h..6+8h the x, y steps of group 2h,
 * 7+8h..8+8h those of group 2h+1. */
static void walk_split(const orc_setup* s, uint32_t* hist, orc_track_counts* counts, uint32_t ctr[4],
                       const uint32_t key[2], uint32_t frames, float sd, float half_az, float* px, float* py,
                       float* pz, uint32_t* pk, float* pde)
{
    static const float sqrt_m[5] = {0.0f, 1.0f, 1.41421356237f, 1.73205080757f, 2.0f};
    static const float inv_m[5] = {0.0f, 1.0f, 0.5f, 0.333333333333f, 0.25f};
    float x = *px, y = *py, z = *pz, de = *pde;
    uint32_t k = *pk;
    const uint32_t steps = frames > 0u ? frames - 1u : 0u;
    const uint32_t groups = (steps + 3u) / 4u;
    uint32_t w[4];
    float agg[4] = {0, 0, 0, 0};
    for (uint32_t g = 0; g < groups; ++g) {
        const uint32_t m = (steps - 4u * g < 4u) ? steps - 4u * g : 4u;
        const uint32_t base = 2u + 8u * (g >> 1), odd = g & 1u;
        float nz[4];
        ctr[1] = base + odd;
        orc_philox4x32_10(ctr, key, w);
        bm_pair(w[0], w[1], &nz[0], &nz[1]);
        bm_pair(w[2], w[3], &nz[2], &nz[3]);
        if (!odd) {
            ctr[1] = base + 2u;
            orc_philox4x32_10(ctr, key, w);
            bm_pair(w[0], w[1], &agg[0], &agg[1]);
            bm_pair(w[2], w[3], &agg[2], &agg[3]);
        }
        uint32_t zbits = 0;
        for (uint32_t i = 0; i < m; ++i) {
            const float dz = sd * nz[i];
            z = periodic_bounds(z + dz, s->half_lz);
            if (fabsf(z) <= half_az) zbits |= 1u << i;
        }
        const float sds = sd * sqrt_m[m];
        const float sx = sds * agg[2 * odd], sy = sds * agg[2 * odd + 1];
        const float xs = x, ys = y;
        x = periodic_bounds(x + sx, s->half_lx);
        y = periodic_bounds(y + sy, s->half_ly);
        if (!zbits) {
            track_step(s, hist, counts, 0, 0.0f, &k, &de);
            continue;
        }
        float nx[4], ny[4];
        ctr[1] = base + 3u + 2u * odd;
        orc_philox4x32_10(ctr, key, w);
        bm_pair(w[0], w[1], &nx[0], &ny[0]);
        bm_pair(w[2], w[3], &nx[1], &ny[1]);
        ctr[1] = base + 4u + 2u * odd;
        orc_philox4x32_10(ctr, key, w);
        bm_pair(w[0], w[1], &nx[2], &ny[2]);
        bm_pair(w[2], w[3], &nx[3], &ny[3]);
        float mx = 0.0f, my = 0.0f;
        for (uint32_t i = 0; i < m; ++i) {
            mx = mx + nx[i];
            my = my + ny[i];
        }
        mx = mx * inv_m[m];
        my = my * inv_m[m];
        const float cx = sx * inv_m[m], cy = sy * inv_m[m];
        float xx = xs, yy = ys;
        for (uint32_t i = 0; i < m; ++i) {
            const float dx = cx + sd * (nx[i] - mx);
            const float dy = cy + sd * (ny[i] - my);
            xx = periodic_bounds(xx + dx, s->half_lx);
            yy = periodic_bounds(yy + dy, s->half_ly);
            const int det = ((zbits >> i) & 1u) && fabsf(xx) <= s->half_ax && fabsf(yy) <= s->half_ay;
            const float dx2 = dx * dx;
            const float dy2 = dy * dy;
            track_step(s, hist, counts, det, dx2 + dy2, &k, &de);
        }
    }
    *px = x;
    *py = y;
    *pz = z;
    *pk = k;
    *pde = de;
}

static int simulate_philox_(const orc_setup* s, const orc_run* r, uint64_t seed, uint32_t slot,
                            uint32_t trial, uint32_t generation, uint32_t* hist,
                            orc_track_counts* counts, int split)
{
    orc_track_counts local = {0, 0};
    if (!counts) counts = &local;
    /* fixed key, seed folded into counter words 2 and 3 through the
     * splitmix64 finaliser (the product's stream layout) */
    const uint32_t key[2] = {0xA4093822u, 0x299F31D0u};
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const uint32_t m0 = (uint32_t)z, m1 = (uint32_t)(z >> 32);
    const uint32_t gt = ((generation << 20) | (trial & 0xFFFFFu)) ^ m1;
    slot ^= m0;
    uint32_t n = 0;
    for (uint32_t v = 0; v < s->video_count; ++v) {
        const uint32_t frames = r->frames[v];
        for (uint32_t p = 0; p < r->particles[v]; ++p, ++n) {
            uint32_t ctr[4] = {n, 0u, slot, gt}, w[4];
            orc_philox4x32_10(ctr, key, w);
            float u[4];
            for (int i = 0; i < 4; ++i) u[i] = (float)(w[i] >> 8) * (1.0f / 16777216.0f);
            float x = s->half_lx * (2.0f * u[0] - 1.0f);
            float y = s->half_ly * (2.0f * u[1] - 1.0f);
            float z = s->half_lz * (2.0f * u[2] - 1.0f);
            uint32_t idx = 0;
            if (s->component_count > 1) idx = wrand_index(u[3], s->component_count, r->pre_comp_prob);
            if (idx >= s->component_count) return -3;
            float half_az = (s->model == ORC_MODEL_DISCRETE_VARIABLE_Z) ? r->half_az[idx] : r->half_az[0];
            float sd = r->rand_walk_stddev[idx];
            if (s->model == ORC_MODEL_LOGNORMAL) {
                ctr[1] = 1u;
                orc_philox4x32_10(ctr, key, w);
                float z0, z1;
                bm_pair(w[0], w[1], &z0, &z1);
                sd = r->ln_scale[idx] * (float)exp((double)(r->ln_shape[idx] * z0));
            }
            float de = 0.0f;
            uint32_t k = detected(x, y, z, half_az, s) ? 1u : 0u;
            if (split) {
                walk_split(s, hist, counts, ctr, key, frames, sd, half_az, &x, &y, &z, &k, &de);
                if (k >= s->kmin) record(s, hist, k, de, counts);
                continue;
            }
            float nn[12];
            for (uint32_t frame = 1; frame < frames; ++frame) {
                const uint32_t g = (frame - 1) >> 2, sub = (frame - 1) & 3u;
                if (sub == 0) {
                    for (uint32_t b = 0; b < 3; ++b) {
                        ctr[1] = 2u + 3u * g + b;
                        orc_philox4x32_10(ctr, key, w);
                        bm_pair(w[0], w[1], &nn[4 * b + 0], &nn[4 * b + 1]);
                        bm_pair(w[2], w[3], &nn[4 * b + 2], &nn[4 * b + 3]);
                    }
                }
                float dx = sd * nn[3 * sub + 0];
                x = periodic_bounds(x + dx, s->half_lx);
                float dy = sd * nn[3 * sub + 1];
                y = periodic_bounds(y + dy, s->half_ly);
                float dz = sd * nn[3 * sub + 2];
                z = periodic_bounds(z + dz, s->half_lz);
                if (detected(x, y, z, half_az, s)) {
                    ++k;
                    if (k >= 2u) {
                        float dx2 = dx * dx;
                        float dy2 = dy * dy;
                        float sum = dx2 + dy2;
                        de = de + sum;
                    }
                } else {
                    if (k >= s->kmin) record(s, hist, k, de, counts);
                    k = 0;
                    de = 0.0f;
                }
            }
            if (k >= s->kmin) record(s, hist, k, de, counts);
        }
    }
    return 0;
}

int orc_simulate_philox(const orc_setup* s, const orc_run* r, uint64_t seed, uint32_t slot,
                        uint32_t trial, uint32_t generation, uint32_t* hist,
                        orc_track_counts* counts)
{
    return simulate_philox_(s, r, seed, slot, trial, generation, hist, counts, 0);
}

int orc_simulate_philox_split(const orc_setup* s, const orc_run* r, uint64_t seed, uint32_t slot,
                              uint32_t trial, uint32_t generation, uint32_t* hist,
                              orc_track_counts* counts)
{
    return simulate_philox_(s, r, seed, slot, trial, generation, hist, counts, 1);
}

/* ------------------------------------------------------------------ */
/* Observed cumulative histogram (simulation_impl.inl:605-629)         */
/* ------------------------------------------------------------------ */

int orc_observed_sat(const uint32_t* K, const double* DE, size_t n, uint32_t rows,
                     uint32_t bins, double ub_de, uint32_t* sat)
{
    double width = ub_de / (double)bins; /* mDEBinWidth (:516) */
    uint64_t total = (uint64_t)rows * bins;
    memset(sat, 0, sizeof(uint32_t) * total);
    for (size_t i = 0; i < n; ++i) {
        if (DE[i] >= ub_de) continue;
        long idx = (long)(DE[i] / width);
        /* reference(K, idx) on a row-major R x B matrix */
        long long flat = (long long)K[i] * bins + idx;
        if (flat < 0 || (unsigned long long)flat >= total) return -1;
        sat[flat] += 1u;
    }
    for (uint32_t c = 0; c < bins; ++c) /* column-wise partial_sum (:620-624) */
        for (uint32_t r = 1; r < rows; ++r) sat[(uint64_t)r * bins + c] += sat[(uint64_t)(r - 1) * bins + c];
    for (uint32_t r = 0; r < rows; ++r) /* row-wise partial_sum (:625-629) */
        for (uint32_t c = 1; c < bins; ++c) sat[(uint64_t)r * bins + c] += sat[(uint64_t)r * bins + c - 1];
    return 0;
}

/* ------------------------------------------------------------------ */
/* K_distance (kernel-distance.inl:81-241)                             */
/* ------------------------------------------------------------------ */

/* reduce0 (kernel-distance.inl:69-78) as seen by lane 0: a shfl_down tree
 * 16, 8, 4, 2, 1 where out-of-range lanes read their own value. */
static float reduce0_f32(const float* v32)
{
    float v[32], t[32];
    memcpy(v, v32, sizeof v);
    for (int d = 16; d >= 1; d >>= 1) {
        for (int l = 0; l < 32; ++l) t[l] = v[l] + ((l + d < 32) ? v[l + d] : v[l]);
        memcpy(v, t, sizeof v);
    }
    return v[0];
}

static double reduce0_f64(const double* v32)
{
    double v[32], t[32];
    memcpy(v, v32, sizeof v);
    for (int d = 16; d >= 1; d >>= 1) {
        for (int l = 0; l < 32; ++l) t[l] = v[l] + ((l + d < 32) ? v[l + d] : v[l]);
        memcpy(v, t, sizeof v);
    }
    return v[0];
}

static uint32_t* prefix2d(const uint32_t* hist, uint32_t rows, uint32_t bins)
{
    uint64_t total = (uint64_t)rows * bins;
    uint32_t* cum = (uint32_t*)malloc(sizeof(uint32_t) * (total ? total : 1));
    if (!cum) return NULL;
    memcpy(cum, hist, sizeof(uint32_t) * total);
    /* first pass: along DE within each row (:105-148) */
    for (uint32_t r = 0; r < rows; ++r)
        for (uint32_t c = 1; c < bins; ++c) cum[(uint64_t)r * bins + c] += cum[(uint64_t)r * bins + c - 1];
    /* second pass: along K within each column (:152-208) */
    for (uint32_t c = 0; c < bins; ++c)
        for (uint32_t r = 1; r < rows; ++r) cum[(uint64_t)r * bins + c] += cum[(uint64_t)(r - 1) * bins + c];
    return cum;
}

float orc_distance_kdist(const uint32_t* hist, const uint32_t* ref_sat, uint32_t rows,
                         uint32_t bins, uint32_t* cum_out, uint64_t* ssd_hi, uint64_t* ssd_lo)
{
    uint32_t* cum = prefix2d(hist, rows, bins);
    if (!cum) return -1.0f;
    unsigned __int128 ssd = 0;
    float acc[32][32];
    for (int w = 0; w < 32; ++w) {
        for (int l = 0; l < 32; ++l) {
            float a = 0.0f;
            for (uint32_t col = (uint32_t)w; col < bins; col += 32) {
                float a2 = 0.0f;
                for (uint32_t row = (uint32_t)l; row < rows; row += 32) {
                    uint64_t i = (uint64_t)row * bins + col;
                    float dd = (float)cum[i] - (float)ref_sat[i];
                    float sq = dd * dd;
                    a2 = a2 + sq;
                }
                a = a + a2;
            }
            acc[w][l] = a;
        }
    }
    for (uint64_t i = 0; i < (uint64_t)rows * bins; ++i) {
        int64_t d = (int64_t)cum[i] - (int64_t)ref_sat[i];
        unsigned __int128 ad = (unsigned __int128)(d < 0 ? -d : d);
        ssd += ad * ad;
    }
    float totals[32];
    for (int w = 0; w < 32; ++w) totals[w] = reduce0_f32(acc[w]);
    float fin = reduce0_f32(totals);
    if (cum_out) memcpy(cum_out, cum, sizeof(uint32_t) * (uint64_t)rows * bins);
    if (ssd_hi) *ssd_hi = (uint64_t)(ssd >> 64);
    if (ssd_lo) *ssd_lo = (uint64_t)ssd;
    free(cum);
    return fin;
}

double orc_distance_kdist_f64(const uint32_t* hist, const uint32_t* ref_sat, uint32_t rows,
                              uint32_t bins)
{
    uint32_t* cum = prefix2d(hist, rows, bins);
    if (!cum) return -1.0;
    double acc[32][32];
    for (int w = 0; w < 32; ++w) {
        for (int l = 0; l < 32; ++l) {
            double a = 0.0;
            for (uint32_t col = (uint32_t)w; col < bins; col += 32) {
                double a2 = 0.0;
                for (uint32_t row = (uint32_t)l; row < rows; row += 32) {
                    uint64_t i = (uint64_t)row * bins + col;
                    double dd = (double)cum[i] - (double)ref_sat[i];
                    double sq = dd * dd;
                    a2 = a2 + sq;
                }
                a = a + a2;
            }
            acc[w][l] = a;
        }
    }
    double totals[32];
    for (int w = 0; w < 32; ++w) totals[w] = reduce0_f64(acc[w]);
    free(cum);
    return reduce0_f64(totals);
}

/* ------------------------------------------------------------------ */
/* Julia conventions (src/cpu/simulate.jl, distance.jl)                */
/* ------------------------------------------------------------------ */

/* position_periodic (position_periodic.jl:1-9) */
static double position_periodic(double x, double L)
{
    if (x > L)
        x = x - L;
    else if (x < 0.0)
        x = x + L;
    return x;
}

static void julia_record(int64_t* H, uint32_t k, double de, double deltat, double d_de,
                         uint32_t B)
{
    de = de / ((double)(k - 1) * 4.0 * deltat);
    double q = ceil(de / d_de);
    if (q >= 1.0 && q <= (double)B) {
        int64_t idx = (int64_t)q;
        H[(uint64_t)(k - 1) * B + (uint64_t)(idx - 1)] += 1;
    }
}

int orc_simulate_julia(uint32_t C, const double* m, const double* c, double ax, double ay,
                       const double* az, double Lx, double Ly, double Lz,
                       const uint32_t* frames, const uint32_t* particles, uint32_t V,
                       double deltat, uint32_t kmin, uint32_t B, double ub_de,
                       const orc_replay_f64* rp, int64_t* H)
{
    if (C < 1 || C > ORC_MAX_COMPONENTS) return -1;
    double csum = 0.0;
    for (uint32_t i = 0; i < C; ++i) csum += c[i];
    double cum[ORC_MAX_COMPONENTS];
    double acc = 0.0;
    for (uint32_t i = 0; i < C; ++i) {
        acc += c[i] / csum;
        cum[i] = acc;
    }
    double d_de = ub_de / (double)B;
    uint64_t n = 0;
    for (uint32_t v = 0; v < V; ++v) {
        for (uint32_t p = 0; p < particles[v]; ++p, ++n) {
            const double* u = rp->uniforms + 4 * n;
            /* rand_weighted_index (rand_weighted_index.jl:1-8) */
            uint32_t index = 0;
            while (index + 1 < C && cum[index] < u[0]) ++index;
            double sd = sqrt(2.0 * m[index] * deltat);
            double x = Lx * u[1], y = Ly * u[2], z = Lz * u[3];
            double de = 0.0;
            uint32_t k = (fabs(z - 0.5 * Lz) <= 0.5 * az[index] && fabs(x - 0.5 * Lx) <= 0.5 * ax &&
                          fabs(y - 0.5 * Ly) <= 0.5 * ay)
                             ? 1u
                             : 0u;
            for (uint32_t f = 2; f <= frames[v]; ++f) {
                const double* nn = rp->normals + ((uint64_t)n * rp->normal_stride + (f - 2)) * 3;
                double dxv = sd * nn[0], dyv = sd * nn[1], dzv = sd * nn[2];
                x = position_periodic(x + dxv, Lx);
                y = position_periodic(y + dyv, Ly);
                z = position_periodic(z + dzv, Lz);
                if (fabs(z - 0.5 * Lz) <= 0.5 * az[index] && fabs(x - 0.5 * Lx) <= 0.5 * ax &&
                    fabs(y - 0.5 * Ly) <= 0.5 * ay) {
                    k = k + 1;
                    if (k >= 2) de = de + dxv * dxv + dyv * dyv;
                } else if (k > 0) {
                    if (k >= kmin) julia_record(H, k, de, deltat, d_de, B);
                    k = 0;
                    de = 0.0;
                }
            }
            if (k >= kmin && k > 0) julia_record(H, k, de, deltat, d_de, B);
        }
    }
    return 0;
}

int orc_observed_sat_julia(const uint32_t* K, const double* DE, size_t n, uint32_t kmax, uint32_t B,
                           double ub_de, uint32_t* sat)
{
    const double d_de = ub_de / (double)B; /* estimate.jl:29 */
    memset(sat, 0, sizeof(uint32_t) * (size_t)kmax * B);
    int rc = 0;
    for (size_t i = 0; i < n; ++i) {
        const double q = ceil(DE[i] / d_de);
        if (!(q >= 1.0 && q <= (double)B)) continue;
        if (K[i] < 1u || K[i] > kmax) {
            rc = -1;
            continue;
        }
        sat[(size_t)(K[i] - 1u) * B + (size_t)q - 1u] += 1u;
    }
    for (uint32_t c = 0; c < B; ++c)
        for (uint32_t r = 1; r < kmax; ++r) sat[(size_t)r * B + c] += sat[(size_t)(r - 1) * B + c];
    for (uint32_t r = 0; r < kmax; ++r)
        for (uint32_t c = 1; c < B; ++c) sat[(size_t)r * B + c] += sat[(size_t)r * B + c - 1];
    return rc;
}

double orc_distance_julia(const int64_t* H, const int64_t* Hsim, uint32_t kmax, uint32_t B)
{
    /* cumsum(cumsum(H - Hsim, 1), 2) then log10(sum(.^2)) */
    uint64_t total = (uint64_t)kmax * B;
    double* d = (double*)malloc(sizeof(double) * (total ? total : 1));
    if (!d) return NAN;
    for (uint64_t i = 0; i < total; ++i) d[i] = (double)(H[i] - Hsim[i]);
    for (uint32_t col = 0; col < B; ++col)
        for (uint32_t r = 1; r < kmax; ++r) d[(uint64_t)r * B + col] += d[(uint64_t)(r - 1) * B + col];
    for (uint32_t r = 0; r < kmax; ++r)
        for (uint32_t col = 1; col < B; ++col) d[(uint64_t)r * B + col] += d[(uint64_t)r * B + col - 1];
    double s = 0.0;
    for (uint64_t i = 0; i < total; ++i) s += d[i] * d[i];
    free(d);
    return log10(s);
}

/* ------------------------------------------------------------------ */
/* PMC pieces                                                          */
/* ------------------------------------------------------------------ */

/* var_ (simulation_impl.inl:24-44): uncorrected 1/N variance. */
double orc_var_uncorrected(const double* x, size_t n, size_t stride)
{
    double accum = 0.0, count = 0.0;
    for (size_t i = 0; i < n; ++i, count += 1.0) accum += x[i * stride];
    double mean = accum / count;
    double var = 0.0;
    for (size_t i = 0; i < n; ++i) {
        double d = x[i * stride] - mean;
        var += d * d;
    }
    return var / count;
}

/* normpdf_ (simulation_impl.inl:46-52). */
double orc_normpdf(double x, double mu, double sigma)
{
    double xm = x - mu;
    return exp(-0.5 * xm * xm / (sigma * sigma)) / (sqrt(2.0 * M_PI) * sigma);
}

/* displace_ (simulation_impl.inl:64-79) with the normal draw supplied. */
double orc_displace(double current, double delta, double lower, double upper)
{
    double bis = current + delta;
    while (bis < lower || bis > upper) {
        if (bis < lower) bis += 2.0 * (lower - bis);
        if (bis > upper) bis -= 2.0 * (bis - upper);
    }
    return bis;
}

/* weighting_scheme_pmc_standard_ (simulation_impl.inl:832-871). */
void orc_weights_pmc_standard(const double* theta_star, const double* theta, const double* w,
                              const double* tau, const int* fixed, size_t N, size_t P,
                              double* w_out)
{
    double wsum = 0.0;
    for (size_t a = 0; a < N; ++a) {
        double ws = 0.0;
        for (size_t i = 0; i < N; ++i) {
            double term = 1.0;
            for (size_t p = 0; p < P; ++p) {
                if (fixed && fixed[p]) continue;
                term *= orc_normpdf(theta_star[a * P + p] - theta[i * P + p], 0.0, tau[p]);
            }
            ws += w[i] * term;
        }
        w_out[a] = 1.0 / ws;
        wsum += w_out[a];
    }
    for (size_t a = 0; a < N; ++a) w_out[a] = w_out[a] / wsum;
}

/* weighting_scheme_inv_dist_sq_ (simulation_impl.inl:872-887). */
void orc_weights_inv_dist_sq(const double* dist, size_t N, double* w_out)
{
    double wsum = 0.0;
    for (size_t i = 0; i < N; ++i) {
        w_out[i] = 1.0 / (dist[i] * dist[i]);
        wsum += w_out[i];
    }
    for (size_t i = 0; i < N; ++i) w_out[i] /= wsum;
}

int orc_weighted_cov_cholesky(const double* theta, const double* w, size_t N, size_t P,
                              double scale, double* cov, double* chol)
{
    double mean[64];
    if (P > 64) return -1;
    double wsum = 0.0;
    for (size_t i = 0; i < N; ++i) wsum += w[i];
    for (size_t p = 0; p < P; ++p) {
        double s = 0.0;
        for (size_t i = 0; i < N; ++i) s += w[i] * theta[i * P + p];
        mean[p] = s / wsum;
    }
    for (size_t a = 0; a < P; ++a)
        for (size_t b = 0; b < P; ++b) {
            double s = 0.0;
            for (size_t i = 0; i < N; ++i) s += w[i] * (theta[i * P + a] - mean[a]) * (theta[i * P + b] - mean[b]);
            cov[a * P + b] = scale * s / wsum;
        }
    memset(chol, 0, sizeof(double) * P * P);
    for (size_t j = 0; j < P; ++j) {
        double d = cov[j * P + j];
        for (size_t k = 0; k < j; ++k) d -= chol[j * P + k] * chol[j * P + k];
        if (!(d > 0.0)) return -2;
        double l = sqrt(d);
        chol[j * P + j] = l;
        for (size_t i = j + 1; i < P; ++i) {
            double s = cov[i * P + j];
            for (size_t k = 0; k < j; ++k) s -= chol[i * P + k] * chol[j * P + k];
            chol[i * P + j] = s / l;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Proposal construction (simulation_impl.inl:256-347)                 */
/* ------------------------------------------------------------------ */

enum { STREAM_POISSON = 1u, STREAM_PERTURB = 2u, STREAM_PICK = 3u };

/* one Philox block of a job's stream: counter (c0, tag << 28 | j,
 * slot ^ m0, (generation << 20 | trial) ^ m1), fixed key */
static void job_draw(uint64_t seed, uint32_t c0, uint32_t tag, uint32_t j, uint32_t slot, uint32_t gen,
                     uint32_t trial, uint32_t w[4])
{
    const uint32_t key[2] = {0xA4093822u, 0x299F31D0u};
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const uint32_t ctr[4] = {c0, (tag << 28) | (j & 0x0FFFFFFFu), slot ^ (uint32_t)z,
                             ((gen << 20) | (trial & 0xFFFFFu)) ^ (uint32_t)(z >> 32)};
    orc_philox4x32_10(ctr, key, w);
}

/* [0,1) with 53 bits: 27 bits of the first word, 26 of the second */
static double unit53(uint32_t a, uint32_t b)
{
    return (double)((((uint64_t)(a >> 5)) << 26) | (uint64_t)(b >> 6)) / 9007199254740992.0;
}

/* Poisson(lam) for one video.  lam < 12: inversion, one uniform.  lam >=
 * 12: PTRS, the transformed rejection with squeeze of W. Hoermann, "The
 * transformed rejection method for generating Poisson random variables",
 * Insurance: Mathematics and Economics 12 (1993) 39-45, attempt t drawing
 * (U, V) from block 1 + t; after 256 rejected attempts, round(lam). */
static uint32_t poisson_video(uint64_t seed, double lam, uint32_t video, uint32_t slot, uint32_t gen,
                              uint32_t trial)
{
    uint32_t w[4];
    if (!(lam > 0.0)) return 0u;
    if (lam < 12.0) {
        job_draw(seed, video, STREAM_POISSON, 0u, slot, gen, trial, w);
        const double u = unit53(w[0], w[1]);
        double pk = exp(-lam), cdf = pk;
        uint32_t k = 0;
        while (cdf < u && k < 1000u) {
            k += 1u;
            pk = pk * (lam / (double)k);
            cdf = cdf + pk;
        }
        return k;
    }
    const double b = 0.931 + 2.53 * sqrt(lam);
    const double a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
    const double v_r = 0.9277 - 3.6224 / (b - 2.0);
    for (uint32_t t = 0; t < 256u; ++t) {
        job_draw(seed, video, STREAM_POISSON, 1u + t, slot, gen, trial, w);
        const double U = unit53(w[0], w[1]) - 0.5;
        const double V = unit53(w[2], w[3]);
        const double us = 0.5 - fabs(U);
        const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
        if (us >= 0.07 && V <= v_r) return (uint32_t)k;
        if (k < 0.0) continue;
        if (us < 0.013 && V > us) continue;
        /* accept iff V inv_alpha / (a / us^2 + b) <= lam^k e^-lam / k!, in logs */
        const double lhs = log(V) + log(inv_alpha) - log(a / (us * us) + b);
        const double rhs = -lam + k * log(lam) - lgamma(k + 1.0);
        if (lhs <= rhs) return (uint32_t)k;
    }
    return (uint32_t)floor(lam + 0.5);
}

int orc_build_proposal(const orc_prop_job* j, const double* theta, const double* wcum, const double* factor,
                       uint32_t slot, uint32_t trial, uint32_t generation, double* theta_out,
                       uint32_t* counts, orc_proposal* out)
{
    const uint32_t P = j->P, C = j->C, Z = j->Z, N = j->N;
    if (P > 32 || C > ORC_MAX_COMPONENTS || Z > ORC_MAX_COMPONENTS || N == 0) return -1;
    const int lognormal = j->model == ORC_MODEL_LOGNORMAL;
    const uint32_t om = 0, os = C, oc = lognormal ? 2 * C : C, oaz = oc + C;
    double th[32];
    uint32_t w[4];
    memset(out, 0, sizeof *out);
    if (generation == 0u) {
        memcpy(th, theta + (size_t)slot * P, P * sizeof(double));
        out->parent = slot;
    } else {
        /* wrand_idx_: first cumulative weight not below U, at most N - 1 */
        job_draw(j->seed, 0u, STREAM_PICK, 0u, slot, generation, trial, w);
        const double u = unit53(w[0], w[1]);
        uint32_t idx = N - 1u;
        for (uint32_t i = 0; i < N; ++i)
            if (!(wcum[i] < u)) {
                idx = i;
                break;
            }
        out->parent = idx;
        /* normals, pair q/2 from one block: u1 in (0, 1], u2 in [0, 1) */
        double n[32];
        for (uint32_t q = 0; q < P; q += 2) {
            job_draw(j->seed, q / 2u, STREAM_PERTURB, 0u, slot, generation, trial, w);
            const double u1 = 1.0 - unit53(w[0], w[1]);
            const double u2 = unit53(w[2], w[3]);
            const double r = sqrt(-2.0 * log(u1));
            n[q] = r * sin(2.0 * M_PI * u2);
            if (q + 1 < P) n[q + 1] = r * cos(2.0 * M_PI * u2);
        }
        const double* parent = theta + (size_t)idx * P;
        for (uint32_t p = 0; p < P; ++p) {
            if (j->lo[p] == j->hi[p]) { /* a fixed parameter is not perturbed */
                th[p] = j->lo[p];
                continue;
            }
            double delta = 0.0;
            if (j->perturbation == 1u) {
                for (uint32_t i = 0; i <= p; ++i)
                    if (j->lo[i] != j->hi[i]) delta += factor[p * P + i] * n[i];
            } else {
                delta = factor[p * P + p] * n[p];
            }
            th[p] = orc_displace(parent[p], delta, j->lo[p], j->hi[p]);
        }
        /* label switching: order the components by m (std::sort on indices) */
        uint32_t order[ORC_MAX_COMPONENTS];
        for (uint32_t i = 0; i < C; ++i) order[i] = i;
        for (uint32_t i = 1; i < C; ++i)
            for (uint32_t x = i; x > 0 && th[om + order[x]] < th[om + order[x - 1]]; --x) {
                const uint32_t t = order[x];
                order[x] = order[x - 1];
                order[x - 1] = t;
            }
        double tmp[32];
        memcpy(tmp, th, P * sizeof(double));
        for (uint32_t i = 0; i < C; ++i) {
            th[om + i] = tmp[om + order[i]];
            th[oc + i] = tmp[oc + order[i]];
            if (lognormal) th[os + i] = tmp[os + order[i]];
            if (Z > 1u) th[oaz + i] = tmp[oaz + order[i]];
        }
    }
    memcpy(theta_out, th, P * sizeof(double));

    /* concentrations, Poisson mean, component probabilities, step sd */
    double powc[ORC_MAX_COMPONENTS], csum = 0.0;
    for (uint32_t i = 0; i < C; ++i) {
        powc[i] = pow(10.0, th[oc + i]);
        csum += powc[i];
    }
    const double lambda = csum * j->volume_factor;
    out->lambda = lambda;
    for (uint32_t i = 0; i < ORC_MAX_COMPONENTS; ++i) out->pre_comp_prob[i] = 2.0f;
    double acc = 0.0;
    for (uint32_t i = 0; i < C; ++i) {
        acc += powc[i] / csum;
        out->pre_comp_prob[i] = (float)acc;
        if (lognormal) {
            const double mu = th[om + i], sd = th[os + i];
            const double sl2 = log1p((sd * sd) / (mu * mu));
            const double mul = log(mu) - 0.5 * sl2;
            out->sd_scale[i] = (float)(j->sd_const * exp(-0.5 * mul));
            out->sd_shape[i] = (float)(-0.5 * sqrt(sl2));
        } else {
            out->sd_scale[i] = (float)sqrt(2.0 * th[om + i] * j->delta_t);
        }
    }
    out->pre_comp_prob[C - 1] = 2.0f;
    for (uint32_t z = 0; z < Z; ++z) {
        const float az = (float)th[oaz + z];
        out->half_az[z] = (generation == 0u && j->full_az_prior) ? az : 0.5f * az;
    }
    uint64_t total = 0;
    for (uint32_t v = 0; v < j->V; ++v) {
        counts[v] = poisson_video(j->seed, lambda, v, slot, generation, trial);
        total += counts[v];
    }
    out->total_particles = total > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)total;
    return 0;
}
