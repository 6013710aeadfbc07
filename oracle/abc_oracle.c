/*
 * abc_oracle.c -- an independent CPU run of the whole ABC-PMC estimation.
 *
 * TEST INFRASTRUCTURE ONLY: the statistical checker for posteriors
 * (tests/test_gpu_posterior.py).  It follows the reference's algorithm
 * (src/gpu/detail/simulation_impl.inl:178-887; src/cpu/estimate.jl) with
 * none of the GPU path's machinery: its own random numbers (xoshiro256+ per
 * slot and generation, polar-method normals), the Julia exponential-gap
 * Poisson sampler (src/cpu/rand_poisson.jl), the forward model of
 * pcs_oracle.c's conventions (GPU conventions, float walk, one thread per
 * slot at a time), the cumulative distance in the reference order, the
 * reference's double-precision pmc-standard weights and tau = sqrt(2 var).
 * Models: lognormal diameters (mean m, sd s) with Stokes-Einstein steps,
 * log10 concentrations, one fixed depth; or the reference's discrete
 * diffusivities with one depth parameter (discrete-fixed-depth,
 * simulation_impl.inl:178-455), whose prior pass uses az itself as the half
 * depth when full_az_prior is set (:782).  Schedules: epsilon = q-quantile of
 * the previous generation's distances (prior pass for the first), or the
 * reference's gamma_0 = rank N/2 of the prior distances (:819-829) lowered
 * by delta_gamma at the start of each generation (:202-219), with the trial
 * cap discarding the generation that reaches it (:425-428).
 */
#include <math.h>
#include <stdio.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pcs_oracle.h"

typedef struct rng {
    uint64_t s[4];
    int have;
    double spare;
} rng;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint64_t rn_next(rng* r)
{
    uint64_t* s = r->s;
    uint64_t res = s[0] + s[3], t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return res;
}
static inline double rn_u(rng* r) { return (double)(rn_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static void rn_seed(rng* r, uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t seed = a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull) * 0xBF58476D1CE4E5B9ull ^ c * 0x94D049BB133111EBull;
    for (int i = 0; i < 4; ++i) {
        uint64_t z = (seed += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        r->s[i] = z ^ (z >> 31);
    }
    r->have = 0;
    r->spare = 0.0;
}
static inline double rn_n(rng* r)
{
    if (r->have) {
        r->have = 0;
        return r->spare;
    }
    double u, v, q;
    do {
        u = 2.0 * rn_u(r) - 1.0;
        v = 2.0 * rn_u(r) - 1.0;
        q = u * u + v * v;
    } while (q >= 1.0 || q == 0.0);
    double f = sqrt(-2.0 * log(q) / q);
    r->spare = v * f;
    r->have = 1;
    return u * f;
}



#define OP_MAXP 24

typedef struct ctx_t {
    const orc_abc_problem* pb;
    uint32_t P;
    double lo[OP_MAXP], hi[OP_MAXP];
    double* theta;     /* [N*P] */
    double* theta_new; /* [N*P] */
    double* w;
    double* wcum;
    double* dist;
    double* dist_new;
    double tau[OP_MAXP];
    double gamma;
    uint32_t gen;
    uint64_t seed;
    uint32_t oc, oaz;  /* offsets of log10c and az in a parameter vector */
    uint64_t trial_cap; /* trials per generation at which it is discarded (0: none) */
    atomic_uint next;
    atomic_ullong trials;
    atomic_ullong gen_trials;
} ctx_t;

/* forward model of one proposal, GPU conventions (pcs_oracle.c) */
static double simulate_distance(const ctx_t* c, const double* th, rng* r, uint32_t* hist)
{
    const orc_abc_problem* pb = c->pb;
    const uint32_t C = pb->C;
    memset(hist, 0, sizeof(uint32_t) * (size_t)pb->R * pb->B);
    const int lognormal = pb->model == ORC_MODEL_LOGNORMAL;
    double csum = 0.0, powc[ORC_MAX_COMPONENTS];
    for (uint32_t i = 0; i < C; ++i) {
        powc[i] = pow(10.0, th[c->oc + i]);
        csum += powc[i];
    }
    float pre[ORC_MAX_COMPONENTS];
    double acc = 0.0;
    for (uint32_t i = 0; i < C; ++i) {
        acc += powc[i] / csum;
        pre[i] = (float)acc;
    }
    pre[C - 1] = 2.0f;
    const double kB = 1.380649e-23;
    const double g = sqrt(2.0 * pb->deltat * kB * pb->temperature * 1e21 / (3.0 * M_PI * pb->viscosity));
    double mul[ORC_MAX_COMPONENTS], sl[ORC_MAX_COMPONENTS];
    float sd_fixed[ORC_MAX_COMPONENTS];
    for (uint32_t i = 0; i < C; ++i) {
        if (lognormal) {
            const double mu = th[i], sd = th[C + i];
            const double s2 = log1p(sd * sd / (mu * mu));
            sl[i] = sqrt(s2);
            mul[i] = log(mu) - 0.5 * s2;
        } else {
            sd_fixed[i] = (float)sqrt(2.0 * th[i] * pb->deltat); /* randWalkStddev (:337-340) */
        }
    }
    const double lambda = csum * pb->Lx * pb->Ly * pb->Lz / 1e12;
    const float hlx = 0.5f * (float)pb->Lx, hly = 0.5f * (float)pb->Ly, hlz = 0.5f * (float)pb->Lz;
    const float hax = 0.5f * (float)pb->ax, hay = 0.5f * (float)pb->ay;
    const float azf = (float)th[c->oaz];
    const float haz = (c->gen == 0 && pb->full_az_prior && !lognormal) ? azf : 0.5f * azf;
    const float four_dt = 4.0f * (float)pb->deltat, dde = (float)(pb->ub_de / pb->B);
    for (uint32_t v = 0; v < pb->V; ++v) {
        /* rand_poisson.jl: exponential gaps */
        int64_t np = 0;
        double t = 0.0;
        while (t < lambda) {
            ++np;
            t += -log(1.0 - rn_u(r));
        }
        np -= 1;
        const uint32_t F = pb->frames[v];
        for (int64_t p = 0; p < np; ++p) {
            float x = hlx * (2.0f * (float)rn_u(r) - 1.0f);
            float y = hly * (2.0f * (float)rn_u(r) - 1.0f);
            float z = hlz * (2.0f * (float)rn_u(r) - 1.0f);
            const float u = (float)rn_u(r);
            uint32_t idx = 0;
            while (idx + 1 < C && pre[idx] <= u) ++idx;
            const float sd = lognormal ? (float)(g * exp(-0.5 * (mul[idx] + sl[idx] * rn_n(r)))) : sd_fixed[idx];
            float de = 0.0f;
            uint32_t k = (fabsf(z) <= haz && fabsf(x) <= hax && fabsf(y) <= hay) ? 1u : 0u;
            for (uint32_t f = 1; f < F; ++f) {
                const float dx = sd * (float)rn_n(r), dy = sd * (float)rn_n(r), dz = sd * (float)rn_n(r);
                x = x + dx;
                if (fabsf(x) > hlx) x -= copysignf(2.0f * hlx, x);
                y = y + dy;
                if (fabsf(y) > hly) y -= copysignf(2.0f * hly, y);
                z = z + dz;
                if (fabsf(z) > hlz) z -= copysignf(2.0f * hlz, z);
                if (fabsf(z) <= haz && fabsf(x) <= hax && fabsf(y) <= hay) {
                    ++k;
                    if (k >= 2) de = de + (dx * dx + dy * dy);
                } else {
                    if (k >= pb->kmin) {
                        const float DE = de / ((float)(k - 1) * four_dt);
                        const float q = DE / dde;
                        if (q >= 0.0f && q < (float)pb->B) hist[(size_t)k * pb->B + (uint32_t)q] += 1u;
                    }
                    k = 0;
                    de = 0.0f;
                }
            }
            if (k >= pb->kmin) {
                const float DE = de / ((float)(k - 1) * four_dt);
                const float q = DE / dde;
                if (q >= 0.0f && q < (float)pb->B) hist[(size_t)k * pb->B + (uint32_t)q] += 1u;
            }
        }
    }
    const float d = orc_distance_kdist(hist, pb->ref_sat, pb->R, pb->B, NULL, NULL, NULL);
    return log10((double)d);
}

static void propose(const ctx_t* c, rng* r, double* th)
{
    const uint32_t P = c->P, N = c->pb->N, C = c->pb->C;
    if (c->gen == 0) return; /* prior pass: the slot's own parameters (caller copies) */
    /* wrand_idx_: lower_bound on cumulative weights */
    const double u = rn_u(r);
    uint32_t lo = 0, hi = N;
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (c->wcum[mid] < u)
            lo = mid + 1;
        else
            hi = mid;
    }
    const uint32_t parent = lo < N ? lo : N - 1;
    for (uint32_t p = 0; p < P; ++p) {
        if (c->lo[p] == c->hi[p]) {
            th[p] = c->lo[p];
            continue;
        }
        th[p] = orc_displace(c->theta[(size_t)parent * P + p], c->tau[p] * rn_n(r), c->lo[p], c->hi[p]);
    }
    /* sort components by m, their other per-component parameters with them */
    const uint32_t groups = c->oc / C + 1;
    for (uint32_t i = 1; i < C; ++i)
        for (uint32_t x = i; x > 0 && th[x] < th[x - 1]; --x)
            for (uint32_t g = 0; g < groups; ++g) {
                double t = th[g * C + x];
                th[g * C + x] = th[g * C + x - 1];
                th[g * C + x - 1] = t;
            }
}

static void* slot_worker(void* arg)
{
    ctx_t* c = (ctx_t*)arg;
    const orc_abc_problem* pb = c->pb;
    uint32_t* hist = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)pb->R * pb->B);
    const uint32_t P = c->P;
    for (;;) {
        const uint32_t s = atomic_fetch_add(&c->next, 1u);
        if (s >= pb->N) break;
        rng r;
        rn_seed(&r, c->seed, c->gen, s);
        double th[OP_MAXP];
        for (uint32_t t = 0;; ++t) {
            if (c->gen == 0)
                memcpy(th, c->theta + (size_t)s * P, sizeof(double) * P);
            else
                propose(c, &r, th);
            const double d = simulate_distance(c, th, &r, hist);
            atomic_fetch_add(&c->trials, 1ull);
            const uint64_t gt = atomic_fetch_add(&c->gen_trials, 1ull) + 1ull;
            if (c->gen == 0 || d <= c->gamma || t > 200000 || (c->trial_cap && gt >= c->trial_cap)) {
                memcpy(c->theta_new + (size_t)s * P, th, sizeof(double) * P);
                c->dist_new[s] = d;
                break;
            }
        }
    }
    free(hist);
    return NULL;
}

static int cmp_d(const void* a, const void* b)
{
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

static double quantile_of(const double* d, uint32_t N, double q)
{
    double* t = (double*)malloc(sizeof(double) * N);
    memcpy(t, d, sizeof(double) * N);
    qsort(t, N, sizeof(double), cmp_d);
    uint32_t k = (uint32_t)floor(q * N);
    if (k > N - 1) k = N - 1;
    double v = t[k];
    free(t);
    return v;
}

/* Runs the estimation; theta_out [N * P] (layout m | s | log10c | az for
 * the lognormal model, m | log10c | az for the discrete one), w_out [N].
 * Returns the total number of trials. */
uint64_t orc_abc_pmc(const orc_abc_problem* pb, uint64_t seed, uint32_t nthreads, double* theta_out,
                     double* w_out, uint32_t* generations_out, int* converged_out)
{
    ctx_t c;
    memset(&c, 0, sizeof c);
    c.pb = pb;
    const int lognormal = pb->model == ORC_MODEL_LOGNORMAL;
    const uint32_t C = pb->C, N = pb->N, P = (lognormal ? 3 : 2) * C + 1;
    if (P > OP_MAXP || C > ORC_MAX_COMPONENTS) return 0;
    c.P = P;
    c.seed = seed;
    c.oc = lognormal ? 2 * C : C;
    c.oaz = c.oc + C;
    for (uint32_t i = 0; i < C; ++i) {
        c.lo[i] = pb->lb_m;
        c.hi[i] = pb->ub_m;
        if (lognormal) {
            c.lo[C + i] = pb->lb_s;
            c.hi[C + i] = pb->ub_s;
        }
        c.lo[c.oc + i] = log10(pb->lb_c);
        c.hi[c.oc + i] = log10(pb->ub_c);
    }
    if (lognormal) {
        c.lo[c.oaz] = c.hi[c.oaz] = pb->az;
    } else {
        c.lo[c.oaz] = pb->lb_az;
        c.hi[c.oaz] = pb->ub_az;
    }
    c.theta = (double*)malloc(sizeof(double) * N * P);
    c.theta_new = (double*)malloc(sizeof(double) * N * P);
    c.w = (double*)malloc(sizeof(double) * N);
    c.wcum = (double*)malloc(sizeof(double) * N);
    c.dist = (double*)malloc(sizeof(double) * N);
    c.dist_new = (double*)malloc(sizeof(double) * N);
    rng r0;
    rn_seed(&r0, seed, 0xFFFFFFFFull, 0);
    for (uint32_t i = 0; i < N; ++i) {
        for (uint32_t p = 0; p < P; ++p) c.theta[(size_t)i * P + p] = c.lo[p] + (c.hi[p] - c.lo[p]) * rn_u(&r0);
        c.w[i] = 1.0 / N;
    }
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
    double* wstar = (double*)malloc(sizeof(double) * N);
    uint32_t committed = 0;
    int converged = 0;
    int fixed[OP_MAXP] = {0};
    for (uint32_t p = 0; p < P; ++p) fixed[p] = c.lo[p] == c.hi[p];
    for (uint32_t gen = 0; gen <= pb->generations; ++gen) {
        c.gen = gen;
        if (gen > 0 && pb->schedule == 0) c.gamma -= pb->delta_gamma;
        c.trial_cap = (gen > 0 && pb->avg_trials) ? (uint64_t)pb->avg_trials * N : 0ull;
        atomic_store(&c.gen_trials, 0ull);
        /* tau from the current population (compute_tau_) */
        for (uint32_t p = 0; p < P; ++p) c.tau[p] = sqrt(2.0 * orc_var_uncorrected(c.theta + p, N, P));
        double acc = 0.0;
        for (uint32_t i = 0; i < N; ++i) {
            acc += c.w[i];
            c.wcum[i] = acc;
        }
        atomic_store(&c.next, 0u);
        for (uint32_t t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, slot_worker, &c);
        for (uint32_t t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
        if (c.trial_cap && atomic_load(&c.gen_trials) >= c.trial_cap) {
            converged = 1; /* the generation that reached the trial cap is discarded */
            break;
        }
        if (gen == 0) {
            memcpy(c.dist, c.dist_new, sizeof(double) * N);
        } else {
            /* pmc-standard weights (simulation_impl.inl:832-871), fixed parameters skipped */
            orc_weights_pmc_standard(c.theta_new, c.theta, c.w, c.tau, fixed, N, P, wstar);
            memcpy(c.w, wstar, sizeof(double) * N);
            memcpy(c.theta, c.theta_new, sizeof(double) * N * P);
            memcpy(c.dist, c.dist_new, sizeof(double) * N);
            committed += 1;
        }
        if (pb->schedule == 0) {
            if (gen == 0) c.gamma = quantile_of(c.dist, N, 0.5); /* rank N/2: the upper median */
        } else {
            c.gamma = quantile_of(c.dist, N, pb->quantile);
        }
        if (getenv("PCS_ORACLE_TRACE")) {
            double ess = 0.0, s2 = 0.0;
            for (uint32_t i = 0; i < N; ++i) s2 += c.w[i] * c.w[i];
            ess = 1.0 / s2;
            fprintf(stderr, "oracle abc: generation %u gamma %.4f trials %llu ess %.1f\n", gen, c.gamma,
                    (unsigned long long)atomic_load(&c.trials), ess);
        }
    }
    memcpy(theta_out, c.theta, sizeof(double) * N * P);
    memcpy(w_out, c.w, sizeof(double) * N);
    if (generations_out) *generations_out = committed;
    if (converged_out) *converged_out = converged;
    const uint64_t trials = atomic_load(&c.trials);
    free(th);
    free(wstar);
    free(c.theta);
    free(c.theta_new);
    free(c.w);
    free(c.wcum);
    free(c.dist);
    free(c.dist_new);
    return trials;
}
