/*
 * cpu_baseline.c -- the reference's CPU path (Julia, src/cpu), restated in C
 * for timing on the host cores.
 *
 * TEST INFRASTRUCTURE ONLY: used as the cpu_baseline leg of bench.py and by
 * `bench.py --impl reference` (Julia 0.6 is not available on these machines).
 *
 * What is timed is the forward model of src/cpu/simulate.jl:1-127 in Float64
 * with the Julia conventions: box [0, L], position_periodic
 * (position_periodic.jl), ceil() DE bins, Poisson counts by the exponential
 * gap method (rand_poisson.jl), component by rand_weighted_index
 * (rand_weighted_index.jl), one proposal per worker at a time with dynamic
 * assignment of proposals to workers, like `@sync @parallel` over population
 * slots (estimate.jl:120).  Random numbers come from xoshiro256+ (Blackman
 * and Vigna) with polar-method normals (Marsaglia and Bray 1964) and
 * inversion exponentials; Julia uses MersenneTwister and a ziggurat, so the
 * streams differ and only the cost per particle-step is comparable.  The
 * lognormal diameter model (per-particle Stokes-Einstein diffusivity) is the
 * same model layer the GPU path adds.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "pcs_oracle.h"



typedef struct xs {
    uint64_t s[4];
} xs;

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xs_next(xs* r)
{
    uint64_t* s = r->s;
    uint64_t res = s[0] + s[3];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return res;
}

static inline double xs_rand(xs* r) { return (double)(xs_next(r) >> 11) * (1.0 / 9007199254740992.0); }

static void xs_seed(xs* r, uint64_t seed)
{
    /* splitmix64 */
    for (int i = 0; i < 4; ++i) {
        uint64_t z = (seed += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        r->s[i] = z ^ (z >> 31);
    }
}

typedef struct normal_gen {
    xs r;
    int have;
    double spare;
} normal_gen;

static inline double randn(normal_gen* g)
{
    if (g->have) {
        g->have = 0;
        return g->spare;
    }
    double u, v, q;
    do {
        u = 2.0 * xs_rand(&g->r) - 1.0;
        v = 2.0 * xs_rand(&g->r) - 1.0;
        q = u * u + v * v;
    } while (q >= 1.0 || q == 0.0);
    double f = sqrt(-2.0 * log(q) / q);
    g->spare = v * f;
    g->have = 1;
    return u * f;
}

static inline double randexp(normal_gen* g) { return -log(1.0 - xs_rand(&g->r)); }

static inline double position_periodic(double x, double L)
{
    if (x > L)
        x = x - L;
    else if (x < 0.0)
        x = x + L;
    return x;
}

/* one proposal (simulate.jl:1-127); returns particle-steps, fills H (kmax x B) */
static uint64_t simulate_one(const orc_cpu_job* j, normal_gen* g, int64_t* H, uint32_t kmax)
{
    double csum = 0.0, cum[ORC_MAX_COMPONENTS];
    for (uint32_t i = 0; i < j->C; ++i) csum += j->c[i];
    double acc = 0.0;
    for (uint32_t i = 0; i < j->C; ++i) {
        acc += j->c[i] / csum;
        cum[i] = acc;
    }
    const double lambda = csum * j->Lx * j->Ly * j->Lz / 1e12;
    const double d_de = j->ub_de / (double)j->B;
    const double kB = 1.380649e-23;
    double mul[ORC_MAX_COMPONENTS], sl[ORC_MAX_COMPONENTS];
    if (j->lognormal)
        for (uint32_t i = 0; i < j->C; ++i) {
            double s2 = log1p(j->s[i] * j->s[i] / (j->m[i] * j->m[i]));
            sl[i] = sqrt(s2);
            mul[i] = log(j->m[i]) - 0.5 * s2;
        }
    uint64_t steps = 0;
    for (uint32_t v = 0; v < j->V; ++v) {
        /* rand_poisson.jl */
        int64_t np = 0;
        double t = 0.0;
        while (t < lambda) {
            ++np;
            t += randexp(g);
        }
        np -= 1;
        const uint32_t F = j->frames[v];
        for (int64_t p = 0; p < np; ++p) {
            double val = xs_rand(&g->r);
            uint32_t idx = 0;
            while (idx + 1 < j->C && cum[idx] < val) ++idx;
            double D = j->m[idx];
            if (j->lognormal) {
                double d_nm = exp(mul[idx] + sl[idx] * randn(g));
                D = kB * j->temperature / (3.0 * M_PI * j->viscosity * d_nm * 1e-9) * 1e12;
            }
            const double sd = sqrt(2.0 * D * j->deltat);
            double x = j->Lx * xs_rand(&g->r), y = j->Ly * xs_rand(&g->r), z = j->Lz * xs_rand(&g->r);
            const double haz = 0.5 * j->az[j->lognormal ? 0 : idx];
            double de = 0.0;
            uint32_t k = (fabs(z - 0.5 * j->Lz) <= haz && fabs(x - 0.5 * j->Lx) <= 0.5 * j->ax &&
                          fabs(y - 0.5 * j->Ly) <= 0.5 * j->ay)
                             ? 1u
                             : 0u;
            for (uint32_t f = 2; f <= F; ++f) {
                double dx = sd * randn(g), dy = sd * randn(g), dz = sd * randn(g);
                x = position_periodic(x + dx, j->Lx);
                y = position_periodic(y + dy, j->Ly);
                z = position_periodic(z + dz, j->Lz);
                if (fabs(z - 0.5 * j->Lz) <= haz && fabs(x - 0.5 * j->Lx) <= 0.5 * j->ax &&
                    fabs(y - 0.5 * j->Ly) <= 0.5 * j->ay) {
                    ++k;
                    if (k >= 2) de += dx * dx + dy * dy;
                } else if (k > 0) {
                    if (k >= j->kmin && k >= 2) {
                        double DE = de / ((double)(k - 1) * 4.0 * j->deltat);
                        double q = ceil(DE / d_de);
                        if (q >= 1.0 && q <= (double)j->B && k <= kmax) H[(uint64_t)(k - 1) * j->B + (uint64_t)q - 1] += 1;
                    }
                    k = 0;
                    de = 0.0;
                }
            }
            if (k >= j->kmin && k >= 2) {
                double DE = de / ((double)(k - 1) * 4.0 * j->deltat);
                double q = ceil(DE / d_de);
                if (q >= 1.0 && q <= (double)j->B && k <= kmax) H[(uint64_t)(k - 1) * j->B + (uint64_t)q - 1] += 1;
            }
            steps += F;
        }
    }
    return steps;
}

typedef struct worker_arg {
    const orc_cpu_job* jobs;
    uint32_t n_jobs;
    atomic_uint* next;
    uint64_t seed;
    uint64_t steps;
    uint32_t kmax;
    int64_t* H;
    uint64_t checksum;
} worker_arg;

static void* worker(void* p)
{
    worker_arg* a = (worker_arg*)p;
    normal_gen g;
    memset(&g, 0, sizeof g);
    xs_seed(&g.r, a->seed);
    for (;;) {
        uint32_t i = atomic_fetch_add(a->next, 1u);
        if (i >= a->n_jobs) break;
        const orc_cpu_job* j = &a->jobs[i];
        memset(a->H, 0, sizeof(int64_t) * (uint64_t)a->kmax * j->B);
        a->steps += simulate_one(j, &g, a->H, a->kmax);
        for (uint64_t k = 0; k < (uint64_t)a->kmax * j->B; ++k) a->checksum += (uint64_t)a->H[k] * (k + 1);
    }
    return NULL;
}

/* Times n_jobs forward simulations on nthreads worker threads.  Returns the
 * total particle-steps; *seconds gets the wall time. */
uint64_t orc_cpu_forward_batch(const orc_cpu_job* jobs, uint32_t n_jobs, uint32_t nthreads, uint64_t seed,
                               double* seconds, uint64_t* checksum)
{
    if (nthreads < 1) nthreads = 1;
    uint32_t kmax = 1, bmax = 1;
    for (uint32_t i = 0; i < n_jobs; ++i) {
        for (uint32_t v = 0; v < jobs[i].V; ++v)
            if (jobs[i].frames[v] > kmax) kmax = jobs[i].frames[v];
        if (jobs[i].B > bmax) bmax = jobs[i].B;
    }
    pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
    worker_arg* args = (worker_arg*)calloc(nthreads, sizeof(worker_arg));
    atomic_uint next;
    atomic_init(&next, 0u);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (uint32_t t = 0; t < nthreads; ++t) {
        args[t].jobs = jobs;
        args[t].n_jobs = n_jobs;
        args[t].next = &next;
        args[t].seed = seed * 0x9E3779B97F4A7C15ull + t + 1;
        args[t].kmax = kmax;
        args[t].H = (int64_t*)calloc((uint64_t)kmax * bmax, sizeof(int64_t));
        pthread_create(&th[t], NULL, worker, &args[t]);
    }
    uint64_t steps = 0, cs = 0;
    for (uint32_t t = 0; t < nthreads; ++t) {
        pthread_join(th[t], NULL);
        steps += args[t].steps;
        cs += args[t].checksum;
        free(args[t].H);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (seconds) *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    if (checksum) *checksum = cs;
    free(th);
    free(args);
    return steps;
}
