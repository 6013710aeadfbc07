/*
 * pcs_common.h -- types and counter-based random streams shared by the host
 * engine and the sm_103a kernels.
 *
 * Layout in HBM (one GPU, everything device-resident for the life of a job):
 *   per job        JobDev descriptor, observed cumulative histogram (R x B,
 *                  row-major) and its column-major copy with the columns
 *                  interleaved in pairs (pcs_sat_t_index), frame counts [V],
 *                  population theta [N x P] f64, weights/cumulative weights
 *                  [N] f64, distances [N] f64, perturbation factor [P x P] f64,
 *                  slot bookkeeping [N] u32.
 *   per round      PropDev descriptors [M], proposed parameters [M x P] f64,
 *                  particle counts [M x V] u32, histograms (sum of R_j*B_j
 *                  over the round's proposals) u32, distances [M],
 *                  work-item -> proposal map.
 */
#ifndef PCS_COMMON_H
#define PCS_COMMON_H

#include <stdint.h>

#if defined(__CUDACC__)
#define PCS_HD __host__ __device__ __forceinline__
#else
#define PCS_HD inline
#endif

#define PCS_MAX_C 8           /* mixture components per job */
#define PCS_MAX_P 32          /* parameters per job: 3*C + Z for the lognormal model */
#define PCS_MAX_V 4096        /* videos per job */
#define PCS_WARP 32

/* models: the reference's two (shared/common.hpp:9-16) plus the per-particle
 * lognormal diameter model with Stokes-Einstein diffusivity */
enum pcs_model_e {
    PCS_DEV_MODEL_FIXED_Z = 0,
    PCS_DEV_MODEL_VARIABLE_Z = 1,
    PCS_DEV_MODEL_LOGNORMAL = 2
};

/* Stream tags (top byte of counter word 1): every random draw of a job is
 * Philox4x32-10(counter, key = job seed) with a counter that names what the
 * draw is for, so a draw depends only on (seed, generation, slot, trial,
 * particle, step) and never on how work is scheduled or batched. */
enum pcs_stream_e {
    PCS_STREAM_PARTICLE = 0x0u,  /* c0 particle, c1 block j (0 position, 1 size, 2+ steps) */
    PCS_STREAM_POISSON = 0x1u,   /* c0 video */
    PCS_STREAM_PERTURB = 0x2u,   /* c0 parameter pair */
    PCS_STREAM_PICK = 0x3u,      /* c0 0 */
    PCS_STREAM_PRIOR = 0x4u      /* c0 parameter pair */
};

/* ----------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11, "Parallel random      */
/* numbers: as easy as 1, 2, 3"): 10 rounds of the published S-box with    */
/* the published multipliers and Weyl key increments.                       */
/* ----------------------------------------------------------------------- */
struct pcs_u4 {
    uint32_t x, y, z, w;
};

PCS_HD void pcs_mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo)
{
#if defined(__CUDA_ARCH__)
    *hi = __umulhi(a, b);
    *lo = a * b;
#else
    uint64_t p = (uint64_t)a * b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
#endif
}

PCS_HD pcs_u4 pcs_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        pcs_mulhilo(0xD2511F53u, c0, &hi0, &lo0);
        pcs_mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    pcs_u4 o = {c0, c1, c2, c3};
    return o;
}

/* Every stream of the engine uses one fixed Philox key (so the ten round
 * keys are compile-time constants) and folds the job seed into counter words
 * 2 and 3 through two 32-bit masks from the splitmix64 finaliser of the seed.
 * Within a job the map (slot, generation|trial) -> counter is a bijection, so
 * no two draws of a job share a counter; jobs with different seeds get
 * unrelated masks. */
#define PCS_PHILOX_K0 0xA4093822u
#define PCS_PHILOX_K1 0x299F31D0u

PCS_HD void pcs_seed_masks(uint64_t seed, uint32_t* m0, uint32_t* m1)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    *m0 = (uint32_t)z;
    *m1 = (uint32_t)(z >> 32);
}

PCS_HD pcs_u4 pcs_draw(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t m0, uint32_t m1)
{
    return pcs_philox(c0, c1, c2 ^ m0, c3 ^ m1, PCS_PHILOX_K0, PCS_PHILOX_K1);
}

/* Draws of one particle's stream differ only in counter word 1 (the block):
 * word 0 (particle) and words 2, 3 (slot and generation|trial, masked) are
 * fixed.  pcs_philox_prepare runs, once per particle, the first round and
 * the halves of rounds 2 and 3 that depend on the fixed words only;
 * pcs_draw_pre(state, block) then finishes the ten rounds with 34 instead of
 * 40 multiply/xor steps.  The outputs equal pcs_draw's bit for bit. */
struct pcs_philox_pre {
    uint32_t p0;     /* round-1 word 0 without the block */
    uint32_t a3;     /* round-1 word 3 */
    uint32_t b1;     /* word 1 after Philox round 2 */
    uint32_t h3, l3; /* round-3 product of word 0 */
};

#define PCS_PHILOX_W0 0x9E3779B9u
#define PCS_PHILOX_W1 0xBB67AE85u

PCS_HD pcs_philox_pre pcs_philox_prepare(uint32_t c0, uint32_t c2, uint32_t c3, uint32_t m0, uint32_t m1)
{
    pcs_philox_pre s;
    uint32_t hi0, lo0, hi1, lo1;
    pcs_mulhilo(0xD2511F53u, c0, &hi0, &lo0);
    pcs_mulhilo(0xCD9E8D57u, c2 ^ m0, &hi1, &lo1);
    s.p0 = hi1 ^ PCS_PHILOX_K0;
    const uint32_t a1 = lo1, a2 = hi0 ^ (c3 ^ m1) ^ PCS_PHILOX_K1;
    s.a3 = lo0;
    uint32_t h2, l2;
    pcs_mulhilo(0xCD9E8D57u, a2, &h2, &l2);
    const uint32_t b0 = h2 ^ a1 ^ (PCS_PHILOX_K0 + PCS_PHILOX_W0);
    s.b1 = l2;
    pcs_mulhilo(0xD2511F53u, b0, &s.h3, &s.l3);
    return s;
}

PCS_HD pcs_u4 pcs_draw_pre(const pcs_philox_pre& s, uint32_t c1)
{
    uint32_t h, l;
    /* Philox round 2: only the product of word 0 depends on the block */
    pcs_mulhilo(0xD2511F53u, s.p0 ^ c1, &h, &l);
    const uint32_t b2 = h ^ s.a3 ^ (PCS_PHILOX_K1 + PCS_PHILOX_W1), b3 = l;
    /* round 3: the product of word 0 is fixed */
    pcs_mulhilo(0xCD9E8D57u, b2, &h, &l);
    uint32_t c0 = h ^ s.b1 ^ (PCS_PHILOX_K0 + 2u * PCS_PHILOX_W0);
    uint32_t cc1 = l;
    uint32_t c2 = s.h3 ^ b3 ^ (PCS_PHILOX_K1 + 2u * PCS_PHILOX_W1);
    uint32_t c3 = s.l3;
    uint32_t k0 = PCS_PHILOX_K0 + 3u * PCS_PHILOX_W0, k1 = PCS_PHILOX_K1 + 3u * PCS_PHILOX_W1;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 3; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        pcs_mulhilo(0xD2511F53u, c0, &hi0, &lo0);
        pcs_mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
        const uint32_t n0 = hi1 ^ cc1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        cc1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += PCS_PHILOX_W0;
        k1 += PCS_PHILOX_W1;
    }
    pcs_u4 o = {c0, cc1, c2, c3};
    return o;
}

/* counter word 3: generation (12 bits) and trial (20 bits); a job stops
 * before its generation counter would leave 12 bits */
#define PCS_MAX_GENERATION 4095u
PCS_HD uint32_t pcs_ctr_gen_trial(uint32_t gen, uint32_t trial)
{
    return (gen << 20) | (trial & 0xFFFFFu);
}

PCS_HD uint32_t pcs_ctr_tag(uint32_t tag, uint32_t j)
{
    return (tag << 28) | (j & 0x0FFFFFFFu);
}

/* 24-bit uniform in [0,1): exact float, as the parity fixtures use */
PCS_HD float pcs_u01_24(uint32_t r)
{
    return (float)(r >> 8) * (1.0f / 16777216.0f);
}

/* 53-bit uniform in [0,1) from two words */
PCS_HD double pcs_u01_53(uint32_t a, uint32_t b)
{
    uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)m * (1.0 / 9007199254740992.0);
}

/* ----------------------------------------------------------------------- */
/* Device-resident descriptors                                             */
/* ----------------------------------------------------------------------- */

/* Per-job constants read by the forward model and the distance kernel.
 * Float fields are formed on the host exactly as the reference forms its
 * SimulateSetup (detail/simulation_impl.inl:568-579): 0.5f * float(x). */
struct JobDev {
    float half_lx, half_ly, half_lz;
    float half_ax, half_ay;
    float four_delta_t;
    float dde;             /* float(double(ub_de) / B) */
    uint32_t kmin;
    uint32_t V, R, B;
    uint32_t model, C, Z, P;
    uint32_t seed_lo, seed_hi;
    uint32_t frames_max;
    uint32_t tmap_depth;   /* histograms the job's tensor map spans (0: no tensor map) */
    const uint32_t* frames;     /* [V] */
    const uint32_t* ref_sat;    /* [R*B] observed cumulative histogram */
    const uint32_t* ref_sat_t;  /* [B*R] column-major copy, pairs interleaved (pcs_sat_t_index) */
};

/* A TMA tensor map (CUtensorMap: 128 bytes, 64-byte aligned), stored as
 * plain words so device tables need no driver header.  The histogram map of
 * a job is three-dimensional -- B columns, R rows, histograms -- over a
 * histogram area whose proposals of that job start at multiples of R x B
 * words. */
struct alignas(64) TmapDev {
    uint64_t w[16];
};

/* Cell (row r, column b) of the column-major observed histogram of R rows
 * and B columns, with columns 2j and 2j+1 interleaved: pair j occupies words
 * [2jR, 2jR + 2R) as (r, 2j), (r, 2j+1) for r = 0..R-1, so one 8-byte load
 * per row serves two columns and 32 consecutive rows are one coalesced
 * 256-byte request.  An odd B's last column stands alone at [(B-1)R, BR). */
PCS_HD uint64_t pcs_sat_t_index(uint32_t r, uint32_t b, uint32_t R, uint32_t B)
{
    const uint64_t base = (uint64_t)(b & ~1u) * R;
    if ((b | 1u) < B) return base + 2ull * r + (b & 1u);
    return base + r;
}

/* Per-proposal forward-model arguments (the SimulateRun of one proposal,
 * detail/simulation_impl.inl:319-340) plus its place in the round. */
struct PropDev {
    uint32_t job;          /* index into the round's job table */
    uint32_t slot;         /* population slot the proposal is for */
    uint32_t trial;        /* trial ordinal of the slot in this generation */
    uint32_t gen;          /* generation */
    uint32_t total_particles;
    uint32_t item_begin;   /* first work item */
    uint32_t item_count;
    uint32_t hist_z;       /* this histogram's index along its job's tensor map (hist_off / (R x B)) */
    uint64_t hist_off;     /* offset of this proposal's R x B histogram (u32 words) */
    uint64_t counts_off;   /* offset of this proposal's [V] particle counts and [V+1] prefix */
    float half_az[PCS_MAX_C];
    float pre_comp_prob[PCS_MAX_C];
    float sd_scale[PCS_MAX_C]; /* discrete: float(sqrt(2 m dt)); lognormal: step sd at z = 0 */
    float sd_shape[PCS_MAX_C]; /* lognormal: -0.5 * sigma_ln; discrete: 0 */
};

#endif
