/*
 * pcs_kernels.h -- launch interfaces of the sm_103a kernels (host side).
 */
#ifndef PCS_KERNELS_H
#define PCS_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "pcs_common.h"

/* bits of the device error word */
#define PCS_ERRBIT_HIST_BOUNDS 0x1u   /* a record fell outside R x B */
#define PCS_ERRBIT_COMPONENT 0x2u     /* component search ran past C */
#define PCS_ERRBIT_ITEMS 0x4u         /* work items exceeded capacity */
#define PCS_ERRBIT_COUNTS 0x8u        /* particle counts exceeded capacity */
#define PCS_ERRBIT_HISTCAP 0x10u      /* histogram capacity exceeded */
#define PCS_ERRBIT_ROWS 0x20u         /* distance kernel: rows exceed shared memory */
#define PCS_ERRBIT_PARAM 0x40u        /* non-finite parameter or weight */
#define PCS_ERRBIT_TIMEOUT 0x80u      /* distance kernel: a copy wait ran out */

namespace pcs {

/* ---------------- forward model (kernels_sim.cu) ---------------- */
struct SimArgs {
    const JobDev* jobs;
    const PropDev* props;
    const uint32_t* counts;    /* per proposal at counts_off: [V] counts, [V+1] prefix */
    uint32_t* hist;
    const uint32_t* item_prop; /* [items] proposal of each work item */
    const uint32_t* n_items;   /* device: number of items this round */
    uint32_t* queue_head;      /* device: next item (reset to 0 before the launch) */
    uint32_t chunk;            /* particles per item */
    uint32_t tile_words;       /* shared-memory histogram capacity (u32 words) */
    const float* rp_uniforms;  /* replay (single proposal) or NULL */
    const float* rp_normals;
    uint32_t rp_stride;
    const float* rp_sigmas;
    uint32_t* err;
    unsigned long long* tasks; /* nullable: slab-split walk task count (added to) */
};

struct SimLaunch {
    uint32_t grid, block;
    int ppt;
    bool replay;
    bool aggregate;
    bool split; /* slab-split walk (k_simulate_split: 256 threads, 1 particle each, no replay) */
};

cudaError_t launch_simulate(const SimArgs& a, const SimLaunch& l, cudaStream_t st);
/* largest CTA the forward model's build for `ppt` walkers per thread launches */
__host__ __device__ constexpr uint32_t sim_max_block(int ppt) { return ppt == 1 ? 1024u : (ppt == 2 ? 512u : 256u); }
int simulate_occupancy(const SimLaunch& l, uint32_t tile_words);
cudaError_t launch_debug_stream(uint64_t seed, uint32_t slot, uint32_t gen, uint32_t trial,
                                uint32_t particle, uint32_t block, uint32_t* d_out,
                                cudaStream_t st);

/* ---------------- scan + distance (kernels_dist.cu) ---------------- */
struct DistArgs {
    const JobDev* jobs;
    const PropDev* props;       /* hist_off, job */
    const uint32_t* n_props;    /* device: proposals this round */
    uint32_t* hist;             /* zeroed on return, as K_distance does */
    uint32_t* cum_out;          /* nullable: prefix sums at hist offsets */
    float* dist_f32;            /* [M] */
    double* dist_f64;           /* [M] nullable: double-accumulator distance */
    uint64_t* ssd;              /* [M][2] nullable: exact integer sum (hi, lo) */
    uint32_t* err;
    uint32_t max_rows;          /* rows of the carry array in shared memory */
    const TmapDev* tmaps;       /* nullable: per job (index of jobs), tensor maps over hist */
};
/* grid: CTAs at most (one histogram each).  cl > 1 (at least every job's
 * strips of 32 bins; 0 or 1: none) allows clusters of cl CTAs, one strip of
 * a histogram per CTA, which the launch takes where the histograms have at
 * least kClusterRowsMin rows or `grid` clusters fit at once; otherwise one
 * CTA walks each histogram's strips.  Variants with the double or integer
 * sums or the prefix-sum output take no clusters. */
cudaError_t launch_distance(const DistArgs& a, uint32_t grid, cudaStream_t st, uint32_t cl = 0u);
/* the cluster size for histograms of up to max_rows x max_bins, or 0 */
uint32_t distance_cluster_size(uint32_t max_rows, uint32_t max_bins);
const uint32_t kMaxDistCluster = 8u;
const uint32_t kClusterRowsMin = 512u;
/* Host: the tensor map of `depth` histograms of R x B u32 cells stored one
 * after another from `base` (boxes of 32 columns x 32 rows, 128-byte
 * swizzle).  False where the shape does not suit one (B a multiple of 4, R
 * and B at least 32) or the driver refuses it; the kernel then copies cell
 * by cell. */
bool encode_hist_tmap(TmapDev* out, const uint32_t* base, uint32_t R, uint32_t B, uint64_t depth);
size_t distance_smem_bytes(uint32_t max_rows, uint32_t cl = 0u);
uint32_t distance_block_threads(uint32_t max_rows);
int distance_ctas_per_sm(uint32_t max_rows, uint32_t cl = 0u);
const uint32_t kDistRowBlock = 256;

/* ---------------- ABC-PMC step (kernels_pmc.cu) ---------------- */

/* Per-job PMC state on the device. */
struct JobPmcDev {
    /* configuration */
    uint32_t N, P, C, Z, V, model, weighting, schedule, perturbation, avg_trials;
    uint32_t quirk_full_az;   /* prior pass uses az (not az/2) as half depth */
    uint32_t max_generations; /* 0 = no cap */
    double delta_t, volume_factor, delta_gamma, quantile, sd_const; /* sd_const: lognormal G */
    double lo[PCS_MAX_P], hi[PCS_MAX_P];
    uint32_t fixed[PCS_MAX_P]; /* lo == hi: not perturbed, not in the kernel density */
    /* state */
    double* theta;      /* [N*P] committed population */
    double* theta_new;  /* [N*P] accepted proposals of the running generation */
    double* w;          /* [N] */
    double* wcum;       /* [N] cumulative weights */
    double* dist;       /* [N] log10 distances of the committed population */
    double* dist_new;   /* [N] */
    double* factor;     /* [P*P] diag: tau on the diagonal; cholesky: lower factor */
    double* scratch;    /* [N] */
    uint32_t* next_trial; /* [N] */
    uint32_t* pending;    /* [N] compacted list of slots still searching */
    uint32_t* accepted;   /* [N] 1 once the slot accepted in this generation */
    float* ybuf;          /* [2*N*P] whitened coordinates for the kernel density */
    /* scalars (device-written) */
    double gamma;
    uint32_t generation;  /* 0 = prior pass */
    uint32_t pending_count;
    uint64_t trials;      /* semantic trials of the running generation */
    uint64_t simulations; /* all proposals simulated */
    uint64_t accepted_total;
    uint64_t accepted_gen;    /* accepted in the running generation */
    uint64_t particle_steps;
    uint32_t iterations;  /* reference "iterations" counter */
    uint32_t converged;
    uint32_t done;
    uint32_t gen_ended;   /* set by accept when the running generation ended this round */
    uint32_t status;      /* error bits */
};

/* One round's plan: which jobs take part and how. */
struct RoundDev {
    uint32_t n_jobs;
    uint32_t capacity;        /* max proposals */
    uint32_t max_spec;        /* max trials per slot */
    uint32_t chunk;           /* particles per item */
    uint32_t items_cap;
    uint64_t counts_cap;      /* u32 words */
    uint64_t hist_cap;        /* u32 words */
    uint32_t v_max;           /* counts stride = 2 * v_max + 1 per proposal */
    uint32_t fill;            /* particles a round is topped up to with extra trials (0: none) */
    /* device-written */
    uint32_t n_props;
    uint32_t n_items;
    uint32_t queue_head;
    uint32_t order;           /* capacity order: 0 admission, 1 least remaining work first */
    unsigned long long round_steps;  /* particle-steps of the round's proposals */
    unsigned long long round_cells;  /* histogram cells of the round's proposals */
    uint32_t job_base[64];    /* first proposal of each job */
    uint32_t job_k[64];       /* trials per pending slot */
    uint32_t job_count[64];   /* proposals of each job */
    uint64_t job_hist_base[64];/* first histogram word of each job */
};
const uint32_t kMaxRoundJobs = 64;

struct PmcArgs {
    JobPmcDev* pmc;           /* [n_jobs] */
    JobDev* jobs;             /* [n_jobs] forward-model descriptors */
    RoundDev* round;
    PropDev* props;           /* [capacity] */
    double* theta_prop;       /* [capacity * PCS_MAX_P] */
    uint32_t* counts;         /* counts + prefix area */
    uint32_t* item_prop;      /* [items_cap] */
    float* dist_f32;          /* [capacity] */
    double* dist_f64;         /* [capacity] nullable */
    uint32_t* err;
    uint32_t use_f64_distance;
    uint32_t logfact_n;       /* entries of logfact */
    const double* logfact;    /* nullable: log(k!) for k < logfact_n, for the Poisson sampler */
};

/* entries of the device log-factorial table (covers 1e5 particles per video) */
const uint32_t kLogFactEntries = 1u << 17;

cudaError_t launch_round_plan(const PmcArgs& a, cudaStream_t st);
cudaError_t launch_propose(const PmcArgs& a, uint32_t capacity, cudaStream_t st);
cudaError_t launch_items(const PmcArgs& a, cudaStream_t st);
cudaError_t launch_accept(const PmcArgs& a, uint32_t n_jobs, cudaStream_t st);
/* whiten + kernel sum + finalize */
cudaError_t launch_finalize(const PmcArgs& a, uint32_t n_jobs, uint32_t max_n, cudaStream_t st);

/* ---------------- observed data (kernels_pmc.cu) ---------------- */
cudaError_t launch_observed_sat(const uint32_t* K, const double* DE, size_t n, uint32_t rows,
                                uint32_t bins, double ub_de, uint32_t* sat, uint32_t* sat_t,
                                uint32_t* err, cudaStream_t st);
cudaError_t launch_observed_sat_julia(const uint32_t* K, const double* DE, size_t n, uint32_t kmax,
                                      uint32_t bins, double ub_de, uint32_t* sat, uint32_t* err, cudaStream_t st);

} // namespace pcs

#endif
