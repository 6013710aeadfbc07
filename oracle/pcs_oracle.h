/*
 * pcs_oracle.h -- CPU restatement of the reference's ABC-PMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests compare the CUDA implementation in
 * part_conc_spt_abc_gb300/csrc against this library: it is loaded by tests/,
 * by __graft_entry__.smoke() and by the cpu_baseline leg of bench.py, and by
 * nothing else.  The product never links, loads or calls it.
 *
 * Every function restates one piece of the reference and cites the file:line
 * it follows (paths relative to the reference project root):
 *
 *   forward model, GPU conventions  src/gpu/cusim/kernel-simulate.inl:113-185
 *                                   src/gpu/cusim/utility.inl:8-185
 *                                   src/gpu/cusim/histogram2d.inl:313-321
 *   observed cumulative histogram   src/gpu/detail/simulation_impl.inl:605-629
 *   cumulative distance             src/gpu/cusim/kernel-distance.inl:81-241
 *   PMC weights / tau / displace    src/gpu/detail/simulation_impl.inl:24-79,733-887
 *   forward model, Julia conventions src/cpu/simulate.jl:1-127, distance.jl:1-8
 *
 * Floating-point contract: compiled with -ffp-contract=off, every float
 * operation is one IEEE-754 round-to-nearest operation in source order, which
 * is what the reference's kernels compute when built without FMA contraction.
 * Parity is pinned by running the reference's own kernel source, compiled for
 * the host by oracle/build_ref.sh, on the same replayed draws
 * (tests/golden/make_golden.py); see oracle/ref_harness.cpp.
 */
#ifndef PCS_ORACLE_H
#define PCS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_COMPONENTS 8

enum {
    ORC_MODEL_DISCRETE_FIXED_Z = 0,    /* EModel::discreteFixedZ    (shared/common.hpp:11) */
    ORC_MODEL_DISCRETE_VARIABLE_Z = 1, /* EModel::discreteVariableZ (shared/common.hpp:12) */
    ORC_MODEL_LOGNORMAL = 2            /* per-particle lognormal diameter (the library's model layer) */
};

/* cusim::SimulateSetup (kernel-simulate.cuh:19-38) plus the recorder's bin
 * width (histogram2d.cuh HistogramRecorder). */
typedef struct orc_setup {
    uint32_t model;
    uint32_t component_count; /* C */
    uint32_t video_count;     /* V (jobCount) */
    uint32_t kmin;
    float four_delta_t;
    float half_lx, half_ly, half_lz;
    float half_ax, half_ay;
    float dde;        /* DE bin width, float(double(ub_de)/B) */
    uint32_t rows;    /* R = kmax + 1 */
    uint32_t de_bins; /* B */
} orc_setup;

/* cusim::SimulateRun (kernel-simulate.cuh:52-63). */
typedef struct orc_run {
    const uint32_t* frames;    /* [V] */
    const uint32_t* particles; /* [V] */
    float half_az[ORC_MAX_COMPONENTS];          /* [Z]; Z = 1 for the fixed-depth model */
    float pre_comp_prob[ORC_MAX_COMPONENTS];    /* [C] cumulative component probabilities */
    float rand_walk_stddev[ORC_MAX_COMPONENTS]; /* [C] discrete models */
    float ln_scale[ORC_MAX_COMPONENTS];         /* lognormal: sd = ln_scale * exp(ln_shape * z) */
    float ln_shape[ORC_MAX_COMPONENTS];
} orc_run;

/* Pre-generated draws.  Particle n of the flattened order (video-major, then
 * particle within the video) consumes uniforms[4n+0..2] for its position,
 * uniforms[4n+3] for its component (only when C > 1) and
 * normals[(n*normal_stride + s)*3 + 0..2] for walk step s (0-based). */
typedef struct orc_replay {
    const float* uniforms;
    const float* normals;
    uint32_t normal_stride;
    const float* sigmas; /* [n] per-particle step sd for the lognormal model, else NULL */
} orc_replay;

typedef struct orc_track_counts {
    uint64_t closed;   /* tracks with K >= kmin handed to the recorder */
    uint64_t recorded; /* of those, the ones whose DE bin was < B */
} orc_track_counts;

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers:
 * as easy as 1, 2, 3"). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Deterministic replay draws for parity fixtures (not the product's stream):
 * uniforms for particle n come from Philox(ctr = {n, 0, 0, 0xA5A5A5A5},
 * key = seed) as (r >> 8) * 2^-24; the normal for (n, step s, axis a) comes
 * from Philox(ctr = {n, 1 + 3s + a, 0, 0xA5A5A5A5}) as
 * float((sum_i (r_i >> 8) * 2^-24 - 2) * sqrt(3)) (scaled Irwin-Hall sum of
 * four uniforms: unit variance, exactly reproducible).  sigmas (nullable)
 * gets base_sigma * (0.5 + u) per particle with u from counter word 1 =
 * 0xFFFFFFFF. */
void orc_replay_draws(uint64_t seed, uint64_t n_particles, uint32_t stride, float* uniforms,
                      float* normals, float* sigmas, float base_sigma);

/* Forward model on replayed draws, GPU conventions, float.  Adds into hist
 * (R x B, row-major, not cleared). */
int orc_simulate_replay(const orc_setup* s, const orc_run* r, const orc_replay* rp,
                        uint32_t* hist, orc_track_counts* counts);

/* Forward model on the product's Philox streams (counter layout of
 * part_conc_spt_abc_gb300/csrc/pcs_common.h: particle n, block 0 position and
 * component, block 1 size, blocks 2+3g.. the normals of steps 4g+1..4g+4),
 * with the Box-Muller logarithm and sine/cosine evaluated in double.  The
 * uniforms equal the GPU's bit for bit; the normals differ from the GPU's
 * fast-math ones in the last bits, so histograms agree closely but not
 * exactly (used for statistical parity). */
int orc_simulate_philox(const orc_setup* s, const orc_run* r, uint64_t seed, uint32_t slot,
                        uint32_t trial, uint32_t generation, uint32_t* hist,
                        orc_track_counts* counts);

/* The same model with the slab-split walk (walk_split in pcs_oracle.c): z
 * walked per step, x and y drawn per group of four steps as their sum and,
 * only where a z of the group lies in the detection slab, as the individual
 * steps conditioned on that sum.  Same distribution of histograms as
 * orc_simulate_philox from different draws. */
int orc_simulate_philox_split(const orc_setup* s, const orc_run* r, uint64_t seed, uint32_t slot,
                              uint32_t trial, uint32_t generation, uint32_t* hist,
                              orc_track_counts* counts);

/* Observed-data cumulative histogram (simulation_impl.inl:605-629). */
int orc_observed_sat(const uint32_t* K, const double* DE, size_t n, uint32_t rows,
                     uint32_t bins, double ub_de, uint32_t* sat);

/* K_distance (kernel-distance.inl:81-241): in-order 2-D inclusive prefix sums
 * of hist and the float squared-difference sum in the kernel's reduction
 * order.  cum_out (nullable) receives the prefix sums; ssd_hi/lo receive the
 * exact integer sum of squared differences. */
float orc_distance_kdist(const uint32_t* hist, const uint32_t* ref_sat, uint32_t rows,
                         uint32_t bins, uint32_t* cum_out, uint64_t* ssd_hi,
                         uint64_t* ssd_lo);

/* Same reduction with a double accumulator (K_distance<double,unsigned>,
 * kernel-distance.cu:5-8). */
double orc_distance_kdist_f64(const uint32_t* hist, const uint32_t* ref_sat,
                              uint32_t rows, uint32_t bins);

/* Julia conventions (src/cpu/simulate.jl, distance.jl): box [0,L],
 * ceil() binning into 1..B, kmax rows, Float64.  Replay in double. */
typedef struct orc_replay_f64 {
    const double* uniforms; /* [n][4]: component, x, y, z (simulate.jl:62-68 draw order) */
    const double* normals;  /* [n][stride][3] */
    uint32_t normal_stride;
} orc_replay_f64;

int orc_simulate_julia(uint32_t C, const double* m, const double* c, double ax, double ay,
                       const double* az, double Lx, double Ly, double Lz,
                       const uint32_t* frames, const uint32_t* particles, uint32_t V,
                       double deltat, uint32_t kmin, uint32_t B, double ub_de,
                       const orc_replay_f64* rp, int64_t* H /* kmax x B, row-major */);
double orc_distance_julia(const int64_t* H, const int64_t* Hsim, uint32_t kmax, uint32_t B);
/* The Julia path's observed histogram (estimate.jl:32-40) and its 2-D
 * inclusive prefix sums: kmax x B, row K-1, bin ceil(DE / (ub_de/B)) - 1
 * for 1 <= ceil(..) <= B.  Returns -1 for a K outside 1..kmax. */
int orc_observed_sat_julia(const uint32_t* K, const double* DE, size_t n, uint32_t kmax, uint32_t B,
                           double ub_de, uint32_t* sat);

/* PMC pieces, Float64 (simulation_impl.inl:24-79,733-887). */
double orc_var_uncorrected(const double* x, size_t n, size_t stride);
double orc_normpdf(double x, double mu, double sigma);
double orc_displace(double current, double delta, double lower, double upper);
/* theta_star [N][P], theta [N][P], w [N], tau [P]; fixed[p] != 0 skips p. */
void orc_weights_pmc_standard(const double* theta_star, const double* theta, const double* w,
                              const double* tau, const int* fixed, size_t N, size_t P,
                              double* w_out);
void orc_weights_inv_dist_sq(const double* dist, size_t N, double* w_out);
/* Weighted covariance (weights w, normalised) and its lower Cholesky factor. */
int orc_weighted_cov_cholesky(const double* theta, const double* w, size_t N, size_t P,
                              double scale, double* cov, double* chol);

/* One ABC-PMC proposal (simulation_impl.inl:256-347) drawn from the
 * library's counter-based streams instead of the host std::mt19937:
 * weighted parent pick (wrand_idx_ :54-62) on stream PICK, reflected
 * Gaussian displacement of every free parameter (displace_ :64-79; the
 * normals by Box-Muller from stream PERTURB, one counter per parameter pair;
 * with a Cholesky factor, delta_p = sum_i<=p L[p][i] n_i), components sorted
 * by m (:276-303, s and az moving with them), 10^log10c, lambda = sum c x
 * volume factor (:305-306), one Poisson count per video (:310-317; stream
 * POISSON, inversion below 12, Hoermann's PTRS above), the float forward-
 * model arguments (:319-340).  Parameter layout [m | s (lognormal) | log10c
 * | az].  Generation 0 (the prior pass) takes the slot's own parameters. */
typedef struct orc_prop_job {
    uint32_t model, C, Z, P, N, V;
    uint32_t perturbation;      /* 0 diagonal tau, 1 lower Cholesky factor */
    uint32_t full_az_prior;     /* prior pass uses the full az as half depth */
    uint64_t seed;
    double lo[32], hi[32];
    double volume_factor;       /* Lx Ly Lz / 1e12 */
    double delta_t;             /* discrete: step sd = sqrt(2 m dt) */
    double sd_const;            /* lognormal: step sd = sd_const exp(-mu_ln / 2) at z = 0 */
} orc_prop_job;

typedef struct orc_proposal {
    uint32_t parent;
    uint32_t total_particles;
    double lambda;
    float half_az[ORC_MAX_COMPONENTS];
    float pre_comp_prob[ORC_MAX_COMPONENTS];
    float sd_scale[ORC_MAX_COMPONENTS];
    float sd_shape[ORC_MAX_COMPONENTS];
} orc_proposal;

/* theta [N][P] committed population, wcum [N] cumulative weights, factor
 * [P][P]; writes theta_out [P] and counts [V]. */
int orc_build_proposal(const orc_prop_job* j, const double* theta, const double* wcum, const double* factor,
                       uint32_t slot, uint32_t trial, uint32_t generation, double* theta_out,
                       uint32_t* counts, orc_proposal* out);

/* CPU baseline: the Julia forward model (src/cpu/simulate.jl) in Float64,
 * timed over many proposals on nthreads host threads (cpu_baseline.c). */
typedef struct orc_cpu_job {
    uint32_t C;
    int32_t lognormal;
    double m[ORC_MAX_COMPONENTS]; /* discrete: D [um^2/s]; lognormal: mean diameter [nm] */
    double s[ORC_MAX_COMPONENTS]; /* lognormal: diameter sd [nm] */
    double c[ORC_MAX_COMPONENTS]; /* concentration [particles/ml] */
    double az[ORC_MAX_COMPONENTS];
    double temperature, viscosity;
    double ax, ay, Lx, Ly, Lz, deltat, ub_de;
    uint32_t kmin, B, V;
    const uint32_t* frames;
} orc_cpu_job;

uint64_t orc_cpu_forward_batch(const orc_cpu_job* jobs, uint32_t n_jobs, uint32_t nthreads,
                               uint64_t seed, double* seconds, uint64_t* checksum);

/* An independent CPU run of a whole ABC-PMC estimation (abc_oracle.c),
 * pmc-standard weights.  Models: lognormal diameters (model 2; parameters
 * m | s | log10c | az, the depth fixed at az) or the reference's discrete
 * diffusivities with one depth (model 0, discrete-fixed-depth; parameters
 * m | log10c | az, the depth drawn from [lb_az, ub_az]).  Schedules: the
 * q-quantile of the previous generation's distances (schedule 1), or the
 * reference's (schedule 0): gamma_0 = the distance of rank N/2 of the prior
 * pass, then gamma -= delta_gamma at the start of every generation.  With
 * avg_trials > 0, a generation whose trials reach avg_trials x N is
 * discarded and ends the run (converged). */
typedef struct orc_abc_problem {
    uint32_t C, N, generations, kmin, V, R, B;
    double quantile;
    double lb_m, ub_m, lb_s, ub_s, lb_c, ub_c; /* c in particles/ml */
    double az, Lx, Ly, Lz, ax, ay, deltat, ub_de, temperature, viscosity;
    const uint32_t* frames;  /* [V] */
    const uint32_t* ref_sat; /* [R*B] */
    uint32_t model, schedule, avg_trials, full_az_prior;
    double delta_gamma, lb_az, ub_az;
} orc_abc_problem;
/* theta_out [N * P], w_out [N]; *generations_out (nullable) receives the
 * generations committed after the prior pass and *converged_out (nullable)
 * whether the trial cap ended the run.  Returns the total trials. */
uint64_t orc_abc_pmc(const orc_abc_problem* pb, uint64_t seed, uint32_t nthreads, double* theta_out,
                     double* w_out, uint32_t* generations_out, int* converged_out);

#ifdef __cplusplus
}
#endif
#endif
