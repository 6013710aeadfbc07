/*
 * pcs.h -- C ABI of the GB300 ABC-PMC engine for nanoparticle size and
 * concentration estimation from single-particle tracking.
 *
 * This is the boundary the reference's hot path sits behind, flattened to
 * plain C: no exceptions cross it, every call returns a pcs_status (0 = OK)
 * and pcs_last_error() gives the message of the last failure on the calling
 * thread.  Buffers are owned by the caller unless stated otherwise; host
 * pointers are plain host memory (pageable or pinned).
 *
 * What each group replaces in the reference (paths relative to its root):
 *   pcs_open / pcs_close            the per-GPU setup in SimulationT::prepare_
 *                                   (src/gpu/detail/simulation_impl.inl:631-730)
 *   pcs_input_load, pcs_output_*    input::load (src/gpu/shared/input.cpp:101-235),
 *                                   output::write (src/gpu/shared/output.cpp:184-258)
 *   pcs_job_*                       make_simulation / Simulation::run / ::output
 *                                   (src/gpu/simulation.hpp:45-62)
 *   pcs_serve_*                     (no counterpart: continuous batching of jobs)
 *   pcs_simulate_hist               K_simulate_system[_unr] + HistogramRecorder
 *                                   (src/gpu/cusim/kernel-simulate.cuh:66-83,
 *                                    src/gpu/cusim/histogram2d.cuh:42-61)
 *   pcs_scan_distance               K_distance (src/gpu/cusim/kernel-distance.cuh:264-275)
 *   pcs_observed_sat                reference histogram construction
 *                                   (src/gpu/detail/simulation_impl.inl:605-629)
 */
#ifndef PCS_H
#define PCS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCS_ABI_VERSION 4
#define PCS_MAX_COMPONENTS 8

typedef enum pcs_status {
    PCS_OK = 0,
    PCS_ERR_INVALID_ARGUMENT = 1, /* bad sizes, null pointers, inconsistent parameters */
    PCS_ERR_CUDA = 2,             /* a CUDA runtime call failed (error::CudaError) */
    PCS_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed or admission refused */
    PCS_ERR_XML = 4,              /* input/data/output XML problem (error::XMLLoadError) */
    PCS_ERR_UNSUPPORTED = 5,      /* valid request this library does not implement */
    PCS_ERR_DEVICE = 6,           /* a kernel raised its error word (bounds or timeout) */
    PCS_ERR_BUSY = 7,             /* the object is in use by a running call */
    PCS_ERR_NOT_FOUND = 8         /* unknown job / no result yet */
} pcs_status;

typedef enum pcs_model {
    PCS_MODEL_DISCRETE_FIXED_DEPTH = 0,    /* "discrete-fixed-depth"    (EModel::discreteFixedZ) */
    PCS_MODEL_DISCRETE_VARIABLE_DEPTH = 1, /* "discrete-variable-depth" (EModel::discreteVariableZ) */
    PCS_MODEL_LOGNORMAL = 2                /* "lognormal": per-particle lognormal diameter */
} pcs_model;

typedef enum pcs_weighting {
    PCS_WEIGHTING_PMC_STANDARD = 0,    /* "pmc-standard" */
    PCS_WEIGHTING_INVERSE_DIST_SQ = 1  /* "inverse-distance-squared" */
} pcs_weighting;

typedef enum pcs_schedule {
    PCS_SCHEDULE_DELTA = 0,   /* reference: gamma -= delta_gamma each generation */
    PCS_SCHEDULE_QUANTILE = 1 /* epsilon = q-quantile of the previous generation's distances */
} pcs_schedule;

typedef enum pcs_perturbation {
    PCS_PERTURB_DIAGONAL = 0, /* reference: tau_p = sqrt(2 var_p), reflected per parameter */
    PCS_PERTURB_CHOLESKY = 1  /* 2 x weighted covariance, via its Cholesky factor */
} pcs_perturbation;

typedef struct pcs_ctx pcs_ctx;
typedef struct pcs_job pcs_job;

/* ------------------------------------------------------------------ */
/* Parameters and observed data (input::Parameters, shared/input.hpp:27-53) */
/* ------------------------------------------------------------------ */
typedef struct pcs_params {
    int32_t model;                 /* pcs_model */
    int32_t weighting_scheme;      /* pcs_weighting */
    uint32_t component_count;      /* number_of_components */
    uint32_t kmin;
    uint32_t de_bin_count;         /* number_of_de_bins */
    uint32_t abc_sample_count;     /* number_of_abc_samples (population N) */
    uint32_t avg_trial_count;      /* ub_average_number_of_trials */
    int32_t gamma_adaptive;
    double Lx, Ly, Lz;             /* sample box [um] */
    double gamma_initial, delta_gamma;
    double ub_de;                  /* DE histogram upper bound [um^2/s]; lower is 0 */
    double lb_m, ub_m;             /* discrete: diffusivity [um^2/s]; lognormal: mean diameter [nm] */
    double lb_s, ub_s;             /* lognormal only: diameter sd [nm] */
    double lb_c, ub_c;             /* concentration [particles/ml], sampled as log10 */
    double lb_az, ub_az;           /* detection depth [um] */
    double temperature;            /* lognormal only [K] */
    double viscosity;              /* lognormal only [Pa s] */
    /* schedule extensions (defaults reproduce the reference) */
    int32_t schedule;              /* pcs_schedule */
    int32_t perturbation;          /* pcs_perturbation */
    double quantile;               /* PCS_SCHEDULE_QUANTILE: q in (0,1) */
    uint32_t max_generations;      /* 0 = until convergence (reference -S semantics otherwise) */
    int32_t reference_initial_gamma; /* 1: prior pass uses full az as half depth (reference
                                        detail/simulation_impl.inl:782); discrete models only */
    int32_t distance_double;       /* accel -dt d: accumulate the distance in double
                                      (K_distance<double,unsigned>, kernel-distance.cu:5-8) */
} pcs_params;

typedef struct pcs_observed {
    double ax, ay;                 /* detection area [um] */
    double deltat;                 /* frame interval [s] */
    const uint64_t* frame_counts;  /* number_of_frames per video */
    size_t video_count;
    const uint64_t* K;             /* track lengths */
    const double* DE;              /* track diffusivity estimates [um^2/s] */
    size_t track_count;
} pcs_observed;

/* Fills *params with the reference's defaults for the schedule extensions. */
void pcs_params_defaults(pcs_params* params);

/* ------------------------------------------------------------------ */
/* Context                                                            */
/* ------------------------------------------------------------------ */
/* inflight: number of proposal batches kept in flight (the reference's
 * queue count in -g dev/queues); 0 picks the default. */
pcs_status pcs_open(int device, int inflight, pcs_ctx** out);
pcs_status pcs_close(pcs_ctx* ctx);
const char* pcs_last_error(void);
const char* pcs_status_string(pcs_status s);
int pcs_abi_version(void);
/* accel --list-devices text (sysinfo.cpp:8-40 with current device fields);
 * returns the length written (truncated to cap - 1). */
size_t pcs_device_report(char* buf, size_t cap);

/* Tuning knobs.  In pcs_set_tuning a field of 0 keeps the current /
 * autotuned value; PCS_TUNE_ZERO sets a field to 0 where 0 is meaningful
 * (hist_tile_rows, warp_aggregate, use_graphs, round_fill).  pcs_get_tuning reports
 * plain values. */
#define PCS_TUNE_ZERO 0xFFFFFFFFu
typedef struct pcs_tuning {
    uint32_t block_size;          /* forward-model threads per CTA */
    uint32_t particles_per_thread;/* independent walkers interleaved per thread: 1, 2, 4 or 8;
                                   * block_size is then at most 1024, 512, 256 or 256 */
    uint32_t hist_tile_rows;      /* histogram rows privatised in shared memory.  0 (default):
                                   * none; records are global atomics and each warp takes its
                                   * own 32-particle slices of the work items (no CTA barrier) */
    uint32_t warp_aggregate;      /* 1: warp-aggregated shared atomics, 0: plain */
    uint32_t chunk_particles;     /* particles per work item */
    uint32_t round_capacity;      /* proposals per batched round */
    uint32_t max_speculation;     /* max trials per slot per round */
    uint32_t use_graphs;          /* 1: capture rounds in CUDA graphs, 0: direct launches */
    uint32_t plain_launch;        /* pcs_job_run_plain's simulate launch: 1 the reference's
                                   * geometry (ceil(V/4) CTAs x 128 threads per proposal,
                                   * default), 2 the library's persistent grid */
    uint32_t round_fill;          /* a round whose proposals would carry fewer particles than
                                   * this (the end of a generation) gives its pending slots
                                   * proportionally more trials, up to the capacity.  Default:
                                   * one wave of the simulate launch (SMs x 2048 threads);
                                   * PCS_TUNE_ZERO: none */
    uint32_t walk;                /* forward-model walk on Philox streams: 2 per step (default),
                                   * 1 slab-split (z per step, x, y per group of four steps as
                                   * their sum and, near the detection slab, as the steps
                                   * conditioned on it).  Both draw histograms from the same
                                   * distribution, from different draws; the autotuner never
                                   * changes it.  Replayed draws always take the per-step walk. */
    uint32_t job_order;           /* which jobs take a round's capacity first when it is short:
                                   * 1 admission order, 2 (default) jobs in their prior pass,
                                   * then the least estimated remaining work first.  Results
                                   * do not depend on it; latencies do (64-job stream: p50
                                   * 27 s instead of 138 s, same throughput and p99). */
} pcs_tuning;
pcs_status pcs_get_tuning(pcs_ctx* ctx, pcs_tuning* out);
pcs_status pcs_set_tuning(pcs_ctx* ctx, const pcs_tuning* t);
/* Times the forward model over the tuning grid on a synthetic workload of
 * the given job shape and keeps the fastest setting. */
pcs_status pcs_autotune(pcs_ctx* ctx, const pcs_params* p, const pcs_observed* obs,
                        pcs_tuning* chosen);

/* Device timeline: events on the context's stream (spans host gaps too). */
pcs_status pcs_timer_start(pcs_ctx* ctx);
pcs_status pcs_timer_stop(pcs_ctx* ctx, double* elapsed_ms);

/* Per-kernel accounting of batched rounds, timed with CUDA events recorded
 * around the launches inside the round graph. */
typedef struct pcs_kernel_stats {
    uint64_t rounds;
    uint64_t kernel_launches;     /* all kernels of this library launched by rounds */
    uint64_t simulate_launches;
    double simulate_ms;           /* sum of forward-model launch durations */
    uint64_t distance_launches;
    double distance_ms;
    double round_ms;              /* sum of round durations */
    uint64_t proposals;           /* forward simulations */
    uint64_t particle_steps;      /* walk steps incl. initial placements */
    uint64_t histogram_cells;     /* R x B cells scanned by the distance kernel */
    uint64_t split_tasks;         /* slab-split walk: groups of four steps walked in x, y */
    /* the PMC step: accept, whiten, pairwise kernel sum, finalize (one timed
     * span per round; they do their generation-end work only in rounds that
     * end a job's generation) */
    uint64_t pmc_launches;        /* rounds whose PMC-step span was timed */
    double pmc_ms;                /* sum of the spans */
    uint64_t generations;         /* generations ended across jobs (prior pass included) */
    uint64_t pmc_bytes;           /* per ended generation: population read + write 2 x N x P x 8, weights N x 8 */
    uint64_t pmc_pair_flops;      /* pmc-standard kernel sum: N^2 x (6P + 7) per committed generation > 0 */
} pcs_kernel_stats;
pcs_status pcs_get_kernel_stats(pcs_ctx* ctx, pcs_kernel_stats* out);
pcs_status pcs_reset_kernel_stats(pcs_ctx* ctx);

/* ------------------------------------------------------------------ */
/* Estimation jobs (Simulation, src/gpu/simulation.hpp:45-62)           */
/* ------------------------------------------------------------------ */
pcs_status pcs_job_create(pcs_ctx* ctx, const pcs_params* p, const pcs_observed* obs,
                          uint64_t seed, pcs_job** out);
pcs_status pcs_job_destroy(pcs_job* job);
/* Runs to convergence, or for max_steps generations when max_steps > 0
 * (accel -S).  max_steps = 0 keeps the job's pcs_params.max_generations
 * (0 there too: no cap).  Blocking. */
pcs_status pcs_job_run(pcs_job* job, uint32_t max_steps);
/* The plain form: the reference's schedule (host-side PMC in double, one
 * proposal per simulate + distance launch, `queues` streams in flight, at most
 * one trial per population slot in flight; src/gpu/detail/simulation_impl.inl
 * :178-455) on this library's kernels.  For comparison with pcs_job_run. */
pcs_status pcs_job_run_plain(pcs_job* job, uint32_t max_steps, uint32_t queues);
/* Advances a job by one generation (batched rounds until every slot is
 * accepted or the trial cap is hit).  *done becomes 1 when it has finished. */
pcs_status pcs_job_step(pcs_job* job, int* done);

typedef struct pcs_job_info {
    uint32_t component_count, z_component_count, param_count, abc_sample_count;
    uint32_t iterations;          /* generations started (meta "iterations") */
    uint32_t converged;
    uint64_t simulations;         /* proposals simulated, speculative ones included */
    uint64_t trials;              /* trials counted the reference's way */
    uint64_t accepted;            /* accepted proposals */
    uint64_t particle_steps;      /* walk steps simulated (initial placements included) */
    double gamma;
    double device_ms;             /* GPU time spent in this job's rounds */
} pcs_job_info;
pcs_status pcs_job_info_get(pcs_job* job, pcs_job_info* out);

/* Population of the last completed generation (output::Output,
 * src/gpu/shared/output.hpp:16-34).  Arrays are caller-allocated:
 * m, c: [N*C] sample-major (all components of sample 0 first), as the
 * reference flattens them (detail/simulation_impl.inl:81-97); s: [N*C]
 * (lognormal only, may be NULL); az: [N*Z]; dist, w: [N].  c is written as
 * 10^log10c, like the reference. */
pcs_status pcs_job_output(pcs_job* job, double* m, double* s, double* c, double* az,
                          double* dist, double* w);

/* Checkpoint / resume (no counterpart in the reference).  Between any two
 * API calls a job's state is complete on the host side of a round; since
 * every draw is keyed by (seed, generation, slot, trial), a job restored from
 * a checkpoint continues exactly as the original would have.
 * pcs_job_checkpoint: with buf NULL, *bytes receives the size; otherwise the
 * state is written to buf (cap >= that size).  The job must have run at
 * least one round.  pcs_job_restore loads a checkpoint into a job that has
 * not run yet and was created with the same parameters shape (N, P, C, Z,
 * V, R, B, model), observed data and seed; its own max_generations applies
 * from then on.  Plain-form runs (pcs_job_run_plain) are not checkpointed. */
pcs_status pcs_job_checkpoint(pcs_job* job, void* buf, size_t cap, size_t* bytes);
pcs_status pcs_job_restore(pcs_job* job, const void* buf, size_t bytes);

/* ------------------------------------------------------------------ */
/* Serving: continuous batching of independent jobs                    */
/* ------------------------------------------------------------------ */
/* Queues a job.  Jobs are admitted as device memory allows and their
 * generations run interleaved in shared batched launches. */
pcs_status pcs_serve_submit(pcs_ctx* ctx, pcs_job* job);
/* Runs one batched round over the admitted jobs; returns the number of
 * jobs still queued or running in *active. */
pcs_status pcs_serve_step(pcs_ctx* ctx, uint32_t* active);
/* 1 in *finished once the job has completed. */
pcs_status pcs_serve_poll(pcs_ctx* ctx, pcs_job* job, int* finished);
/* Caps the device memory the serve loop may use (bytes, 0 = free memory):
 * a queued job is admitted while the admitted jobs' arenas, its own and the
 * round histograms (round capacity x the widest admitted job's R x B words)
 * fit; a job that does not fit even alone fails with PCS_ERR_OUT_OF_MEMORY. */
pcs_status pcs_serve_set_memory_cap(pcs_ctx* ctx, uint64_t bytes);

/* ------------------------------------------------------------------ */
/* XML boundary (accel's file formats)                                 */
/* ------------------------------------------------------------------ */
typedef struct pcs_input pcs_input;
/* input.xml + data.xml; data_path NULL uses <data_file_path> of the input. */
pcs_status pcs_input_load(const char* input_path, const char* data_path, pcs_input** out);
pcs_status pcs_input_free(pcs_input* in);
/* Views into the loaded input (valid until pcs_input_free). */
pcs_status pcs_input_params(const pcs_input* in, pcs_params* p, pcs_observed* obs,
                            const char** output_file_path);

typedef struct pcs_output_meta {
    const char* key;
    const char* value;
} pcs_output_meta;

/* output.xml in the reference's layout (src/gpu/shared/output.cpp:184-258). */
pcs_status pcs_output_write(const char* path, int32_t model, int32_t weighting,
                            uint64_t abc_sample_count, uint64_t component_count,
                            uint64_t z_component_count, const pcs_output_meta* meta,
                            size_t meta_count, int converged, double gamma,
                            const double* m, size_t nm, const double* s, size_t ns,
                            const double* c, size_t nc, const double* az, size_t naz,
                            const double* dist, size_t nd, const double* w, size_t nw);

typedef struct pcs_output pcs_output;
/* Reads an output.xml written by accel or by this library (the reference's
 * loader is a stub, src/gpu/shared/output.cpp:125-130). */
pcs_status pcs_output_load(const char* path, pcs_output** out);
pcs_status pcs_output_free(pcs_output* o);
typedef struct pcs_output_view {
    int32_t model, weighting;
    uint64_t abc_sample_count, component_count, z_component_count;
    int converged;
    double gamma;
    const double *m, *s, *c, *az, *dist, *w;
    size_t nm, ns, nc, naz, nd, nw;
    size_t meta_count;
    const pcs_output_meta* meta;
} pcs_output_view;
pcs_status pcs_output_get(const pcs_output* o, pcs_output_view* v);

/* ------------------------------------------------------------------ */
/* Hot-path entry points (parity and benchmarking)                     */
/* ------------------------------------------------------------------ */

/* One forward-model configuration: SimulateSetup + recorder
 * (src/gpu/cusim/kernel-simulate.cuh:13-38; float fields as the reference
 * forms them, detail/simulation_impl.inl:568-579). */
typedef struct pcs_setup {
    int32_t model;          /* pcs_model */
    uint32_t component_count;
    uint32_t video_count;
    uint32_t kmin;
    float four_delta_t;
    float half_lx, half_ly, half_lz;
    float half_ax, half_ay;
    float dde;              /* DE bin width */
    uint32_t rows;          /* R = kmax + 1 */
    uint32_t de_bins;       /* B */
    const uint32_t* frames; /* [video_count], host */
} pcs_setup;

/* One proposal: SimulateRun (kernel-simulate.cuh:46-63). */
typedef struct pcs_run {
    const uint32_t* particles;              /* [video_count], host */
    float half_az[PCS_MAX_COMPONENTS];      /* [Z] */
    float pre_comp_prob[PCS_MAX_COMPONENTS];/* [C], last entry above 1 */
    float sd_scale[PCS_MAX_COMPONENTS];     /* step sd (discrete) / step sd at z = 0 (lognormal) */
    float sd_shape[PCS_MAX_COMPONENTS];     /* lognormal: sd = scale * exp(shape * z) */
    uint32_t slot, trial, generation;       /* random-stream coordinates */
} pcs_run;

/* Pre-generated draws replacing the random streams (parity runs):
 * uniforms [n][4], normals [n][normal_stride][3], sigmas [n] (lognormal,
 * per-particle step sd) for the flattened particle order (video-major). */
typedef struct pcs_replay {
    const float* uniforms;
    const float* normals;
    uint32_t normal_stride;
    const float* sigmas;
} pcs_replay;

/* Forward model of `count` proposals sharing one setup; hist_out receives
 * count x R x B counts (host).  replay may be NULL (Philox streams keyed by
 * seed); with replay, count must be 1. */
pcs_status pcs_simulate_hist(pcs_ctx* ctx, const pcs_setup* setup, const pcs_run* runs,
                             uint32_t count, uint64_t seed, const pcs_replay* replay,
                             uint32_t* hist_out);

/* K_distance on `count` histograms against one observed cumulative
 * histogram (host buffers).  cum_out (nullable) receives the 2-D inclusive
 * prefix sums; dist_f32 the float sum of squared differences in the
 * reference kernel's reduction order; dist_f64 (nullable) the same in
 * double; ssd (nullable) the exact integer sum as [count][2] (hi, lo). */
pcs_status pcs_scan_distance(pcs_ctx* ctx, const uint32_t* hist, const uint32_t* ref_sat,
                             uint32_t rows, uint32_t bins, uint32_t count, uint32_t* cum_out,
                             float* dist_f32, double* dist_f64, uint64_t* ssd);

/* pcs_scan_distance for callers that cannot allocate device memory; this
 * entry point has no counterpart in the reference.  Hosts whose own caching
 * allocator owns all device memory, services under a fixed device-memory
 * budget, and real-time loops where an allocation could stall on device
 * synchronisation cannot let a library call cudaMalloc; this variant takes device pointers
 * and keeps its working buffers (a column-major copy of the observed histogram and one
 * descriptor per histogram) in a fixed __device__ array instead, calling no
 * allocator.  d_hist holds count x rows x bins counts and is reset to zero,
 * as K_distance resets its input; d_ref_sat is rows x bins; d_dist_f32 gets
 * count float distances in the reference kernel's reduction order.  Work is
 * queued on `stream` (a cudaStream_t, NULL = default stream) of the current
 * device, and the call waits for it: it reads the kernel's error word back
 * and returns PCS_ERR_DEVICE if the kernel raised it.  Limits: rows * bins <=
 * PCS_NOALLOC_MAX_CELLS and count <= PCS_NOALLOC_MAX_COUNT, else
 * PCS_ERR_INVALID_ARGUMENT.  The array (about 4.7 MiB) stays reserved on each
 * GPU that loads the library until exit.  The first call on a device looks
 * the array's address up (cudaGetSymbolAddress), so make it before any stream
 * capture; the address is kept for the process's life, so the entry point
 * does not survive cudaDeviceReset on that device.  All calls share the
 * array: calls whose work overlaps on the GPU race and must not be issued. */
#define PCS_NOALLOC_MAX_CELLS 1048576u
#define PCS_NOALLOC_MAX_COUNT 4096u
pcs_status pcs_scan_distance_noalloc(uint32_t* d_hist, const uint32_t* d_ref_sat, uint32_t rows,
                                     uint32_t bins, uint32_t count, float* d_dist_f32, void* stream);

/* Observed cumulative histogram from K / DE lists, on the device. */
pcs_status pcs_observed_sat(pcs_ctx* ctx, const uint32_t* K, const double* DE, size_t n,
                            uint32_t rows, uint32_t bins, double ub_de, uint32_t* sat_out);
/* The same in the Julia path's conventions (src/cpu/estimate.jl:32-40):
 * kmax x bins (row K-1 holds tracks of K frames, K = 1..kmax), DE binned by
 * ceil(DE / (ub_de / bins)) into 1..bins (so DE = 0 and DE > ub_de are
 * dropped), then the same 2-D inclusive prefix sums.  A K outside 1..kmax is
 * an error (Julia raises a bounds error). */
pcs_status pcs_observed_sat_julia(pcs_ctx* ctx, const uint32_t* K, const double* DE, size_t n,
                                  uint32_t kmax, uint32_t bins, double ub_de, uint32_t* sat_out);

/* Raw Philox words of one particle's stream block (checks the counter layout). */
pcs_status pcs_debug_particle_stream(pcs_ctx* ctx, uint64_t seed, uint32_t slot, uint32_t trial,
                                     uint32_t generation, uint32_t particle, uint32_t block,
                                     uint32_t out[4]);

/* The proposals of the context's last batched round that belong to `job`
 * (checks of the proposal construction, src/gpu/detail/simulation_impl.inl
 * :256-347, which the reference builds on the host per proposal): for each,
 * its slot, trial, generation, particle total, float forward-model
 * arguments and the float distance the round's distance kernel gave it
 * (K_distance's value), its parameter vector theta [n][P] (sample layout
 * [m | s (lognormal) | log10c | az]) and its particle counts [n][V].  They are
 * valid until the next round; the job must still be in the round table (not
 * retired).  With props NULL only *n is written. */
typedef struct pcs_debug_proposal {
    uint32_t slot, trial, generation, total_particles;
    float half_az[PCS_MAX_COMPONENTS];
    float pre_comp_prob[PCS_MAX_COMPONENTS];
    float sd_scale[PCS_MAX_COMPONENTS];
    float sd_shape[PCS_MAX_COMPONENTS];
    float distance;
} pcs_debug_proposal;
pcs_status pcs_debug_round_proposals(pcs_job* job, uint32_t cap, uint32_t* n, pcs_debug_proposal* props,
                                     double* theta, uint32_t* counts);

#ifdef __cplusplus
}
#endif
#endif
