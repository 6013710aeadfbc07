/*
 * engine.h -- host runtime of the GB300 ABC-PMC engine (C++17).
 *
 * Replaces the reference's SimulationT orchestration
 * (src/gpu/simulation_impl.cuh:135-374, detail/simulation_impl.inl) with a
 * device-resident design: a job's population, weights and observed
 * histogram live in one device arena; the host only plans rounds, launches a
 * captured CUDA graph per round and reads a small status table back.
 */
#ifndef PCS_ENGINE_H
#define PCS_ENGINE_H

#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pcs.h"
#include "pcs_common.h"
#include "pcs_kernels.h"

namespace pcs {

/* Error carried to the C ABI as a status + message. */
struct Error : std::runtime_error {
    pcs_status status;
    Error(pcs_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void cuda_check(cudaError_t e, const char* what);
#define PCS_CUDA(x) ::pcs::cuda_check((x), #x)

/* device allocation owned by the engine */
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void alloc(size_t n);
    void release();
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct Tuning {
    uint32_t block = 256;
    uint32_t ppt = 1;
    uint32_t tile_rows = 0; /* 0: no shared-memory tile, warps take their own slices of the items */
    uint32_t aggregate = 0;
    uint32_t chunk = 256;
    uint32_t capacity = 2048;
    uint32_t max_spec = 4096;
    uint32_t use_graphs = 1;
    uint32_t plain_launch = 1; /* 1 reference geometry, 2 persistent grid */
    uint32_t round_fill = 0; /* particles a round is topped up to (0: none); set to one wave at open */
    uint32_t walk = 2; /* forward-model walk on Philox streams: 1 slab-split, 2 per step */
    uint32_t job_order = 2; /* capacity order among jobs: 1 admission, 2 least remaining work first */
};

struct Job;

/* Round buffers shared by all jobs of a round (sized by capacity). */
struct RoundBufs {
    uint32_t capacity = 0, items_cap = 0, v_max = 0, max_rows = 0, max_n = 0;
    uint64_t counts_cap = 0, hist_cap = 0, ystride = 0;
    DevBuf round, props, theta_prop, counts, item_prop, hist, dist32, dist64, jobs, pmc;
    DevBuf tmaps; /* [kMaxRoundJobs] TmapDev: each job's histogram tensor map over hist */
};

struct Ctx {
    int device = 0;
    int sm_count = 0;
    int inflight = 1;
    cudaStream_t stream = nullptr;
    Tuning tune;
    DevBuf err;              /* device error word */
    DevBuf sim_tasks;        /* slab-split task counter (u64, cumulative) */
    DevBuf logfact;          /* [kLogFactEntries] log(k!) from the host's lgamma */
    uint64_t sim_tasks_base = 0;
    uint32_t* h_err = nullptr;
    RoundBufs rb;
    JobPmcDev* h_status = nullptr; /* pinned mirror of the pmc table */
    RoundDev* h_round = nullptr;   /* pinned */
    cudaGraphExec_t graph = nullptr;
    bool graph_dirty = true;
    std::vector<Job*> table;       /* jobs in the round table (index = table slot) */
    std::deque<Job*> queue;        /* serve: submitted, not yet admitted */
    uint32_t rb_max_b_ = 0;        /* widest histogram row among admitted jobs */
    uint64_t mem_cap = 0;
    uint64_t mem_used = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_sim0 = nullptr, ev_sim1 = nullptr, ev_dist0 = nullptr, ev_dist1 = nullptr;
    cudaEvent_t ev_pmc0 = nullptr, ev_pmc1 = nullptr;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
    RoundDev* h_round_out = nullptr; /* pinned copy of the round counters */
    pcs_kernel_stats stats{};
    static const uint32_t kKernelsPerRound = 9;
    std::mutex mu;

    explicit Ctx(int dev, int inflight);
    ~Ctx();

    /* round machinery */
    void ensure_round_buffers(uint32_t v_max, uint32_t max_rows, uint32_t max_n, uint64_t rb_max);
    void upload_table();
    void enqueue_round();
    void run_round(double* ms_out);
    void admit(Job* j);
    void retire(Job* j);
    uint32_t sim_grid(uint32_t block, uint32_t ppt, bool agg, uint32_t tile_words, bool split = false) const;
    bool split_walk() const { return tune.walk == 1u; }
    uint64_t read_sim_tasks();
};

struct Job {
    Ctx* ctx = nullptr;
    pcs_params p{};
    double ax = 0, ay = 0, deltat = 0;
    std::vector<uint32_t> frames;
    std::vector<uint32_t> K;
    std::vector<double> DE;
    uint64_t seed = 0;
    uint32_t N = 0, P = 0, C = 0, Z = 0, V = 0, R = 0, B = 0;
    DevBuf arena;
    JobDev jd{};
    JobPmcDev pm{};        /* initial state uploaded at admission */
    JobPmcDev status{};    /* last status read back */
    int slot = -1;         /* index in the round table, -1 when not admitted */
    bool initialised = false;
    bool finished = false;
    bool in_serve = false;
    bool mem_counted = false; /* its arena is counted in the context's serve memory use */
    double device_ms = 0.0;
    std::chrono::steady_clock::time_point t_submit, t_done;

    Job(Ctx* c, const pcs_params& prm, const pcs_observed& obs, uint64_t sd);
    uint64_t arena_bytes() const;
    void build_device_state(); /* allocate arena, observed histogram, prior population */
    void output(double* m, double* s, double* c, double* az, double* dist, double* w) const;
    /* checkpoint.cpp: the job's state between rounds as a byte blob, and back */
    size_t checkpoint_bytes() const;
    void save_state(void* buf) const;
    void load_state(const void* buf, size_t bytes);
};

/* shared-memory histogram words for a tile of tile_rows rows of `bins` bins */
uint32_t tile_words_for(uint32_t tile_rows, uint32_t bins);

/* validates and normalises parameters; throws Error */
void validate(const pcs_params& p, const pcs_observed& o);

} // namespace pcs

struct pcs_ctx {
    std::unique_ptr<pcs::Ctx> impl;
};
struct pcs_job {
    std::unique_ptr<pcs::Job> impl;
};

#endif
