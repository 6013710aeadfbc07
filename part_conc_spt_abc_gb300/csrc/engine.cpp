/*
 * engine.cpp -- host runtime: contexts, jobs, batched rounds, serving.
 *
 * A round is a fixed sequence of kernels over every job in the context's
 * round table (plan -> propose -> items -> simulate -> distance -> accept ->
 * whiten -> kernel sum -> finalize) followed by a copy of the job status
 * table to pinned host memory.  The sequence is captured once into a CUDA
 * graph and replayed; all per-round variation (which jobs, how many
 * proposals, how many work items) is read by the kernels from device memory,
 * so the graph stays valid while jobs come and go.
 */
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace pcs {

void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        char buf[512];
        std::snprintf(buf, sizeof buf, "error::CudaError: %s (%s) from %s", cudaGetErrorString(e),
                      cudaGetErrorName(e), what);
        if (e == cudaErrorMemoryAllocation) throw Error(PCS_ERR_OUT_OF_MEMORY, buf);
        throw Error(PCS_ERR_CUDA, buf);
    }
}

void DevBuf::alloc(size_t n)
{
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
        p = nullptr;
        (void)cudaGetLastError();
        throw Error(PCS_ERR_OUT_OF_MEMORY, "device allocation of " + std::to_string(n) + " bytes failed");
    }
    bytes = n;
}

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

/* ======================================================================= */
/* validation                                                              */
/* ======================================================================= */

void validate(const pcs_params& p, const pcs_observed& o)
{
    auto bad = [](const std::string& m) { throw Error(PCS_ERR_INVALID_ARGUMENT, m); };
    if (p.model < 0 || p.model > 2) bad("unknown model " + std::to_string(p.model));
    if (p.weighting_scheme < 0 || p.weighting_scheme > 1) bad("unknown weighting scheme");
    if (p.component_count < 1 || p.component_count > PCS_MAX_C)
        bad("number_of_components must be in 1.." + std::to_string(PCS_MAX_C));
    if (p.abc_sample_count < 1) bad("number_of_abc_samples must be positive");
    if (p.de_bin_count < 1) bad("number_of_de_bins must be positive");
    if (!(p.ub_de > 0)) bad("ub_de must be positive");
    if (!(p.Lx > 0 && p.Ly > 0 && p.Lz > 0)) bad("box lengths must be positive");
    if (o.video_count < 1) bad("no videos (number_of_frames is empty)");
    if (o.video_count > PCS_MAX_V) bad("more than " + std::to_string(PCS_MAX_V) + " videos");
    if (!o.frame_counts) bad("frame_counts is NULL");
    if (o.track_count && (!o.K || !o.DE)) bad("K/DE are NULL");
    if (!(o.deltat > 0)) bad("deltat must be positive");
    for (size_t v = 0; v < o.video_count; ++v)
        if (o.frame_counts[v] < 1 || o.frame_counts[v] > 1000000) bad("frame counts must be in 1..1e6");
    auto chk = [&](double lo, double hi, const char* n) {
        if (!(lo <= hi)) bad(std::string("lower bound above upper bound for ") + n);
    };
    chk(p.lb_m, p.ub_m, "m");
    chk(p.lb_c, p.ub_c, "c");
    chk(p.lb_az, p.ub_az, "az");
    if (!(p.lb_c > 0)) bad("lb_c must be positive (sampled as log10)");
    if (p.model == PCS_MODEL_LOGNORMAL) {
        chk(p.lb_s, p.ub_s, "s");
        if (!(p.lb_m > 0)) bad("lognormal: lb_m (mean diameter) must be positive");
        if (!(p.lb_s >= 0)) bad("lognormal: lb_s must be non-negative");
        if (!(p.temperature > 0) || !(p.viscosity > 0)) bad("lognormal: temperature and viscosity must be positive");
    } else if (!(p.lb_m >= 0)) {
        bad("lb_m must be non-negative");
    }
    if (p.schedule == PCS_SCHEDULE_QUANTILE && !(p.quantile > 0 && p.quantile < 1)) bad("quantile must be in (0,1)");
    if (p.perturbation < 0 || p.perturbation > 1) bad("unknown perturbation");
}

/* ======================================================================= */
/* Job                                                                     */
/* ======================================================================= */

Job::Job(Ctx* c, const pcs_params& prm, const pcs_observed& obs, uint64_t sd) : ctx(c), p(prm), seed(sd)
{
    validate(prm, obs);
    ax = obs.ax;
    ay = obs.ay;
    deltat = obs.deltat;
    frames.resize(obs.video_count);
    uint32_t fmax = 0;
    for (size_t v = 0; v < obs.video_count; ++v) {
        frames[v] = (uint32_t)obs.frame_counts[v];
        fmax = std::max(fmax, frames[v]);
    }
    K.resize(obs.track_count);
    DE.assign(obs.DE, obs.DE + obs.track_count);
    C = p.component_count;
    Z = (p.model == PCS_MODEL_DISCRETE_VARIABLE_DEPTH) ? C : 1u;
    P = (p.model == PCS_MODEL_LOGNORMAL ? 3u : 2u) * C + Z;
    N = p.abc_sample_count;
    V = (uint32_t)obs.video_count;
    R = 1u + fmax; /* mKMax (detail/simulation_impl.inl:513) */
    B = p.de_bin_count;
    const double width = p.ub_de / (double)B;
    for (size_t i = 0; i < obs.track_count; ++i) {
        if (obs.K[i] >= R) throw Error(PCS_ERR_INVALID_ARGUMENT, "observed track length K=" + std::to_string(obs.K[i]) + " exceeds the longest video");
        K[i] = (uint32_t)obs.K[i];
        if (DE[i] < p.ub_de) {
            const long long flat = (long long)K[i] * B + (long long)(DE[i] / width);
            if (flat < 0 || (unsigned long long)flat >= (unsigned long long)R * B)
                throw Error(PCS_ERR_INVALID_ARGUMENT, "observed track outside the histogram (negative DE?)");
        }
    }
    if ((uint64_t)R * B > (1ull << 31)) throw Error(PCS_ERR_UNSUPPORTED, "histogram larger than 2^31 cells");
}

uint64_t Job::arena_bytes() const
{
    const uint64_t nP = (uint64_t)N * P;
    uint64_t b = 0;
    b += 2 * nP * 8;              /* theta, theta_new */
    b += 6 * (uint64_t)N * 8;     /* w, wcum, dist, dist_new, scratch (x2 for keep list) */
    b += (uint64_t)P * P * 8;     /* factor */
    b += 3 * (uint64_t)N * 4;     /* next_trial, pending, accepted */
    b += 2 * (uint64_t)R * B * 4; /* observed SAT + transpose */
    b += (uint64_t)V * 4;         /* frames */
    b += 2 * nP * 4;              /* whitened coordinates */
    b += 16 * 64;                 /* alignment slack */
    return b;
}

namespace {
template <class T>
T* carve(char*& cur, uint64_t n)
{
    uintptr_t u = reinterpret_cast<uintptr_t>(cur);
    u = (u + 255) & ~uintptr_t(255);
    T* r = reinterpret_cast<T*>(u);
    cur = reinterpret_cast<char*>(u + n * sizeof(T));
    return r;
}
} // namespace

void Job::build_device_state()
{
    if (initialised) return;
    arena.alloc(arena_bytes() + 4096);
    char* cur = arena.as<char>();
    const uint64_t nP = (uint64_t)N * P;
    double* d_theta = carve<double>(cur, nP);
    double* d_theta_new = carve<double>(cur, nP);
    double* d_w = carve<double>(cur, N);
    double* d_wcum = carve<double>(cur, N);
    double* d_dist = carve<double>(cur, N);
    double* d_dist_new = carve<double>(cur, N);
    double* d_scratch = carve<double>(cur, 2ull * N);
    double* d_factor = carve<double>(cur, (uint64_t)P * P);
    uint32_t* d_next = carve<uint32_t>(cur, N);
    uint32_t* d_pending = carve<uint32_t>(cur, N);
    uint32_t* d_acc = carve<uint32_t>(cur, N);
    uint32_t* d_sat = carve<uint32_t>(cur, (uint64_t)R * B);
    uint32_t* d_sat_t = carve<uint32_t>(cur, (uint64_t)R * B);
    uint32_t* d_frames = carve<uint32_t>(cur, V);
    float* d_y = carve<float>(cur, 2 * nP);
    if ((uint64_t)(cur - arena.as<char>()) > arena.bytes) throw Error(PCS_ERR_INVALID_ARGUMENT, "arena overflow");

    cudaStream_t st = ctx->stream;
    /* observed data -> cumulative histogram on the device */
    {
        DevBuf dK, dDE;
        dK.alloc(std::max<size_t>(K.size(), 1) * 4);
        dDE.alloc(std::max<size_t>(DE.size(), 1) * 8);
        if (!K.empty()) {
            PCS_CUDA(cudaMemcpyAsync(dK.p, K.data(), K.size() * 4, cudaMemcpyHostToDevice, st));
            PCS_CUDA(cudaMemcpyAsync(dDE.p, DE.data(), DE.size() * 8, cudaMemcpyHostToDevice, st));
        }
        PCS_CUDA(launch_observed_sat(dK.as<uint32_t>(), dDE.as<double>(), K.size(), R, B, p.ub_de, d_sat, d_sat_t,
                                     ctx->err.as<uint32_t>(), st));
        PCS_CUDA(cudaMemcpyAsync(d_frames, frames.data(), (size_t)V * 4, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaStreamSynchronize(st));
    }

    /* forward-model descriptor (SimulateSetup, simulation_impl.inl:568-579) */
    jd = JobDev{};
    jd.half_lx = 0.5f * (float)p.Lx;
    jd.half_ly = 0.5f * (float)p.Ly;
    jd.half_lz = 0.5f * (float)p.Lz;
    jd.half_ax = 0.5f * (float)ax;
    jd.half_ay = 0.5f * (float)ay;
    jd.four_delta_t = 4.0f * (float)deltat;
    jd.dde = (float)(p.ub_de / (double)B);
    jd.kmin = p.kmin;
    jd.V = V;
    jd.R = R;
    jd.B = B;
    jd.model = (uint32_t)p.model;
    jd.C = C;
    jd.Z = Z;
    jd.P = P;
    pcs_seed_masks(seed, &jd.seed_lo, &jd.seed_hi);
    jd.frames_max = R - 1;
    jd.frames = d_frames;
    jd.ref_sat = d_sat;
    jd.ref_sat_t = d_sat_t;

    /* PMC state */
    pm = JobPmcDev{};
    pm.N = N;
    pm.P = P;
    pm.C = C;
    pm.Z = Z;
    pm.V = V;
    pm.model = (uint32_t)p.model;
    pm.weighting = (uint32_t)p.weighting_scheme;
    pm.schedule = (uint32_t)p.schedule;
    pm.perturbation = (uint32_t)p.perturbation;
    pm.avg_trials = p.avg_trial_count;
    pm.quirk_full_az = (p.reference_initial_gamma && p.model != PCS_MODEL_LOGNORMAL) ? 1u : 0u;
    pm.max_generations = p.max_generations;
    pm.delta_t = deltat;
    pm.volume_factor = p.Lx * p.Ly * p.Lz / 1e12; /* :518 */
    pm.delta_gamma = p.delta_gamma;
    pm.quantile = p.quantile;
    if (p.model == PCS_MODEL_LOGNORMAL) {
        const double kB = 1.380649e-23;
        /* step sd [um] = sqrt(2 dt kB T 1e21 / (3 pi eta)) * d_nm^(-1/2) */
        pm.sd_const = std::sqrt(2.0 * deltat * kB * p.temperature * 1e21 / (3.0 * M_PI * p.viscosity));
    }
    /* parameter bounds, layout [m | s | log10c | az] */
    uint32_t at = 0;
    for (uint32_t i = 0; i < C; ++i, ++at) {
        pm.lo[at] = p.lb_m;
        pm.hi[at] = p.ub_m;
    }
    if (p.model == PCS_MODEL_LOGNORMAL)
        for (uint32_t i = 0; i < C; ++i, ++at) {
            pm.lo[at] = p.lb_s;
            pm.hi[at] = p.ub_s;
        }
    for (uint32_t i = 0; i < C; ++i, ++at) {
        pm.lo[at] = std::log10(p.lb_c); /* :523-524 */
        pm.hi[at] = std::log10(p.ub_c);
    }
    for (uint32_t i = 0; i < Z; ++i, ++at) {
        pm.lo[at] = p.lb_az;
        pm.hi[at] = p.ub_az;
    }
    for (uint32_t q = 0; q < P; ++q) pm.fixed[q] = (pm.lo[q] == pm.hi[q]) ? 1u : 0u;

    /* prior population: uniform draws on Philox stream PRIOR (prepare_ :530-537) */
    std::vector<double> theta(nP), w(N, 1.0 / N), wcum(N), factor((size_t)P * P, 0.0);
    for (uint32_t s = 0; s < N; ++s)
        for (uint32_t q = 0; q < P; q += 2) {
            pcs_u4 r = pcs_draw(q >> 1, pcs_ctr_tag(PCS_STREAM_PRIOR, 0u), s, pcs_ctr_gen_trial(0, 0),
                                  jd.seed_lo, jd.seed_hi);
            double u0 = pcs_u01_53(r.x, r.y), u1 = pcs_u01_53(r.z, r.w);
            theta[(uint64_t)s * P + q] = pm.lo[q] + (pm.hi[q] - pm.lo[q]) * u0;
            if (q + 1 < P) theta[(uint64_t)s * P + q + 1] = pm.lo[q + 1] + (pm.hi[q + 1] - pm.lo[q + 1]) * u1;
        }
    {
        double acc = 0.0;
        for (uint32_t i = 0; i < N; ++i) {
            acc += w[i];
            wcum[i] = acc;
        }
    }
    /* initial perturbation factor (compute_tau_ on the prior population) */
    if (p.perturbation == PCS_PERTURB_DIAGONAL) {
        for (uint32_t q = 0; q < P; ++q) {
            double s = 0, cnt = 0;
            for (uint32_t i = 0; i < N; ++i, cnt += 1) s += theta[(uint64_t)i * P + q];
            const double mean = s / cnt;
            double v = 0;
            for (uint32_t i = 0; i < N; ++i) {
                double x = theta[(uint64_t)i * P + q] - mean;
                v += x * x;
            }
            factor[(size_t)q * P + q] = std::sqrt(2.0 * (v / cnt));
        }
    } else {
        std::vector<double> mean(P, 0.0), cov((size_t)P * P, 0.0);
        for (uint32_t q = 0; q < P; ++q) {
            for (uint32_t i = 0; i < N; ++i) mean[q] += w[i] * theta[(uint64_t)i * P + q];
        }
        for (uint32_t a = 0; a < P; ++a)
            for (uint32_t b = 0; b < P; ++b) {
                double s = 0;
                for (uint32_t i = 0; i < N; ++i)
                    s += w[i] * (theta[(uint64_t)i * P + a] - mean[a]) * (theta[(uint64_t)i * P + b] - mean[b]);
                cov[(size_t)a * P + b] = 2.0 * s;
            }
        for (uint32_t c = 0; c < P; ++c) {
            if (pm.fixed[c]) continue;
            double d = cov[(size_t)c * P + c];
            for (uint32_t t = 0; t < c; ++t)
                if (!pm.fixed[t]) d -= factor[(size_t)c * P + t] * factor[(size_t)c * P + t];
            const double lv = std::sqrt(std::max(d, 1e-300));
            factor[(size_t)c * P + c] = lv;
            for (uint32_t r = c + 1; r < P; ++r) {
                if (pm.fixed[r]) continue;
                double s = cov[(size_t)r * P + c];
                for (uint32_t t = 0; t < c; ++t)
                    if (!pm.fixed[t]) s -= factor[(size_t)r * P + t] * factor[(size_t)c * P + t];
                factor[(size_t)r * P + c] = s / lv;
            }
        }
    }
    std::vector<uint32_t> pending(N), zeros(N, 0u);
    for (uint32_t i = 0; i < N; ++i) pending[i] = i;
    std::vector<double> zd(N, 0.0);
    PCS_CUDA(cudaMemcpyAsync(d_theta, theta.data(), nP * 8, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_theta_new, theta.data(), nP * 8, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_w, w.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_wcum, wcum.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_dist, zd.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_dist_new, zd.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_factor, factor.data(), (size_t)P * P * 8, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_next, zeros.data(), (size_t)N * 4, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_pending, pending.data(), (size_t)N * 4, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaMemcpyAsync(d_acc, zeros.data(), (size_t)N * 4, cudaMemcpyHostToDevice, st));
    PCS_CUDA(cudaStreamSynchronize(st));

    pm.theta = d_theta;
    pm.theta_new = d_theta_new;
    pm.w = d_w;
    pm.wcum = d_wcum;
    pm.dist = d_dist;
    pm.dist_new = d_dist_new;
    pm.factor = d_factor;
    pm.scratch = d_scratch;
    pm.next_trial = d_next;
    pm.pending = d_pending;
    pm.accepted = d_acc;
    pm.ybuf = d_y;
    pm.pending_count = N;
    pm.generation = 0u;
    pm.iterations = 0u;
    const bool prior_pass = p.gamma_adaptive || p.schedule == PCS_SCHEDULE_QUANTILE;
    if (prior_pass) {
        pm.gamma = -1.0;
    } else {
        /* first main iteration starts on the host (simulation_impl.inl:202-219) */
        pm.gamma = p.gamma_initial;
        pm.iterations = 1u;
        if (pm.max_generations && pm.iterations > pm.max_generations) {
            pm.done = 1u;
        } else {
            pm.gamma -= pm.delta_gamma;
            pm.generation = 1u;
        }
    }
    status = pm;
    initialised = true;
}

void Job::output(double* m, double* s, double* c, double* az, double* dist, double* w) const
{
    if (!initialised) throw Error(PCS_ERR_INVALID_ARGUMENT, "job has no device state yet");
    const uint64_t nP = (uint64_t)N * P;
    std::vector<double> theta(nP), hw(N), hd(N);
    PCS_CUDA(cudaMemcpy(theta.data(), pm.theta, nP * 8, cudaMemcpyDeviceToHost));
    PCS_CUDA(cudaMemcpy(hw.data(), pm.w, (size_t)N * 8, cudaMemcpyDeviceToHost));
    PCS_CUDA(cudaMemcpy(hd.data(), pm.dist, (size_t)N * 8, cudaMemcpyDeviceToHost));
    const uint32_t om = 0, os = C, oc = (p.model == PCS_MODEL_LOGNORMAL) ? 2 * C : C, oaz = oc + C;
    for (uint32_t i = 0; i < N; ++i) {
        const double* t = theta.data() + (uint64_t)i * P;
        for (uint32_t k = 0; k < C; ++k) {
            if (m) m[(uint64_t)i * C + k] = t[om + k];
            if (s) s[(uint64_t)i * C + k] = (p.model == PCS_MODEL_LOGNORMAL) ? t[os + k] : 0.0;
            if (c) c[(uint64_t)i * C + k] = std::pow(10.0, t[oc + k]);
        }
        for (uint32_t k = 0; k < Z; ++k)
            if (az) az[(uint64_t)i * Z + k] = t[oaz + k];
        if (dist) dist[i] = hd[i];
        if (w) w[i] = hw[i];
    }
}

/* ======================================================================= */
/* Ctx                                                                     */
/* ======================================================================= */

Ctx::Ctx(int dev, int infl) : device(dev), inflight(infl > 0 ? infl : 1)
{
    int n = 0;
    PCS_CUDA(cudaGetDeviceCount(&n));
    if (dev < 0 || dev >= n) throw Error(PCS_ERR_INVALID_ARGUMENT, "no CUDA device " + std::to_string(dev));
    PCS_CUDA(cudaSetDevice(dev));
    PCS_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
    tune.round_fill = (uint32_t)sm_count * 2048u; /* one full-occupancy wave of walkers */
    PCS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    err.alloc(16);
    sim_tasks.alloc(8);
    PCS_CUDA(cudaMemset(sim_tasks.p, 0, 8));
    PCS_CUDA(cudaMemset(err.p, 0, 16));
    {
        std::vector<double> lf(kLogFactEntries);
        for (uint32_t k = 0; k < kLogFactEntries; ++k) lf[k] = std::lgamma((double)k + 1.0);
        logfact.alloc(sizeof(double) * kLogFactEntries);
        PCS_CUDA(cudaMemcpy(logfact.p, lf.data(), sizeof(double) * kLogFactEntries, cudaMemcpyHostToDevice));
    }
    PCS_CUDA(cudaMallocHost((void**)&h_err, 16));
    PCS_CUDA(cudaMallocHost((void**)&h_status, sizeof(JobPmcDev) * kMaxRoundJobs));
    PCS_CUDA(cudaMallocHost((void**)&h_round, sizeof(RoundDev)));
    std::memset(h_status, 0, sizeof(JobPmcDev) * kMaxRoundJobs);
    std::memset(h_round, 0, sizeof(RoundDev));
    *h_err = 0;
    PCS_CUDA(cudaEventCreate(&ev0));
    PCS_CUDA(cudaEventCreate(&ev1));
    for (cudaEvent_t* e : {&ev_sim0, &ev_sim1, &ev_dist0, &ev_dist1, &ev_pmc0, &ev_pmc1, &ev_t0, &ev_t1}) PCS_CUDA(cudaEventCreate(e));
    PCS_CUDA(cudaMallocHost((void**)&h_round_out, sizeof(RoundDev)));
    std::memset(h_round_out, 0, sizeof(RoundDev));
}

Ctx::~Ctx()
{
    cudaSetDevice(device);
    if (graph) cudaGraphExecDestroy(graph);
    if (stream) cudaStreamSynchronize(stream);
    if (h_err) cudaFreeHost(h_err);
    if (h_status) cudaFreeHost(h_status);
    if (h_round) cudaFreeHost(h_round);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    for (cudaEvent_t e : {ev_sim0, ev_sim1, ev_dist0, ev_dist1, ev_pmc0, ev_pmc1, ev_t0, ev_t1})
        if (e) cudaEventDestroy(e);
    if (h_round_out) cudaFreeHost(h_round_out);
    if (stream) cudaStreamDestroy(stream);
}

uint32_t tile_words_for(uint32_t tile_rows, uint32_t bins)
{
    /* keep the privatised tile within 200 KB of shared memory, whole rows only */
    const uint32_t b = bins ? bins : 1u;
    const uint64_t cap_rows = (200ull * 1024ull / 4ull) / b;
    const uint64_t rows = std::min<uint64_t>(tile_rows, cap_rows);
    return (uint32_t)(rows * b);
}

uint64_t Ctx::read_sim_tasks()
{
    unsigned long long v = 0;
    PCS_CUDA(cudaStreamSynchronize(stream));
    PCS_CUDA(cudaMemcpy(&v, sim_tasks.p, 8, cudaMemcpyDeviceToHost));
    return (uint64_t)v;
}

uint32_t Ctx::sim_grid(uint32_t block, uint32_t ppt, bool agg, uint32_t tw, bool split) const
{
    SimLaunch l{0, block, (int)ppt, false, agg, split};
    int occ = simulate_occupancy(l, tw);
    if (occ < 1) occ = 1;
    return (uint32_t)(occ * sm_count);
}

void Ctx::ensure_round_buffers(uint32_t v_max, uint32_t max_rows, uint32_t max_n, uint64_t rb_max)
{
    const uint32_t cap = tune.capacity;
    uint64_t items_need = 0;
    for (Job* j : table)
        if (j) {
            /* particles per proposal are bounded by the prior's largest Poisson mean */
            const double lam = (double)j->C * j->p.ub_c * j->p.Lx * j->p.Ly * j->p.Lz / 1e12;
            const double per_video = lam + 12.0 * std::sqrt(lam) + 16.0;
            const double parts = per_video * j->V;
            items_need = std::max<uint64_t>(items_need, (uint64_t)std::ceil(parts / tune.chunk) + 1);
        }
    items_need = std::max<uint64_t>(items_need, 2) * cap;
    if (items_need > (1ull << 31)) items_need = 1ull << 31;
    /* each job's histograms start at a multiple of its R x B words: up to one
     * histogram of padding per job */
    const uint64_t hist_need = ((uint64_t)cap + kMaxRoundJobs) * rb_max;
    if (rb.capacity == cap && rb.v_max >= v_max && rb.max_rows >= max_rows && rb.max_n >= max_n &&
        rb.items_cap >= items_need && rb.hist_cap >= hist_need)
        return;
    PCS_CUDA(cudaStreamSynchronize(stream));
    rb.capacity = cap;
    rb.v_max = std::max(v_max, rb.v_max);
    rb.max_rows = std::max(max_rows, rb.max_rows);
    rb.max_n = std::max(max_n, rb.max_n);
    rb.items_cap = (uint32_t)std::max<uint64_t>(items_need, rb.items_cap);
    rb.counts_cap = (uint64_t)cap * (2ull * rb.v_max + 1ull);
    rb.hist_cap = std::max<uint64_t>(hist_need, rb.hist_cap);
    rb.round.alloc(sizeof(RoundDev));
    rb.props.alloc(sizeof(PropDev) * (size_t)cap);
    rb.theta_prop.alloc(sizeof(double) * (size_t)cap * PCS_MAX_P);
    rb.counts.alloc(sizeof(uint32_t) * rb.counts_cap);
    rb.item_prop.alloc(sizeof(uint32_t) * (size_t)rb.items_cap);
    rb.hist.alloc(sizeof(uint32_t) * rb.hist_cap);
    PCS_CUDA(cudaMemsetAsync(rb.hist.p, 0, sizeof(uint32_t) * rb.hist_cap, stream));
    rb.dist32.alloc(sizeof(float) * (size_t)cap);
    rb.dist64.alloc(sizeof(double) * (size_t)cap);
    if (!rb.jobs.p) {
        rb.tmaps.alloc(sizeof(TmapDev) * kMaxRoundJobs);
        PCS_CUDA(cudaMemsetAsync(rb.tmaps.p, 0, sizeof(TmapDev) * kMaxRoundJobs, stream));
        rb.jobs.alloc(sizeof(JobDev) * kMaxRoundJobs);
        rb.pmc.alloc(sizeof(JobPmcDev) * kMaxRoundJobs);
        PCS_CUDA(cudaMemsetAsync(rb.jobs.p, 0, sizeof(JobDev) * kMaxRoundJobs, stream));
        /* empty table slots read as finished jobs */
        std::vector<JobPmcDev> empty(kMaxRoundJobs);
        for (auto& e : empty) {
            std::memset(&e, 0, sizeof e);
            e.done = 1u;
        }
        PCS_CUDA(cudaMemcpyAsync(rb.pmc.p, empty.data(), sizeof(JobPmcDev) * kMaxRoundJobs, cudaMemcpyHostToDevice, stream));
        PCS_CUDA(cudaStreamSynchronize(stream));
    }
    graph_dirty = true;
}

void Ctx::upload_table()
{
    RoundDev& r = *h_round;
    std::memset(&r, 0, sizeof r);
    uint32_t n = 0;
    for (size_t i = 0; i < table.size(); ++i)
        if (table[i]) n = (uint32_t)i + 1;
    r.n_jobs = n;
    r.capacity = rb.capacity;
    r.max_spec = tune.max_spec;
    r.fill = tune.round_fill;
    r.order = tune.job_order == 2u ? 1u : 0u;
    r.chunk = tune.chunk;
    r.items_cap = rb.items_cap;
    r.counts_cap = rb.counts_cap;
    r.hist_cap = rb.hist_cap;
    r.v_max = rb.v_max;
    PCS_CUDA(cudaMemcpyAsync(rb.round.p, &r, sizeof r, cudaMemcpyHostToDevice, stream));
}

void Ctx::enqueue_round()
{
    PmcArgs a{};
    a.pmc = rb.pmc.as<JobPmcDev>();
    a.jobs = rb.jobs.as<JobDev>();
    a.round = rb.round.as<RoundDev>();
    a.props = rb.props.as<PropDev>();
    a.theta_prop = rb.theta_prop.as<double>();
    a.counts = rb.counts.as<uint32_t>();
    a.item_prop = rb.item_prop.as<uint32_t>();
    a.dist_f32 = rb.dist32.as<float>();
    a.dist_f64 = rb.dist64.as<double>();
    a.err = err.as<uint32_t>();
    a.logfact = logfact.as<double>();
    a.logfact_n = kLogFactEntries;
    a.use_f64_distance = 0u;
    for (Job* j : table)
        if (j && j->p.distance_double) a.use_f64_distance = 1u;

    PCS_CUDA(launch_round_plan(a, stream));
    PCS_CUDA(launch_propose(a, rb.capacity, stream));
    PCS_CUDA(launch_items(a, stream));

    SimArgs s{};
    RoundDev* rd = rb.round.as<RoundDev>();
    s.jobs = a.jobs;
    s.props = a.props;
    s.counts = a.counts;
    s.hist = rb.hist.as<uint32_t>();
    s.item_prop = a.item_prop;
    s.n_items = &rd->n_items;
    s.queue_head = &rd->queue_head;
    s.chunk = tune.chunk;
    s.tile_words = tile_words_for(tune.tile_rows, rb_max_b_);
    s.err = a.err;
    s.tasks = sim_tasks.as<unsigned long long>();
    SimLaunch l{};
    l.block = tune.block;
    l.ppt = (int)tune.ppt;
    l.replay = false;
    l.aggregate = tune.aggregate == 1u;
    l.split = split_walk();
    l.grid = sim_grid(l.block, tune.ppt, l.aggregate, s.tile_words, l.split);
    PCS_CUDA(cudaEventRecordWithFlags(ev_sim0, stream, cudaEventRecordExternal));
    PCS_CUDA(launch_simulate(s, l, stream));
    PCS_CUDA(cudaEventRecordWithFlags(ev_sim1, stream, cudaEventRecordExternal));

    DistArgs d{};
    d.jobs = a.jobs;
    d.props = a.props;
    d.n_props = &rd->n_props;
    d.hist = s.hist;
    d.cum_out = nullptr;
    d.dist_f32 = a.dist_f32;
    d.dist_f64 = a.use_f64_distance ? a.dist_f64 : nullptr;
    d.ssd = nullptr;
    d.err = a.err;
    d.max_rows = rb.max_rows;
    d.tmaps = rb.tmaps.as<TmapDev>();
    const uint32_t cl = d.dist_f64 ? 0u : distance_cluster_size(rb.max_rows, rb_max_b_);
    PCS_CUDA(cudaEventRecordWithFlags(ev_dist0, stream, cudaEventRecordExternal));
    PCS_CUDA(launch_distance(d, std::min<uint32_t>(rb.capacity, (uint32_t)(distance_ctas_per_sm(rb.max_rows) * sm_count)),
                             stream, cl));
    PCS_CUDA(cudaEventRecordWithFlags(ev_dist1, stream, cudaEventRecordExternal));

    PCS_CUDA(cudaEventRecordWithFlags(ev_pmc0, stream, cudaEventRecordExternal));
    PCS_CUDA(launch_accept(a, kMaxRoundJobs, stream));
    PCS_CUDA(launch_finalize(a, kMaxRoundJobs, rb.max_n, stream));
    PCS_CUDA(cudaEventRecordWithFlags(ev_pmc1, stream, cudaEventRecordExternal));
    PCS_CUDA(cudaMemcpyAsync(h_status, rb.pmc.p, sizeof(JobPmcDev) * kMaxRoundJobs, cudaMemcpyDeviceToHost, stream));
    PCS_CUDA(cudaMemcpyAsync(h_err, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    PCS_CUDA(cudaMemcpyAsync(h_round_out, rb.round.p, sizeof(RoundDev), cudaMemcpyDeviceToHost, stream));
}

void Ctx::run_round(double* ms_out)
{
    PCS_CUDA(cudaSetDevice(device));
    PCS_CUDA(cudaEventRecord(ev0, stream));
    if (tune.use_graphs) {
        if (graph_dirty || !graph) {
            if (graph) {
                cudaGraphExecDestroy(graph);
                graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            PCS_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue_round();
            } catch (...) {
                cudaStreamEndCapture(stream, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            PCS_CUDA(cudaStreamEndCapture(stream, &g));
            PCS_CUDA(cudaGraphInstantiate(&graph, g, 0));
            cudaGraphDestroy(g);
            graph_dirty = false;
        }
        PCS_CUDA(cudaGraphLaunch(graph, stream));
    } else {
        enqueue_round();
    }
    PCS_CUDA(cudaEventRecord(ev1, stream));
    PCS_CUDA(cudaStreamSynchronize(stream));
    float ms = 0.0f, sim_ms = 0.0f, dist_ms = 0.0f, pmc_ms = 0.0f;
    PCS_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    PCS_CUDA(cudaEventElapsedTime(&sim_ms, ev_sim0, ev_sim1));
    PCS_CUDA(cudaEventElapsedTime(&dist_ms, ev_dist0, ev_dist1));
    PCS_CUDA(cudaEventElapsedTime(&pmc_ms, ev_pmc0, ev_pmc1));
    if (ms_out) *ms_out = ms;
    stats.rounds += 1;
    stats.kernel_launches += kKernelsPerRound;
    stats.simulate_launches += 1;
    stats.simulate_ms += sim_ms;
    stats.distance_launches += 1;
    stats.distance_ms += dist_ms;
    stats.round_ms += ms;
    stats.pmc_launches += 1;
    stats.pmc_ms += pmc_ms;
    stats.proposals += h_round_out->n_props;
    stats.particle_steps += h_round_out->round_steps;
    stats.histogram_cells += h_round_out->round_cells;
    if (*h_err) {
        const uint32_t bits = *h_err;
        *h_err = 0;
        PCS_CUDA(cudaMemset(err.p, 0, 16));
        char buf[160];
        std::snprintf(buf, sizeof buf, "device error word 0x%x (1 hist bounds, 2 component, 4 items, 8 counts, 16 hist cap, 32 rows, 64 param, 128 copy wait)", bits);
        throw Error(PCS_ERR_DEVICE, buf);
    }
    for (size_t i = 0; i < table.size(); ++i)
        if (table[i]) {
            const JobPmcDev& was = table[i]->status;
            const JobPmcDev& now = h_status[i];
            if (now.iterations > was.iterations) {
                /* this round ended generation `was.generation` of the job */
                const uint64_t N = now.N, P = now.P;
                stats.generations += 1;
                stats.pmc_bytes += 2ull * N * P * 8ull + N * 8ull;
                if (was.generation > 0u && now.weighting == 0u && !now.converged)
                    stats.pmc_pair_flops += N * N * (6ull * P + 7ull);
            }
            table[i]->status = now;
            table[i]->device_ms += ms;
        }
}

void Ctx::admit(Job* j)
{
    if (j->slot >= 0) return;
    int slot = -1;
    for (size_t i = 0; i < table.size(); ++i)
        if (!table[i]) {
            slot = (int)i;
            break;
        }
    if (slot < 0) {
        if (table.size() >= kMaxRoundJobs) throw Error(PCS_ERR_BUSY, "round table full");
        table.push_back(nullptr);
        slot = (int)table.size() - 1;
    }
    j->build_device_state();
    table[slot] = j;
    j->slot = slot;
    uint32_t v_max = 0, max_rows = 0, max_n = 0, max_b = 0;
    uint64_t rb_max = 0;
    for (Job* t : table)
        if (t) {
            v_max = std::max(v_max, t->V);
            max_rows = std::max(max_rows, t->R);
            max_n = std::max(max_n, t->N);
            max_b = std::max(max_b, t->B);
            rb_max = std::max<uint64_t>(rb_max, (uint64_t)t->R * t->B);
        }
    if (max_b != rb_max_b_) {
        rb_max_b_ = max_b;
        graph_dirty = true;
    }
    ensure_round_buffers(v_max, max_rows, max_n, rb_max);
    /* every job's tensor map: the histogram area may have moved */
    std::vector<TmapDev> maps(table.size());
    for (size_t i = 0; i < table.size(); ++i) {
        Job* t = table[i];
        if (!t) continue;
        const uint64_t cells = (uint64_t)t->R * t->B;
        const uint64_t depth = cells ? rb.hist_cap / cells : 0u;
        t->jd.tmap_depth =
            encode_hist_tmap(&maps[i], rb.hist.as<uint32_t>(), t->R, t->B, depth) ? (uint32_t)depth : 0u;
        PCS_CUDA(cudaMemcpyAsync(rb.jobs.as<JobDev>() + i, &t->jd, sizeof(JobDev), cudaMemcpyHostToDevice, stream));
    }
    PCS_CUDA(cudaMemcpyAsync(rb.tmaps.p, maps.data(), sizeof(TmapDev) * maps.size(), cudaMemcpyHostToDevice, stream));
    PCS_CUDA(cudaMemcpyAsync(rb.pmc.as<JobPmcDev>() + slot, &j->status, sizeof(JobPmcDev), cudaMemcpyHostToDevice, stream));
    upload_table();
    PCS_CUDA(cudaStreamSynchronize(stream));
}

void Ctx::retire(Job* j)
{
    if (j->slot < 0) return;
    JobPmcDev empty;
    std::memset(&empty, 0, sizeof empty);
    empty.done = 1u;
    JobDev ej;
    std::memset(&ej, 0, sizeof ej);
    PCS_CUDA(cudaMemcpyAsync(rb.pmc.as<JobPmcDev>() + j->slot, &empty, sizeof empty, cudaMemcpyHostToDevice, stream));
    PCS_CUDA(cudaMemcpyAsync(rb.jobs.as<JobDev>() + j->slot, &ej, sizeof ej, cudaMemcpyHostToDevice, stream));
    table[j->slot] = nullptr;
    j->slot = -1;
    while (!table.empty() && !table.back()) table.pop_back();
    upload_table();
    PCS_CUDA(cudaStreamSynchronize(stream));
}

} // namespace pcs
