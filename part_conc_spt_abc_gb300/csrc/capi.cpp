/*
 * capi.cpp -- the extern "C" boundary (include/pcs.h).
 *
 * The reference reports failures as C++ exceptions (error::RuntimeError and
 * error::CudaError, src/gpu/shared/errors.hpp:6-41, support/cuda_error.hpp);
 * here every entry point catches them, stores the message for
 * pcs_last_error() and returns a pcs_status.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"
#include "xml_io.h"

using namespace pcs;

namespace {

thread_local std::string g_last_error;

template <class F>
pcs_status guard(F&& f)
{
    try {
        f();
        g_last_error.clear();
        return PCS_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const XmlError& e) {
        g_last_error = e.what();
        return PCS_ERR_XML;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return PCS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return PCS_ERR_INVALID_ARGUMENT;
    }
}

void need(const void* p, const char* what)
{
    if (!p) throw Error(PCS_ERR_INVALID_ARGUMENT, std::string(what) + " is NULL");
}

Ctx& C_(pcs_ctx* c)
{
    need(c, "ctx");
    PCS_CUDA(cudaSetDevice(c->impl->device));
    return *c->impl;
}

Job& J_(pcs_job* j)
{
    need(j, "job");
    return *j->impl;
}

struct DevTmp {
    std::vector<DevBuf*> bufs;
    ~DevTmp()
    {
        for (auto* b : bufs) delete b;
    }
    template <class T>
    T* get(size_t n)
    {
        DevBuf* b = new DevBuf();
        bufs.push_back(b);
        b->alloc(std::max<size_t>(n, 1) * sizeof(T));
        return b->as<T>();
    }
};

void check_err_word(Ctx& c)
{
    uint32_t bits = 0;
    PCS_CUDA(cudaMemcpy(&bits, c.err.p, 4, cudaMemcpyDeviceToHost));
    if (bits) {
        PCS_CUDA(cudaMemset(c.err.p, 0, 16));
        throw Error(PCS_ERR_DEVICE, "device error word 0x" + std::to_string(bits));
    }
}

} // namespace

namespace pcs {
void set_last_error(const std::string& m) { g_last_error = m; }
} // namespace pcs

extern "C" {

int pcs_abi_version(void) { return PCS_ABI_VERSION; }

size_t pcs_device_report(char* buf, size_t cap)
{
    std::string out;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        (void)cudaGetLastError();
        n = 0;
    }
    char line[512];
    std::snprintf(line, sizeof line, "Found %d CUDA device(s)\n", n);
    out += line;
    for (int i = 0; i < n; ++i) {
        cudaDeviceProp p{};
        if (cudaGetDeviceProperties(&p, i) != cudaSuccess) continue;
        int clk = 0, mclk = 0, bus = 0;
        cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, i);
        cudaDeviceGetAttribute(&mclk, cudaDevAttrMemoryClockRate, i);
        cudaDeviceGetAttribute(&bus, cudaDevAttrGlobalMemoryBusWidth, i);
        std::snprintf(line, sizeof line,
                      "  %d: %s (sm_%d%d), %d SMs, %.1f GiB, %d-bit bus, SM clock %d MHz, memory clock %d MHz, %zu KiB shared/block\n",
                      i + 1, p.name, p.major, p.minor, p.multiProcessorCount, p.totalGlobalMem / 1073741824.0, bus,
                      clk / 1000, mclk / 1000, (size_t)(p.sharedMemPerBlockOptin / 1024));
        out += line;
    }
    if (buf && cap) std::snprintf(buf, cap, "%s", out.c_str());
    return out.size() < cap ? out.size() : (cap ? cap - 1 : 0);
}

const char* pcs_last_error(void) { return g_last_error.c_str(); }

const char* pcs_status_string(pcs_status s)
{
    switch (s) {
    case PCS_OK: return "ok";
    case PCS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PCS_ERR_CUDA: return "CUDA error";
    case PCS_ERR_OUT_OF_MEMORY: return "out of memory";
    case PCS_ERR_XML: return "XML error";
    case PCS_ERR_UNSUPPORTED: return "unsupported";
    case PCS_ERR_DEVICE: return "device error";
    case PCS_ERR_BUSY: return "busy";
    case PCS_ERR_NOT_FOUND: return "not found";
    }
    return "unknown status";
}

void pcs_params_defaults(pcs_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->model = PCS_MODEL_DISCRETE_FIXED_DEPTH;
    p->weighting_scheme = PCS_WEIGHTING_PMC_STANDARD;
    p->component_count = 1;
    p->kmin = 2;
    p->de_bin_count = 100;
    p->abc_sample_count = 256;
    p->avg_trial_count = 500;
    p->delta_gamma = 0.01;
    p->gamma_initial = 15.0;
    p->schedule = PCS_SCHEDULE_DELTA;
    p->perturbation = PCS_PERTURB_DIAGONAL;
    p->quantile = 0.5;
    p->reference_initial_gamma = 1;
    p->temperature = 298.0;
    p->viscosity = 0.95e-3;
}

pcs_status pcs_open(int device, int inflight, pcs_ctx** out)
{
    return guard([&] {
        need(out, "out");
        *out = nullptr;
        auto* c = new pcs_ctx;
        try {
            c->impl.reset(new Ctx(device, inflight));
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
    });
}

pcs_status pcs_close(pcs_ctx* ctx)
{
    return guard([&] {
        if (!ctx) return;
        for (Job* j : ctx->impl->table)
            if (j) j->slot = -1;
        delete ctx;
    });
}

pcs_status pcs_get_tuning(pcs_ctx* ctx, pcs_tuning* out)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(out, "out");
        out->block_size = c.tune.block;
        out->particles_per_thread = c.tune.ppt;
        out->hist_tile_rows = c.tune.tile_rows;
        out->warp_aggregate = c.tune.aggregate;
        out->chunk_particles = c.tune.chunk;
        out->round_capacity = c.tune.capacity;
        out->max_speculation = c.tune.max_spec;
        out->use_graphs = c.tune.use_graphs;
        out->plain_launch = c.tune.plain_launch;
        out->round_fill = c.tune.round_fill;
        out->walk = c.tune.walk;
        out->job_order = c.tune.job_order;
    });
}

pcs_status pcs_set_tuning(pcs_ctx* ctx, const pcs_tuning* t)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(t, "tuning");
        if (t->block_size) {
            if (t->block_size % 32 || t->block_size > 1024) throw Error(PCS_ERR_INVALID_ARGUMENT, "block_size must be a multiple of 32, <= 1024");
            c.tune.block = t->block_size;
        }
        if (t->particles_per_thread) {
            const uint32_t pp = t->particles_per_thread;
            if (pp != 1 && pp != 2 && pp != 4 && pp != 8)
                throw Error(PCS_ERR_INVALID_ARGUMENT, "particles_per_thread must be 1, 2, 4 or 8");
            c.tune.ppt = pp;
        }
        if (c.tune.block > sim_max_block((int)c.tune.ppt))
            throw Error(PCS_ERR_INVALID_ARGUMENT,
                        "block_size " + std::to_string(c.tune.block) + " is above the " +
                            std::to_string(sim_max_block((int)c.tune.ppt)) + " threads of the build for " +
                            std::to_string(c.tune.ppt) + " walkers per thread");
        if (t->hist_tile_rows) c.tune.tile_rows = t->hist_tile_rows == 0xFFFFFFFFu ? 0u : t->hist_tile_rows;
        if (t->warp_aggregate) c.tune.aggregate = t->warp_aggregate == 1u ? 1u : 0u;
        if (t->chunk_particles && t->chunk_particles != c.tune.chunk) {
            if (!c.table.empty()) throw Error(PCS_ERR_BUSY, "the work-item size can only change with no admitted jobs");
            c.tune.chunk = t->chunk_particles;
        }
        if (t->round_capacity) {
            if (!c.table.empty()) throw Error(PCS_ERR_BUSY, "round capacity can only change with no admitted jobs");
            c.tune.capacity = t->round_capacity;
            c.rb.capacity = 0; /* force reallocation */
        }
        if (t->max_speculation) c.tune.max_spec = t->max_speculation;
        if (t->use_graphs) c.tune.use_graphs = t->use_graphs == 1u ? 1u : 0u;
        if (t->plain_launch) {
            if (t->plain_launch != 1u && t->plain_launch != 2u) throw Error(PCS_ERR_INVALID_ARGUMENT, "plain_launch must be 1 or 2");
            c.tune.plain_launch = t->plain_launch;
        }
        if (t->round_fill) c.tune.round_fill = t->round_fill == 0xFFFFFFFFu ? 0u : t->round_fill;
        if (t->walk) {
            if (t->walk != 1u && t->walk != 2u) throw Error(PCS_ERR_INVALID_ARGUMENT, "walk must be 1 (slab-split) or 2 (per step)");
            c.tune.walk = t->walk;
        }
        if (t->job_order) {
            if (t->job_order != 1u && t->job_order != 2u) throw Error(PCS_ERR_INVALID_ARGUMENT, "job_order must be 1 or 2");
            c.tune.job_order = t->job_order;
        }
        /* the round plan on the device carries speculation, fill and order */
        if (c.rb.round.p) {
            c.upload_table();
            PCS_CUDA(cudaStreamSynchronize(c.stream));
        }
        c.graph_dirty = true;
    });
}

pcs_status pcs_timer_start(pcs_ctx* ctx)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        PCS_CUDA(cudaEventRecord(c.ev_t0, c.stream));
    });
}

pcs_status pcs_timer_stop(pcs_ctx* ctx, double* elapsed_ms)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(elapsed_ms, "elapsed_ms");
        PCS_CUDA(cudaEventRecord(c.ev_t1, c.stream));
        PCS_CUDA(cudaEventSynchronize(c.ev_t1));
        float ms = 0;
        PCS_CUDA(cudaEventElapsedTime(&ms, c.ev_t0, c.ev_t1));
        *elapsed_ms = ms;
    });
}

pcs_status pcs_get_kernel_stats(pcs_ctx* ctx, pcs_kernel_stats* out)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(out, "out");
        *out = c.stats;
        out->split_tasks = c.read_sim_tasks() - c.sim_tasks_base;
    });
}

pcs_status pcs_reset_kernel_stats(pcs_ctx* ctx)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        std::memset(&c.stats, 0, sizeof c.stats);
        c.sim_tasks_base = c.read_sim_tasks();
    });
}

/* ----------------------------------------------------------------------- */
/* jobs                                                                    */
/* ----------------------------------------------------------------------- */

pcs_status pcs_job_create(pcs_ctx* ctx, const pcs_params* p, const pcs_observed* obs, uint64_t seed,
                          pcs_job** out)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(p, "params");
        need(obs, "observed");
        need(out, "out");
        *out = nullptr;
        auto* j = new pcs_job;
        try {
            j->impl.reset(new Job(&c, *p, *obs, seed));
        } catch (...) {
            delete j;
            throw;
        }
        *out = j;
    });
}

pcs_status pcs_job_destroy(pcs_job* job)
{
    return guard([&] {
        if (!job) return;
        Job& j = *job->impl;
        Ctx& c = *j.ctx;
        PCS_CUDA(cudaSetDevice(c.device));
        if (j.slot >= 0) c.retire(&j);
        /* a served job destroyed before it finished gives its arena back */
        if (j.mem_counted) c.mem_used -= std::min<uint64_t>(c.mem_used, j.arena_bytes());
        c.queue.erase(std::remove(c.queue.begin(), c.queue.end(), &j), c.queue.end());
        delete job;
    });
}

static void run_until(Job& j, bool one_generation)
{
    Ctx& c = *j.ctx;
    if (j.status.done && j.initialised) return;
    bool admitted_here = false;
    if (j.slot < 0) {
        for (Job* t : c.table)
            if (t) throw Error(PCS_ERR_BUSY, "another job is admitted on this context (use the serve loop)");
        c.admit(&j);
        admitted_here = true;
    }
    const uint32_t gen0 = j.status.generation, it0 = j.status.iterations;
    uint64_t guard_rounds = 0;
    while (!j.status.done) {
        double ms = 0;
        c.run_round(&ms);
        if (++guard_rounds > 50000000ull) throw Error(PCS_ERR_DEVICE, "round limit exceeded");
        if (one_generation && (j.status.generation != gen0 || j.status.iterations != it0)) break;
    }
    if (j.status.done) {
        j.finished = true;
        if (admitted_here || one_generation) c.retire(&j);
    }
}

pcs_status pcs_job_run(pcs_job* job, uint32_t max_steps)
{
    return guard([&] {
        Job& j = J_(job);
        PCS_CUDA(cudaSetDevice(j.ctx->device));
        if (!j.initialised) {
            if (max_steps) j.p.max_generations = max_steps;
        } else if (max_steps) {
            throw Error(PCS_ERR_INVALID_ARGUMENT, "max_steps must be set before the job's first step");
        }
        run_until(j, false);
    });
}

pcs_status pcs_job_step(pcs_job* job, int* done)
{
    return guard([&] {
        Job& j = J_(job);
        PCS_CUDA(cudaSetDevice(j.ctx->device));
        run_until(j, true);
        if (done) *done = j.status.done ? 1 : 0;
    });
}

pcs_status pcs_job_checkpoint(pcs_job* job, void* buf, size_t cap, size_t* bytes)
{
    return guard([&] {
        Job& j = J_(job);
        need(bytes, "bytes");
        const size_t n = j.checkpoint_bytes();
        *bytes = n;
        if (!buf) return;
        if (cap < n) throw Error(PCS_ERR_INVALID_ARGUMENT, "checkpoint buffer too small");
        j.save_state(buf);
    });
}

pcs_status pcs_job_restore(pcs_job* job, const void* buf, size_t bytes)
{
    return guard([&] {
        Job& j = J_(job);
        need(buf, "buf");
        j.load_state(buf, bytes);
    });
}

pcs_status pcs_job_info_get(pcs_job* job, pcs_job_info* out)
{
    return guard([&] {
        Job& j = J_(job);
        need(out, "out");
        const JobPmcDev& s = j.status;
        out->component_count = j.C;
        out->z_component_count = j.Z;
        out->param_count = j.P;
        out->abc_sample_count = j.N;
        out->iterations = s.iterations;
        out->converged = s.converged;
        out->simulations = s.simulations;
        out->trials = s.trials;
        out->accepted = s.accepted_total;
        out->particle_steps = s.particle_steps;
        out->gamma = s.gamma;
        out->device_ms = j.device_ms;
    });
}

pcs_status pcs_job_output(pcs_job* job, double* m, double* s, double* c, double* az, double* dist, double* w)
{
    return guard([&] {
        Job& j = J_(job);
        PCS_CUDA(cudaSetDevice(j.ctx->device));
        if (!j.initialised) j.build_device_state();
        j.output(m, s, c, az, dist, w);
    });
}

/* ----------------------------------------------------------------------- */
/* serving                                                                 */
/* ----------------------------------------------------------------------- */

pcs_status pcs_serve_submit(pcs_ctx* ctx, pcs_job* job)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        Job& j = J_(job);
        if (j.ctx != &c) throw Error(PCS_ERR_INVALID_ARGUMENT, "job belongs to another context");
        if (j.in_serve) throw Error(PCS_ERR_BUSY, "job already submitted");
        j.in_serve = true;
        j.t_submit = std::chrono::steady_clock::now();
        c.queue.push_back(&j);
    });
}

pcs_status pcs_serve_set_memory_cap(pcs_ctx* ctx, uint64_t bytes)
{
    return guard([&] { C_(ctx).mem_cap = bytes; });
}

pcs_status pcs_serve_step(pcs_ctx* ctx, uint32_t* active)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        /* admission: by free device memory (or the cap) and table slots */
        while (!c.queue.empty()) {
            Job* j = c.queue.front();
            uint32_t used = 0;
            for (Job* t : c.table)
                if (t) ++used;
            if (used >= kMaxRoundJobs) break;
            size_t free_b = 0, total_b = 0;
            PCS_CUDA(cudaMemGetInfo(&free_b, &total_b));
            /* the job's arena plus the round histograms, which are shared and
             * sized for the widest admitted job: capacity x max(R x B) words */
            uint64_t rb_max = (uint64_t)j->R * j->B;
            for (Job* t : c.table)
                if (t) rb_max = std::max<uint64_t>(rb_max, (uint64_t)t->R * t->B);
            const uint64_t hist_b = (uint64_t)c.tune.capacity * rb_max * 4ull;
            const uint64_t need_total = c.mem_used + j->arena_bytes() + hist_b;
            const uint64_t need_b = j->arena_bytes() + (uint64_t)c.tune.capacity * j->R * j->B * 4ull;
            const bool over_cap = c.mem_cap && need_total > c.mem_cap;
            if (over_cap || need_b + (64ull << 20) > (uint64_t)free_b) {
                if (used == 0) throw Error(PCS_ERR_OUT_OF_MEMORY, "job does not fit in device memory");
                break;
            }
            c.queue.pop_front();
            c.admit(j);
            c.mem_used += j->arena_bytes();
            j->mem_counted = true;
        }
        uint32_t running = 0;
        for (Job* t : c.table)
            if (t) ++running;
        if (running) {
            double ms = 0;
            c.run_round(&ms);
            for (size_t i = 0; i < c.table.size(); ++i) {
                Job* t = c.table[i];
                if (t && t->status.done) {
                    t->finished = true;
                    t->t_done = std::chrono::steady_clock::now();
                    c.mem_used -= std::min<uint64_t>(c.mem_used, t->arena_bytes());
                    t->mem_counted = false;
                    c.retire(t);
                }
            }
        }
        uint32_t n = (uint32_t)c.queue.size();
        for (Job* t : c.table)
            if (t) ++n;
        if (active) *active = n;
    });
}

pcs_status pcs_serve_poll(pcs_ctx* ctx, pcs_job* job, int* finished)
{
    return guard([&] {
        (void)C_(ctx);
        Job& j = J_(job);
        need(finished, "finished");
        *finished = j.finished ? 1 : 0;
    });
}

/* ----------------------------------------------------------------------- */
/* hot-path entry points                                                   */
/* ----------------------------------------------------------------------- */

pcs_status pcs_simulate_hist(pcs_ctx* ctx, const pcs_setup* setup, const pcs_run* runs, uint32_t count,
                             uint64_t seed, const pcs_replay* replay, uint32_t* hist_out)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(setup, "setup");
        need(runs, "runs");
        need(hist_out, "hist_out");
        need(setup->frames, "setup->frames");
        const uint32_t V = setup->video_count, R = setup->rows, B = setup->de_bins, Cc = setup->component_count;
        if (count == 0) return;
        if (V == 0 || V > PCS_MAX_V) throw Error(PCS_ERR_INVALID_ARGUMENT, "video_count must be in 1..4096");
        if (Cc == 0 || Cc > PCS_MAX_C) throw Error(PCS_ERR_INVALID_ARGUMENT, "component_count must be in 1..8");
        if (R == 0 || B == 0) throw Error(PCS_ERR_INVALID_ARGUMENT, "rows and de_bins must be positive");
        if (setup->model < 0 || setup->model > 2) throw Error(PCS_ERR_INVALID_ARGUMENT, "unknown model");
        if (replay && count != 1) throw Error(PCS_ERR_INVALID_ARGUMENT, "replay needs count == 1");
        uint32_t fmax = 0;
        for (uint32_t v = 0; v < V; ++v) {
            if (setup->frames[v] == 0) throw Error(PCS_ERR_INVALID_ARGUMENT, "frame counts must be positive");
            fmax = std::max(fmax, setup->frames[v]);
        }
        if (fmax >= R) throw Error(PCS_ERR_INVALID_ARGUMENT, "rows must exceed the largest frame count (R = kmax + 1)");
        const uint64_t RB = (uint64_t)R * B;
        if (RB > (1ull << 31)) throw Error(PCS_ERR_UNSUPPORTED, "histogram too large");

        cudaStream_t st = c.stream;
        DevTmp t;
        JobDev jd{};
        jd.half_lx = setup->half_lx;
        jd.half_ly = setup->half_ly;
        jd.half_lz = setup->half_lz;
        jd.half_ax = setup->half_ax;
        jd.half_ay = setup->half_ay;
        jd.four_delta_t = setup->four_delta_t;
        jd.dde = setup->dde;
        jd.kmin = setup->kmin;
        jd.V = V;
        jd.R = R;
        jd.B = B;
        jd.model = (uint32_t)setup->model;
        jd.C = Cc;
        jd.Z = setup->model == PCS_MODEL_DISCRETE_VARIABLE_DEPTH ? Cc : 1u;
        pcs_seed_masks(seed, &jd.seed_lo, &jd.seed_hi);
        jd.frames_max = fmax;
        uint32_t* d_frames = t.get<uint32_t>(V);
        PCS_CUDA(cudaMemcpyAsync(d_frames, setup->frames, V * 4u, cudaMemcpyHostToDevice, st));
        jd.frames = d_frames;

        const uint32_t chunk = c.tune.chunk;
        const uint64_t cstride = 2ull * V + 1ull;
        std::vector<PropDev> props(count);
        std::vector<uint32_t> counts(count * cstride);
        std::vector<uint32_t> item_prop;
        for (uint32_t q = 0; q < count; ++q) {
            const pcs_run& r = runs[q];
            need(r.particles, "run.particles");
            PropDev& pd = props[q];
            std::memset(&pd, 0, sizeof pd);
            pd.job = 0;
            pd.slot = r.slot;
            pd.trial = r.trial;
            pd.gen = r.generation;
            for (int i = 0; i < PCS_MAX_C; ++i) {
                pd.half_az[i] = r.half_az[i];
                pd.pre_comp_prob[i] = r.pre_comp_prob[i];
                pd.sd_scale[i] = r.sd_scale[i];
                pd.sd_shape[i] = r.sd_shape[i];
            }
            uint64_t total = 0;
            uint32_t* cnt = counts.data() + q * cstride;
            cnt[V] = 0;
            for (uint32_t v = 0; v < V; ++v) {
                cnt[v] = r.particles[v];
                total += r.particles[v];
                cnt[V + 1 + v] = (uint32_t)total;
            }
            if (total > 0xFFFFFFFFull) throw Error(PCS_ERR_INVALID_ARGUMENT, "too many particles");
            pd.total_particles = (uint32_t)total;
            pd.counts_off = q * cstride;
            pd.hist_off = (uint64_t)q * RB;
            pd.item_begin = (uint32_t)item_prop.size();
            pd.item_count = (uint32_t)((total + chunk - 1) / chunk);
            for (uint32_t i = 0; i < pd.item_count; ++i) item_prop.push_back(q);
        }
        if (replay) {
            need(replay->uniforms, "replay->uniforms");
            need(replay->normals, "replay->normals");
            if (replay->normal_stride + 1 < fmax) throw Error(PCS_ERR_INVALID_ARGUMENT, "replay normal_stride < frames - 1");
            if (setup->model == PCS_MODEL_LOGNORMAL) need(replay->sigmas, "replay->sigmas");
        }
        JobDev* d_jobs = t.get<JobDev>(1);
        PropDev* d_props = t.get<PropDev>(count);
        uint32_t* d_counts = t.get<uint32_t>(counts.size());
        uint32_t* d_items = t.get<uint32_t>(item_prop.size());
        uint32_t* d_ctl = t.get<uint32_t>(2);
        uint32_t* d_hist = t.get<uint32_t>(count * RB);
        uint32_t ctl[2] = {(uint32_t)item_prop.size(), 0u};
        PCS_CUDA(cudaMemcpyAsync(d_jobs, &jd, sizeof jd, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_props, props.data(), sizeof(PropDev) * count, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_counts, counts.data(), counts.size() * 4, cudaMemcpyHostToDevice, st));
        if (!item_prop.empty())
            PCS_CUDA(cudaMemcpyAsync(d_items, item_prop.data(), item_prop.size() * 4, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_ctl, ctl, 8, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemsetAsync(d_hist, 0, count * RB * 4, st));

        SimArgs a{};
        a.jobs = d_jobs;
        a.props = d_props;
        a.counts = d_counts;
        a.hist = d_hist;
        a.item_prop = d_items;
        a.n_items = d_ctl;
        a.queue_head = d_ctl + 1;
        a.chunk = chunk;
        a.err = c.err.as<uint32_t>();
        a.tile_words = tile_words_for(std::min<uint32_t>(c.tune.tile_rows, R), B);
        if (replay) {
            const uint64_t n = props[0].total_particles;
            float* du = t.get<float>(4 * n);
            float* dn = t.get<float>((uint64_t)n * replay->normal_stride * 3);
            PCS_CUDA(cudaMemcpyAsync(du, replay->uniforms, 16 * n, cudaMemcpyHostToDevice, st));
            PCS_CUDA(cudaMemcpyAsync(dn, replay->normals, 12ull * n * replay->normal_stride, cudaMemcpyHostToDevice, st));
            a.rp_uniforms = du;
            a.rp_normals = dn;
            a.rp_stride = replay->normal_stride;
            if (replay->sigmas) {
                float* ds = t.get<float>(n);
                PCS_CUDA(cudaMemcpyAsync(ds, replay->sigmas, 4 * n, cudaMemcpyHostToDevice, st));
                a.rp_sigmas = ds;
            }
        }
        SimLaunch l{};
        l.block = c.tune.block;
        l.ppt = replay ? 1 : (int)c.tune.ppt;
        l.replay = replay != nullptr;
        l.aggregate = c.tune.aggregate == 1u;
        l.split = !replay && c.split_walk();
        int occ = simulate_occupancy(l, a.tile_words);
        l.grid = (uint32_t)std::max(1, occ) * (uint32_t)c.sm_count;
        PCS_CUDA(launch_simulate(a, l, st));
        PCS_CUDA(cudaMemcpyAsync(hist_out, d_hist, count * RB * 4, cudaMemcpyDeviceToHost, st));
        PCS_CUDA(cudaStreamSynchronize(st));
        check_err_word(c);
    });
}

pcs_status pcs_scan_distance(pcs_ctx* ctx, const uint32_t* hist, const uint32_t* ref_sat, uint32_t rows,
                             uint32_t bins, uint32_t count, uint32_t* cum_out, float* dist_f32,
                             double* dist_f64, uint64_t* ssd)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(hist, "hist");
        need(ref_sat, "ref_sat");
        need(dist_f32, "dist_f32");
        if (count == 0) return;
        if (rows == 0 || bins == 0) throw Error(PCS_ERR_INVALID_ARGUMENT, "rows and bins must be positive");
        const uint64_t RB = (uint64_t)rows * bins;
        const size_t smem = distance_smem_bytes(rows);
        if (smem > 227u * 1024u) throw Error(PCS_ERR_UNSUPPORTED, "too many histogram rows for one CTA");
        cudaStream_t st = c.stream;
        DevTmp t;
        std::vector<uint32_t> refT(RB);
        for (uint32_t r = 0; r < rows; ++r)
            for (uint32_t b = 0; b < bins; ++b)
                refT[pcs_sat_t_index(r, b, rows, bins)] = ref_sat[(uint64_t)r * bins + b];
        uint32_t* d_hist = t.get<uint32_t>(count * RB);
        uint32_t* d_ref = t.get<uint32_t>(RB);
        uint32_t* d_refT = t.get<uint32_t>(RB);
        uint32_t* d_cum = cum_out ? t.get<uint32_t>(count * RB) : nullptr;
        float* d_d32 = t.get<float>(count);
        double* d_d64 = dist_f64 ? t.get<double>(count) : nullptr;
        uint64_t* d_ssd = ssd ? t.get<uint64_t>(2ull * count) : nullptr;
        JobDev jd{};
        jd.R = rows;
        jd.B = bins;
        jd.ref_sat = d_ref;
        jd.ref_sat_t = d_refT;
        TmapDev map;
        jd.tmap_depth = encode_hist_tmap(&map, d_hist, rows, bins, count) ? count : 0u;
        TmapDev* d_map = t.get<TmapDev>(1);
        std::vector<PropDev> props(count);
        for (uint32_t q = 0; q < count; ++q) {
            std::memset(&props[q], 0, sizeof(PropDev));
            props[q].hist_off = (uint64_t)q * RB;
            props[q].hist_z = q;
        }
        JobDev* d_jobs = t.get<JobDev>(1);
        PropDev* d_props = t.get<PropDev>(count);
        uint32_t* d_n = t.get<uint32_t>(1);
        PCS_CUDA(cudaMemcpyAsync(d_hist, hist, count * RB * 4, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_ref, ref_sat, RB * 4, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_refT, refT.data(), RB * 4, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_jobs, &jd, sizeof jd, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_map, &map, sizeof map, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_props, props.data(), sizeof(PropDev) * count, cudaMemcpyHostToDevice, st));
        PCS_CUDA(cudaMemcpyAsync(d_n, &count, 4, cudaMemcpyHostToDevice, st));
        DistArgs d{};
        d.jobs = d_jobs;
        d.props = d_props;
        d.n_props = d_n;
        d.hist = d_hist;
        d.cum_out = d_cum;
        d.dist_f32 = d_d32;
        d.dist_f64 = d_d64;
        d.ssd = d_ssd;
        d.err = c.err.as<uint32_t>();
        d.max_rows = rows;
        d.tmaps = d_map;
        const uint32_t cl = (d_cum || d_d64 || d_ssd) ? 0u : distance_cluster_size(rows, bins);
        PCS_CUDA(launch_distance(d, std::min<uint32_t>(count, (uint32_t)(distance_ctas_per_sm(rows) * c.sm_count)), st, cl));
        if (cum_out) PCS_CUDA(cudaMemcpyAsync(cum_out, d_cum, count * RB * 4, cudaMemcpyDeviceToHost, st));
        PCS_CUDA(cudaMemcpyAsync(dist_f32, d_d32, count * 4, cudaMemcpyDeviceToHost, st));
        if (dist_f64) PCS_CUDA(cudaMemcpyAsync(dist_f64, d_d64, count * 8, cudaMemcpyDeviceToHost, st));
        if (ssd) PCS_CUDA(cudaMemcpyAsync(ssd, d_ssd, 16ull * count, cudaMemcpyDeviceToHost, st));
        PCS_CUDA(cudaStreamSynchronize(st));
        check_err_word(c);
    });
}

pcs_status pcs_observed_sat(pcs_ctx* ctx, const uint32_t* K, const double* DE, size_t n, uint32_t rows,
                            uint32_t bins, double ub_de, uint32_t* sat_out)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(sat_out, "sat_out");
        if (n && (!K || !DE)) throw Error(PCS_ERR_INVALID_ARGUMENT, "K/DE are NULL");
        if (rows == 0 || bins == 0) throw Error(PCS_ERR_INVALID_ARGUMENT, "rows and bins must be positive");
        cudaStream_t st = c.stream;
        DevTmp t;
        const uint64_t RB = (uint64_t)rows * bins;
        uint32_t* dK = t.get<uint32_t>(n);
        double* dDE = t.get<double>(n);
        uint32_t* dS = t.get<uint32_t>(RB);
        if (n) {
            PCS_CUDA(cudaMemcpyAsync(dK, K, n * 4, cudaMemcpyHostToDevice, st));
            PCS_CUDA(cudaMemcpyAsync(dDE, DE, n * 8, cudaMemcpyHostToDevice, st));
        }
        PCS_CUDA(launch_observed_sat(dK, dDE, n, rows, bins, ub_de, dS, nullptr, c.err.as<uint32_t>(), st));
        PCS_CUDA(cudaMemcpyAsync(sat_out, dS, RB * 4, cudaMemcpyDeviceToHost, st));
        PCS_CUDA(cudaStreamSynchronize(st));
        check_err_word(c);
    });
}

pcs_status pcs_observed_sat_julia(pcs_ctx* ctx, const uint32_t* K, const double* DE, size_t n, uint32_t kmax,
                                  uint32_t bins, double ub_de, uint32_t* sat_out)
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(sat_out, "sat_out");
        if (n && (!K || !DE)) throw Error(PCS_ERR_INVALID_ARGUMENT, "K/DE are NULL");
        if (kmax == 0 || bins == 0) throw Error(PCS_ERR_INVALID_ARGUMENT, "kmax and bins must be positive");
        cudaStream_t st = c.stream;
        DevTmp t;
        const uint64_t RB = (uint64_t)kmax * bins;
        uint32_t* dK = t.get<uint32_t>(n);
        double* dDE = t.get<double>(n);
        uint32_t* dS = t.get<uint32_t>(RB);
        if (n) {
            PCS_CUDA(cudaMemcpyAsync(dK, K, n * 4, cudaMemcpyHostToDevice, st));
            PCS_CUDA(cudaMemcpyAsync(dDE, DE, n * 8, cudaMemcpyHostToDevice, st));
        }
        PCS_CUDA(launch_observed_sat_julia(dK, dDE, n, kmax, bins, ub_de, dS, c.err.as<uint32_t>(), st));
        PCS_CUDA(cudaMemcpyAsync(sat_out, dS, RB * 4, cudaMemcpyDeviceToHost, st));
        PCS_CUDA(cudaStreamSynchronize(st));
        check_err_word(c);
    });
}

pcs_status pcs_debug_particle_stream(pcs_ctx* ctx, uint64_t seed, uint32_t slot, uint32_t trial,
                                     uint32_t generation, uint32_t particle, uint32_t block, uint32_t out[4])
{
    return guard([&] {
        Ctx& c = C_(ctx);
        need(out, "out");
        DevTmp t;
        uint32_t* d = t.get<uint32_t>(4);
        PCS_CUDA(launch_debug_stream(seed, slot, generation, trial, particle, block, d, c.stream));
        PCS_CUDA(cudaMemcpyAsync(out, d, 16, cudaMemcpyDeviceToHost, c.stream));
        PCS_CUDA(cudaStreamSynchronize(c.stream));
    });
}

pcs_status pcs_debug_round_proposals(pcs_job* job, uint32_t cap, uint32_t* n, pcs_debug_proposal* props,
                                     double* theta, uint32_t* counts)
{
    return guard([&] {
        Job& j = J_(job);
        need(n, "n");
        Ctx& c = *j.ctx;
        PCS_CUDA(cudaSetDevice(c.device));
        if (j.slot < 0) throw Error(PCS_ERR_NOT_FOUND, "job is not in the round table (not admitted, or retired)");
        if (!c.rb.round.p) throw Error(PCS_ERR_NOT_FOUND, "no round has run on this context");
        PCS_CUDA(cudaStreamSynchronize(c.stream));
        RoundDev rd;
        PCS_CUDA(cudaMemcpy(&rd, c.rb.round.p, sizeof rd, cudaMemcpyDeviceToHost));
        const uint32_t js = (uint32_t)j.slot;
        const uint32_t cnt = js < rd.n_jobs ? rd.job_count[js] : 0u;
        const uint32_t base = rd.job_base[js];
        *n = cnt;
        if (!props || cnt == 0) return;
        if (cap < cnt) throw Error(PCS_ERR_INVALID_ARGUMENT, "cap is smaller than the round's proposals of the job");
        need(theta, "theta");
        need(counts, "counts");
        std::vector<PropDev> pd(cnt);
        std::vector<double> th((size_t)cnt * PCS_MAX_P);
        const uint64_t stride = 2ull * rd.v_max + 1ull;
        std::vector<uint32_t> cv((size_t)cnt * stride);
        PCS_CUDA(cudaMemcpy(pd.data(), c.rb.props.as<PropDev>() + base, cnt * sizeof(PropDev), cudaMemcpyDeviceToHost));
        PCS_CUDA(cudaMemcpy(th.data(), c.rb.theta_prop.as<double>() + (size_t)base * PCS_MAX_P, th.size() * 8,
                            cudaMemcpyDeviceToHost));
        PCS_CUDA(cudaMemcpy(cv.data(), c.rb.counts.as<uint32_t>() + base * stride, cv.size() * 4,
                            cudaMemcpyDeviceToHost));
        std::vector<float> dv(cnt);
        PCS_CUDA(cudaMemcpy(dv.data(), c.rb.dist32.as<float>() + base, cnt * sizeof(float), cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < cnt; ++i) {
            const PropDev& q = pd[i];
            pcs_debug_proposal& o = props[i];
            o.slot = q.slot;
            o.trial = q.trial;
            o.generation = q.gen;
            o.total_particles = q.total_particles;
            for (int k = 0; k < PCS_MAX_COMPONENTS; ++k) {
                o.half_az[k] = q.half_az[k];
                o.pre_comp_prob[k] = q.pre_comp_prob[k];
                o.sd_scale[k] = q.sd_scale[k];
                o.sd_shape[k] = q.sd_shape[k];
            }
            o.distance = dv[i];
            for (uint32_t p = 0; p < j.P; ++p) theta[(size_t)i * j.P + p] = th[(size_t)i * PCS_MAX_P + p];
            const uint64_t off = q.counts_off - (uint64_t)base * stride;
            for (uint32_t v = 0; v < j.V; ++v) counts[(size_t)i * j.V + v] = cv[off + v];
        }
    });
}

} // extern "C"
