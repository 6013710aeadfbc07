/*
 * plain.cpp -- the plain form: the reference's schedule on this library's
 * kernels.
 *
 * SimulationT::run (src/gpu/detail/simulation_impl.inl:178-455) keeps the
 * ABC-PMC state on the host in double and ships one proposal at a time:
 * per proposal it uploads the forward-model arguments, launches the
 * simulate and distance kernels on one of Q streams (queues, -g dev/Q), and
 * reads the distance back when the stream reports completion; each
 * population slot has at most one trial in flight.  This file does the same
 * with the sm_103a kernels: proposals are built on the host with the same
 * code and random streams as the batched path (pcs_proposal.h), weights are
 * the reference's O(N^2 P) double loop.  It exists to measure what batching
 * and serving buy; pcs_job_run is the fast path.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "engine.h"
#include "pcs_proposal.h"

namespace pcs {

namespace {

struct Queue {
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    DevBuf d_prop, d_counts, d_items, d_ctl, d_hist, d_dist, d_nprops;
    PropDev* h_prop = nullptr;
    uint32_t* h_counts = nullptr;
    uint32_t* h_ctl = nullptr;
    float* h_dist = nullptr;
    int slot = -1;
    double theta[PCS_MAX_P];
};

double normpdf0(double x, double sigma)
{
    /* normpdf_ (simulation_impl.inl:46-52) with mu = 0 */
    return std::exp(-0.5 * x * x / (sigma * sigma)) / (std::sqrt(2.0 * M_PI) * sigma);
}

} // namespace

void run_plain(Job& j, uint32_t max_steps, uint32_t queues)
{
    Ctx& c = *j.ctx;
    if (j.slot >= 0) throw Error(PCS_ERR_BUSY, "job is admitted to the batched engine");
    if (!j.initialised) {
        if (max_steps) j.p.max_generations = max_steps;
        j.build_device_state();
    } else if (j.status.iterations > 0) {
        throw Error(PCS_ERR_INVALID_ARGUMENT, "the plain form runs a job from its start");
    }
    if (queues == 0) queues = 30;
    const JobPmcDev& pm = j.pm;
    const uint32_t N = j.N, P = j.P, V = j.V;
    const uint64_t RB = (uint64_t)j.R * j.B;

    /* host state (prior population drawn by build_device_state) */
    std::vector<double> theta((size_t)N * P), theta_new((size_t)N * P), w(N, 1.0 / N), wcum(N), factor((size_t)P * P);
    std::vector<double> dist(N, 0.0), dist_new(N, 0.0), wstar(N);
    PCS_CUDA(cudaMemcpy(theta.data(), pm.theta, theta.size() * 8, cudaMemcpyDeviceToHost));
    PCS_CUDA(cudaMemcpy(factor.data(), pm.factor, factor.size() * 8, cudaMemcpyDeviceToHost));

    DevBuf d_job;
    d_job.alloc(sizeof(JobDev));
    PCS_CUDA(cudaMemcpy(d_job.p, &j.jd, sizeof(JobDev), cudaMemcpyHostToDevice));

    /* particles per proposal are bounded by the prior's largest Poisson mean */
    const double lam_max = (double)j.C * j.p.ub_c * j.p.Lx * j.p.Ly * j.p.Lz / 1e12;
    const uint64_t parts_max = (uint64_t)std::ceil((lam_max + 12.0 * std::sqrt(lam_max) + 16.0) * V);
    /* launch geometry: the reference's (ceil(V/4) CTAs of 128 threads per
     * proposal, simulation_impl.inl:655-656, launched at :1065), or this
     * build's full persistent grid */
    const bool ref_geometry = c.tune.plain_launch != 2u;
    const uint32_t chunk = ref_geometry ? 128u : c.tune.chunk;
    const uint32_t items_cap = (uint32_t)std::min<uint64_t>(parts_max / chunk + 2, 1u << 30);
    std::vector<Queue> qs(queues);
    for (auto& q : qs) {
        PCS_CUDA(cudaStreamCreateWithFlags(&q.st, cudaStreamNonBlocking));
        PCS_CUDA(cudaEventCreateWithFlags(&q.done, cudaEventDisableTiming));
        q.d_prop.alloc(sizeof(PropDev));
        q.d_counts.alloc(sizeof(uint32_t) * (2 * V + 1));
        q.d_items.alloc(sizeof(uint32_t) * items_cap);
        q.d_ctl.alloc(16);
        q.d_hist.alloc(sizeof(uint32_t) * RB);
        q.d_dist.alloc(sizeof(float));
        q.d_nprops.alloc(4);
        PCS_CUDA(cudaMemset(q.d_items.p, 0, sizeof(uint32_t) * items_cap));
        PCS_CUDA(cudaMemset(q.d_hist.p, 0, sizeof(uint32_t) * RB));
        const uint32_t one = 1u;
        PCS_CUDA(cudaMemcpy(q.d_nprops.p, &one, 4, cudaMemcpyHostToDevice));
        PCS_CUDA(cudaMallocHost((void**)&q.h_prop, sizeof(PropDev)));
        PCS_CUDA(cudaMallocHost((void**)&q.h_counts, sizeof(uint32_t) * (2 * V + 1)));
        PCS_CUDA(cudaMallocHost((void**)&q.h_ctl, 16));
        PCS_CUDA(cudaMallocHost((void**)&q.h_dist, sizeof(float)));
    }
    auto cleanup = [&] {
        for (auto& q : qs) {
            if (q.st) cudaStreamSynchronize(q.st);
            if (q.st) cudaStreamDestroy(q.st);
            if (q.done) cudaEventDestroy(q.done);
            if (q.h_prop) cudaFreeHost(q.h_prop);
            if (q.h_counts) cudaFreeHost(q.h_counts);
            if (q.h_ctl) cudaFreeHost(q.h_ctl);
            if (q.h_dist) cudaFreeHost(q.h_dist);
        }
    };

    const uint32_t tile_words = tile_words_for(std::min<uint32_t>(c.tune.tile_rows, j.R), j.B);
    SimLaunch sl{};
    sl.block = ref_geometry ? 128u : c.tune.block;
    sl.ppt = ref_geometry ? 1 : (int)c.tune.ppt;
    sl.replay = false;
    sl.aggregate = c.tune.aggregate == 1u;
    sl.split = c.split_walk();
    /* the split walk runs 256-thread CTAs: half as many of them give the
     * reference geometry's thread count */
    const uint32_t sim_slots = ref_geometry ? (sl.split ? (V + 7u) / 8u : (V + 3u) / 4u)
                                            : c.sim_grid(sl.block, c.tune.ppt, sl.aggregate, tile_words, sl.split);

    JobPmcDev st = j.status; /* counters reported through pcs_job_info */
    uint64_t gen_trials = 0;

    /* submit trial `trial` of `slot` (generation `gen`) on queue q */
    auto submit = [&](Queue& q, uint32_t slot, uint32_t trial, uint32_t gen) {
        pcs_build_theta(pm, theta.data(), wcum.data(), factor.data(), slot, trial, gen, j.jd.seed_lo, j.jd.seed_hi, q.theta);
        PropDev& pd = *q.h_prop;
        std::memset(&pd, 0, sizeof pd);
        pd.job = 0;
        pd.slot = slot;
        pd.trial = trial;
        pd.gen = gen;
        const double lambda = pcs_build_args(pm, q.theta, gen, pd);
        uint64_t steps = 0;
        const uint64_t total = pcs_draw_counts(lambda, V, j.frames.data(), slot, trial, gen, j.jd.seed_lo, j.jd.seed_hi,
                                               q.h_counts, q.h_counts + V, &steps);
        if (total > 0xFFFFFFFFull) throw Error(PCS_ERR_DEVICE, "too many particles in one proposal");
        pd.total_particles = (uint32_t)total;
        pd.counts_off = 0;
        pd.hist_off = 0;
        pd.item_begin = 0;
        pd.item_count = (uint32_t)((total + chunk - 1) / chunk);
        if (pd.item_count > items_cap) throw Error(PCS_ERR_DEVICE, "work items exceed the plain-form capacity");
        q.h_ctl[0] = pd.item_count;
        q.h_ctl[1] = 0u;
        PCS_CUDA(cudaMemcpyAsync(q.d_prop.p, q.h_prop, sizeof(PropDev), cudaMemcpyHostToDevice, q.st));
        PCS_CUDA(cudaMemcpyAsync(q.d_counts.p, q.h_counts, sizeof(uint32_t) * (2 * V + 1), cudaMemcpyHostToDevice, q.st));
        PCS_CUDA(cudaMemcpyAsync(q.d_ctl.p, q.h_ctl, 8, cudaMemcpyHostToDevice, q.st));
        SimArgs a{};
        a.jobs = d_job.as<JobDev>();
        a.props = q.d_prop.as<PropDev>();
        a.counts = q.d_counts.as<uint32_t>();
        a.hist = q.d_hist.as<uint32_t>();
        a.item_prop = q.d_items.as<uint32_t>();
        a.n_items = q.d_ctl.as<uint32_t>();
        a.queue_head = q.d_ctl.as<uint32_t>() + 1;
        a.chunk = chunk;
        a.tile_words = tile_words;
        a.err = c.err.as<uint32_t>();
        SimLaunch l = sl;
        l.grid = ref_geometry ? sim_slots : std::max<uint32_t>(1u, std::min<uint32_t>(pd.item_count, sim_slots));
        PCS_CUDA(launch_simulate(a, l, q.st));
        DistArgs d{};
        d.jobs = d_job.as<JobDev>();
        d.props = q.d_prop.as<PropDev>();
        d.n_props = q.d_nprops.as<uint32_t>();
        d.hist = q.d_hist.as<uint32_t>();
        d.dist_f32 = q.d_dist.as<float>();
        d.err = c.err.as<uint32_t>();
        d.max_rows = j.R;
        /* the reference's geometry: one CTA per histogram; the persistent
         * form spreads the histogram's strips over a cluster */
        PCS_CUDA(launch_distance(d, 1, q.st, ref_geometry ? 0u : distance_cluster_size(j.R, j.B)));
        PCS_CUDA(cudaMemcpyAsync(q.h_dist, q.d_dist.p, sizeof(float), cudaMemcpyDeviceToHost, q.st));
        PCS_CUDA(cudaEventRecord(q.done, q.st));
        q.slot = (int)slot;
        st.simulations += 1;
        st.particle_steps += steps;
    };

    /* one pass over the population: every slot tries until its distance is
     * within gamma (or, in the prior pass, once); returns the trial count */
    auto generation = [&](uint32_t gen, double gamma, bool prior) -> bool {
        std::vector<uint32_t> next_trial(N, 0u);
        std::vector<double> dist_bis(N, INFINITY);
        std::vector<uint8_t> done(N, 0u);
        std::vector<uint32_t> waiting(N);
        std::iota(waiting.begin(), waiting.end(), 0u);
        uint64_t trials_total = 0;
        double trials_avg = 0.0;
        uint32_t active = N, pending = 0;
        size_t rr = 0;
        std::vector<uint32_t> carry;
        while (active) {
            /* submit (simulation_impl.inl:256-347) */
            carry.clear();
            for (uint32_t s : waiting) {
                const bool again = prior ? next_trial[s] == 0 : (dist_bis[s] > gamma && trials_avg < (double)j.p.avg_trial_count);
                if (!again) {
                    if (!done[s]) {
                        done[s] = 1;
                        --active;
                    }
                    continue;
                }
                Queue* free_q = nullptr;
                for (auto& q : qs)
                    if (q.slot < 0) {
                        free_q = &q;
                        break;
                    }
                if (!free_q) {
                    carry.push_back(s);
                    continue;
                }
                submit(*free_q, s, next_trial[s]++, gen);
                ++pending;
            }
            waiting.swap(carry);
            if (!pending) continue;
            /* gather (simulation_impl.inl:358-389): wait for the next queue to finish */
            for (;;) {
                Queue& q = qs[rr % qs.size()];
                ++rr;
                if (q.slot < 0) continue;
                if (cudaEventQuery(q.done) == cudaErrorNotReady) {
                    bool any = false;
                    for (auto& o : qs)
                        if (o.slot >= 0 && cudaEventQuery(o.done) == cudaSuccess) any = true;
                    if (!any) PCS_CUDA(cudaEventSynchronize(q.done));
                    else continue;
                }
                const uint32_t s = (uint32_t)q.slot;
                q.slot = -1;
                --pending;
                const double d = std::log10((double)*q.h_dist);
                dist_bis[s] = d;
                std::memcpy(&theta_new[(size_t)s * P], q.theta, sizeof(double) * P);
                dist_new[s] = d;
                ++trials_total;
                trials_avg = (double)trials_total / (double)N;
                waiting.push_back(s);
                break;
            }
        }
        for (auto& q : qs)
            if (q.slot >= 0) throw Error(PCS_ERR_DEVICE, "plain form: a queue is still busy");
        gen_trials = trials_total;
        st.trials = trials_total;
        return trials_avg >= (double)j.p.avg_trial_count;
    };

    try {
        const bool prior_pass = j.p.gamma_adaptive || j.p.schedule == PCS_SCHEDULE_QUANTILE;
        double gamma = j.p.gamma_initial;
        std::partial_sum(w.begin(), w.end(), wcum.begin());
        if (prior_pass) {
            /* compute_initial_gamma_ (simulation_impl.inl:750-830) */
            generation(0, INFINITY, true);
            st.accepted_total += N; /* the prior pass accepts every slot, as the batched path counts it */
            std::vector<double> dd = dist_new;
            const size_t n = (j.p.schedule == PCS_SCHEDULE_QUANTILE)
                                 ? std::min<size_t>(N - 1, (size_t)std::floor(j.p.quantile * N))
                                 : N / 2;
            std::nth_element(dd.begin(), dd.begin() + n, dd.end());
            gamma = dd[n];
            if (j.p.schedule == PCS_SCHEDULE_QUANTILE) dist = dist_new;
        }
        st.iterations = 0;
        st.converged = 0;
        uint32_t gen = 0;
        for (;;) {
            /* simulation_impl.inl:202-222 */
            st.iterations += 1;
            if (j.p.max_generations && st.iterations > j.p.max_generations) break;
            if (gen >= PCS_MAX_GENERATION) break; /* the random-stream counter holds 12 bits of generation */
            if (j.p.schedule == PCS_SCHEDULE_DELTA) gamma -= j.p.delta_gamma;
            gen += 1;
            std::partial_sum(w.begin(), w.end(), wcum.begin());
            const bool capped = generation(gen, gamma, false);
            st.gamma = gamma;
            st.generation = gen;
            if (capped) {
                st.converged = 1;
                break;
            }
            st.accepted_total += N;
            /* weights (simulation_impl.inl:832-887) */
            if (j.p.weighting_scheme == PCS_WEIGHTING_PMC_STANDARD) {
                double wsum = 0.0;
                for (uint32_t a = 0; a < N; ++a) {
                    double acc = 0.0;
                    for (uint32_t i = 0; i < N; ++i) {
                        double term = 1.0;
                        for (uint32_t q = 0; q < P; ++q) {
                            if (pm.fixed[q]) continue;
                            term *= normpdf0(theta_new[(size_t)a * P + q] - theta[(size_t)i * P + q], factor[(size_t)q * P + q]);
                        }
                        acc += w[i] * term;
                    }
                    wstar[a] = 1.0 / acc;
                    wsum += wstar[a];
                }
                for (uint32_t a = 0; a < N; ++a) w[a] = wstar[a] / wsum;
            } else {
                double wsum = 0.0;
                for (uint32_t a = 0; a < N; ++a) {
                    wstar[a] = 1.0 / (dist_new[a] * dist_new[a]);
                    wsum += wstar[a];
                }
                for (uint32_t a = 0; a < N; ++a) w[a] = wstar[a] / wsum;
            }
            theta = theta_new;
            dist = dist_new;
            /* compute_tau_ (simulation_impl.inl:733-749) */
            for (uint32_t q = 0; q < P; ++q) {
                double s = 0, cnt = 0;
                for (uint32_t i = 0; i < N; ++i, cnt += 1) s += theta[(size_t)i * P + q];
                const double mean = s / cnt;
                double v = 0;
                for (uint32_t i = 0; i < N; ++i) {
                    const double x = theta[(size_t)i * P + q] - mean;
                    v += x * x;
                }
                for (uint32_t r = 0; r < P; ++r) factor[(size_t)q * P + r] = 0.0;
                factor[(size_t)q * P + q] = std::sqrt(2.0 * (v / cnt));
            }
            if (j.p.schedule == PCS_SCHEDULE_QUANTILE) {
                std::vector<double> dd = dist;
                const size_t n = std::min<size_t>(N - 1, (size_t)std::floor(j.p.quantile * N));
                std::nth_element(dd.begin(), dd.begin() + n, dd.end());
                gamma = dd[n];
            }
        }
        (void)gen_trials;
        /* publish the committed population where pcs_job_output reads it */
        PCS_CUDA(cudaMemcpy(pm.theta, theta.data(), theta.size() * 8, cudaMemcpyHostToDevice));
        PCS_CUDA(cudaMemcpy(pm.w, w.data(), w.size() * 8, cudaMemcpyHostToDevice));
        PCS_CUDA(cudaMemcpy(pm.dist, dist.data(), dist.size() * 8, cudaMemcpyHostToDevice));
        st.done = 1;
        st.gamma = gamma;
        j.status = st;
        j.finished = true;
        uint32_t bits = 0;
        PCS_CUDA(cudaMemcpy(&bits, c.err.p, 4, cudaMemcpyDeviceToHost));
        if (bits) throw Error(PCS_ERR_DEVICE, "device error word " + std::to_string(bits));
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
}

} // namespace pcs

namespace pcs {
void set_last_error(const std::string& m);
}

extern "C" pcs_status pcs_job_run_plain(pcs_job* job, uint32_t max_steps, uint32_t queues)
{
    try {
        if (!job) throw pcs::Error(PCS_ERR_INVALID_ARGUMENT, "job is NULL");
        PCS_CUDA(cudaSetDevice(job->impl->ctx->device));
        pcs::run_plain(*job->impl, max_steps, queues);
        pcs::set_last_error("");
        return PCS_OK;
    } catch (const pcs::Error& e) {
        pcs::set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        pcs::set_last_error(e.what());
        return PCS_ERR_INVALID_ARGUMENT;
    }
}
