/*
 * autotune.cpp -- the engine's own tuner for the forward-model launch.
 *
 * Times the fused simulate kernel on the first batched round of a job of
 * the requested shape (its prior-pass proposals: real Poisson particle
 * counts, real frame counts) over a grid of block sizes (128-1024),
 * interleaved walkers per thread (1, 2, 4, 8; each count's build limits
 * its block size, sim_max_block), shared-memory histogram tiles
 * and warp aggregation, and keeps the fastest.  The reference has no
 * counterpart; its launch shape is fixed at ceil(V/4) x 128
 * (src/gpu/detail/simulation_impl.inl:655-656).
 */
#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.h"

namespace pcs {

namespace {

struct Candidate {
    uint32_t block, ppt, tile_rows, agg;
};

} // namespace

/* Times one launch configuration on the round buffers prepared by
 * plan/propose/items (queue head reset before each timed launch). */
static float time_config(Ctx& c, const Candidate& k, int reps)
{
    RoundDev* rd = c.rb.round.as<RoundDev>();
    SimArgs s{};
    s.jobs = c.rb.jobs.as<JobDev>();
    s.props = c.rb.props.as<PropDev>();
    s.counts = c.rb.counts.as<uint32_t>();
    s.hist = c.rb.hist.as<uint32_t>();
    s.item_prop = c.rb.item_prop.as<uint32_t>();
    s.n_items = &rd->n_items;
    s.queue_head = &rd->queue_head;
    s.chunk = c.tune.chunk;
    s.tile_words = tile_words_for(k.tile_rows, c.rb_max_b_);
    s.err = c.err.as<uint32_t>();
    SimLaunch l{};
    l.block = k.block;
    l.ppt = (int)k.ppt;
    l.aggregate = k.agg != 0;
    l.replay = false;
    l.split = c.split_walk();
    l.grid = c.sim_grid(l.block, k.ppt, l.aggregate, s.tile_words, l.split);
    float best = 1e30f;
    for (int r = 0; r < reps; ++r) {
        PCS_CUDA(cudaMemsetAsync(&rd->queue_head, 0, 4, c.stream));
        PCS_CUDA(cudaEventRecord(c.ev0, c.stream));
        PCS_CUDA(launch_simulate(s, l, c.stream));
        PCS_CUDA(cudaEventRecord(c.ev1, c.stream));
        PCS_CUDA(cudaEventSynchronize(c.ev1));
        float ms = 0;
        PCS_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        best = std::min(best, ms);
    }
    /* the histogram area accumulated garbage: clear it for real rounds */
    PCS_CUDA(cudaMemsetAsync(c.rb.hist.p, 0, sizeof(uint32_t) * c.rb.hist_cap, c.stream));
    PCS_CUDA(cudaStreamSynchronize(c.stream));
    return best;
}

void autotune(Ctx& c, const pcs_params& p, const pcs_observed& obs, pcs_tuning* chosen)
{
    for (Job* t : c.table)
        if (t) throw Error(PCS_ERR_BUSY, "autotune needs a context with no admitted jobs");
    pcs_params q = p;
    q.gamma_adaptive = 1; /* start with the prior pass so the round has real proposals */
    Job job(&c, q, obs, 0x5EEDull);
    c.admit(&job);
    try {
        PmcArgs a{};
        a.pmc = c.rb.pmc.as<JobPmcDev>();
        a.jobs = c.rb.jobs.as<JobDev>();
        a.round = c.rb.round.as<RoundDev>();
        a.props = c.rb.props.as<PropDev>();
        a.theta_prop = c.rb.theta_prop.as<double>();
        a.counts = c.rb.counts.as<uint32_t>();
        a.item_prop = c.rb.item_prop.as<uint32_t>();
        a.dist_f32 = c.rb.dist32.as<float>();
        a.dist_f64 = c.rb.dist64.as<double>();
        a.err = c.err.as<uint32_t>();
        a.logfact = c.logfact.as<double>();
        a.logfact_n = kLogFactEntries;
        PCS_CUDA(launch_round_plan(a, c.stream));
        PCS_CUDA(launch_propose(a, c.rb.capacity, c.stream));
        PCS_CUDA(launch_items(a, c.stream));
        PCS_CUDA(cudaStreamSynchronize(c.stream));

        const uint32_t B = std::max<uint32_t>(c.rb_max_b_, 1u);
        std::vector<Candidate> grid;
        const uint32_t blocks[] = {128, 256, 512, 1024};
        const uint32_t ppts[] = {1, 2, 4, 8};
        const uint32_t tiles[] = {0, 32, 64, 128, 256};
        for (uint32_t b : blocks)
            for (uint32_t pp : ppts)
                for (uint32_t t : tiles)
                    for (uint32_t g = 0; g < 2; ++g) {
                        if (t == 0 && g == 1) continue;
                        if ((size_t)t * B * 4u > 200u * 1024u) continue;
                        if (b > sim_max_block((int)pp)) continue; /* above the build's launch bound */
                        if (t > job.R) continue;
                        if (c.split_walk() && (pp != 1u || b != 256u)) continue; /* fixed shape */
                        SimLaunch l{0, b, (int)pp, false, g != 0, c.split_walk()};
                        if (simulate_occupancy(l, t * B) < 1) continue;
                        grid.push_back({b, pp, t, g});
                    }
        Candidate best{c.tune.block, c.tune.ppt, c.tune.tile_rows, c.tune.aggregate};
        float best_ms = time_config(c, best, 2);
        for (const Candidate& k : grid) {
            const float ms = time_config(c, k, 2);
            if (ms < best_ms) {
                best_ms = ms;
                best = k;
            }
        }
        c.tune.block = best.block;
        c.tune.ppt = best.ppt;
        c.tune.tile_rows = best.tile_rows;
        c.tune.aggregate = best.agg;
        c.graph_dirty = true;
    } catch (...) {
        c.retire(&job);
        throw;
    }
    c.retire(&job);
    if (chosen) {
        chosen->block_size = c.tune.block;
        chosen->particles_per_thread = c.tune.ppt;
        chosen->hist_tile_rows = c.tune.tile_rows;
        chosen->warp_aggregate = c.tune.aggregate;
        chosen->chunk_particles = c.tune.chunk;
        chosen->round_capacity = c.tune.capacity;
        chosen->max_speculation = c.tune.max_spec;
        chosen->use_graphs = c.tune.use_graphs;
    }
}

} // namespace pcs

extern "C" pcs_status pcs_autotune(pcs_ctx* ctx, const pcs_params* p, const pcs_observed* obs, pcs_tuning* chosen);

namespace pcs {
void set_last_error(const std::string& m);
}

extern "C" pcs_status pcs_autotune(pcs_ctx* ctx, const pcs_params* p, const pcs_observed* obs, pcs_tuning* chosen)
{
    try {
        if (!ctx || !p || !obs) throw pcs::Error(PCS_ERR_INVALID_ARGUMENT, "ctx/params/observed is NULL");
        PCS_CUDA(cudaSetDevice(ctx->impl->device));
        pcs::autotune(*ctx->impl, *p, *obs, chosen);
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
