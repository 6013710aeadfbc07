/*
 * kernels_pmc.cu -- the ABC-PMC step on the device.
 *
 * The reference runs the population Monte Carlo loop on the host in double
 * (SimulationT::run, src/gpu/detail/simulation_impl.inl:178-455): per slot it
 * picks a parent by weight (wrand_idx_ :54-62), perturbs every parameter with
 * a reflected Gaussian (displace_ :64-79), sorts components by m to avoid
 * label switching (:276-303), draws Poisson particle counts (:307-317), ships
 * one proposal per launch and retries the slot until dist <= gamma; at the
 * end of a generation it reweights (:832-887), updates tau (:733-749) and
 * lowers gamma.  Here the same steps run as kernels over all pending slots of
 * all jobs in a round:
 *
 *   k_round_plan   shares the round's proposal capacity among the jobs
 *                  (trials per pending slot k = capacity / pending, clamped)
 *   k_propose      one warp per proposal: parent pick, perturbation,
 *                  label sort, per-proposal forward-model arguments, Poisson
 *                  counts per video (transformed rejection, Hoermann 1993)
 *   k_items        scan of work items and the item -> proposal map
 *   k_accept       per job: first accepted trial of every slot, trial
 *                  accounting, compaction of the pending list
 *   k_whiten       coordinates of old/new populations in the metric of the
 *                  perturbation kernel (double -> float, centred)
 *   k_kernel_sum   pmc-standard importance weights: log-sum-exp over the old
 *                  population in FP32
 *   k_finalize     per job: weight normalisation (FP64), commit, tau or
 *                  weighted covariance + Cholesky (FP64), gamma update
 *
 * Every random draw is Philox keyed by (seed, generation, slot, trial), so a
 * job's result does not depend on the round capacity or on which other jobs
 * share its rounds.
 */
#include <cuda_runtime.h>
#include <math.h>

#include "pcs_common.h"
#include "pcs_kernels.h"
#include "pcs_proposal.h"

namespace pcs {

namespace {

__device__ uint32_t job_of_(const RoundDev* rd, uint32_t q)
{
    uint32_t j = 0;
    for (uint32_t i = 1; i < rd->n_jobs; ++i)
        if (rd->job_base[i] <= q && rd->job_count[i] > 0) j = i;
    /* job_base is non-decreasing; pick the last job whose range contains q */
    for (uint32_t i = 0; i < rd->n_jobs; ++i)
        if (q >= rd->job_base[i] && q < rd->job_base[i] + rd->job_count[i]) return i;
    return j;
}

} // namespace

/* ----------------------------------------------------------------------- */
__global__ void k_round_plan(PmcArgs a)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    RoundDev* rd = a.round;
    uint64_t total_pending = 0;
    for (uint32_t j = 0; j < rd->n_jobs; ++j) {
        const JobPmcDev& pm = a.pmc[j];
        if (!pm.done) total_pending += pm.pending_count;
    }
    uint32_t k = total_pending ? (uint32_t)(rd->capacity / total_pending) : 1u;
    if (k < 1u) k = 1u;
    if (k > rd->max_spec) k = rd->max_spec;
    /* trials per pending slot: enough to fill the round, but not many more
     * than ~0.3 / (acceptance rate so far), so that few trials are simulated
     * after a slot's first acceptance -- unless the round's proposals would
     * then carry fewer than `fill` particles (one wave of the simulate
     * launch; at the end of a generation few slots are left and the GPU
     * would idle), in which case the slots get proportionally more trials,
     * up to k.  Particles per proposal are estimated from the job's history. */
    uint32_t kjs[kMaxRoundJobs];
    double planned = 0.0;
    uint64_t pend_spec = 0;
    for (uint32_t j = 0; j < rd->n_jobs && j < kMaxRoundJobs; ++j) {
        const JobPmcDev& pm = a.pmc[j];
        uint32_t kj = k;
        if (pm.generation == 0u) {
            kj = 1u; /* prior pass: one simulation per slot */
        } else {
            const double pacc = ((double)pm.accepted_gen + 1.0) / ((double)pm.trials + 2.0);
            const double kw = ceil(0.3 / pacc);
            if (kw < (double)kj) kj = (uint32_t)(kw < 1.0 ? 1.0 : kw);
            if (!pm.done) pend_spec += pm.pending_count;
        }
        kjs[j] = kj;
        if (!pm.done) {
            /* particles per proposal so far (steps over the longest video) */
            const double ppp = pm.simulations ? (double)pm.particle_steps / (double)pm.simulations /
                                                    (double)max(a.jobs[j].frames_max, 1u)
                                              : (double)rd->fill;
            planned += (double)pm.pending_count * kj * ppp;
        }
    }
    if (rd->fill && planned < (double)rd->fill && pend_spec > 0) {
        const double f = planned > 0.0 ? (double)rd->fill / planned : (double)k;
        for (uint32_t j = 0; j < rd->n_jobs && j < kMaxRoundJobs; ++j)
            if (a.pmc[j].generation > 0u && !a.pmc[j].done)
                kjs[j] = (uint32_t)min((double)k, fmax((double)kjs[j], ceil((double)kjs[j] * f)));
    }
    /* the order in which jobs take the round's capacity: admission order, or
     * (order == 1) jobs in their prior pass first, then the least estimated
     * remaining work first -- (pending slots + slots of the generations left)
     * x particle-steps per proposal / acceptance rate -- which lets short
     * jobs finish early instead of waiting behind long ones */
    uint32_t ord[kMaxRoundJobs];
    double key[kMaxRoundJobs];
    const uint32_t nj = min(rd->n_jobs, kMaxRoundJobs);
    for (uint32_t j = 0; j < nj; ++j) {
        const JobPmcDev& pm = a.pmc[j];
        double kv = (double)j;
        if (rd->order == 1u && pm.generation > 0u && !pm.done) {
            const double pacc = ((double)pm.accepted_gen + 1.0) / ((double)pm.trials + 2.0);
            const double spp = pm.simulations ? (double)pm.particle_steps / (double)pm.simulations : 1.0;
            const double gens_left =
                pm.max_generations ? fmax(0.0, (double)pm.max_generations - (double)pm.iterations) : 8.0;
            kv = 1e6 + ((double)pm.pending_count + (double)pm.N * gens_left) * spp / pacc;
        }
        key[j] = kv;
        uint32_t x = j;
        while (x > 0 && key[ord[x - 1]] > kv) {
            ord[x] = ord[x - 1];
            --x;
        }
        ord[x] = j;
    }
    for (uint32_t j = nj; j < rd->n_jobs; ++j) {
        rd->job_base[j] = 0u;
        rd->job_count[j] = 0u;
        rd->job_k[j] = 1u;
        rd->job_hist_base[j] = 0u;
    }
    uint32_t base = 0;
    uint64_t hbase = 0, cells = 0;
    for (uint32_t o = 0; o < nj; ++o) {
        const uint32_t j = ord[o];
        const JobPmcDev& pm = a.pmc[j];
        const uint32_t kj = kjs[j];
        uint64_t want = pm.done ? 0u : (uint64_t)pm.pending_count * kj;
        uint64_t room = rd->capacity - base;
        const uint64_t rb = (uint64_t)a.jobs[j].R * a.jobs[j].B;
        if (rb) {
            /* each job's histograms start at a multiple of R x B words, so
             * one tensor map (B x R x histograms over the whole area) reaches
             * every histogram of the job */
            hbase = (hbase + rb - 1u) / rb * rb;
            const uint64_t hroom = hbase < rd->hist_cap ? (rd->hist_cap - hbase) / rb : 0u;
            if (hroom < room) room = hroom;
        }
        uint64_t cnt = want < room ? want : room;
        cnt -= cnt % kj; /* whole slots only */
        rd->job_base[j] = base;
        rd->job_k[j] = kj;
        rd->job_count[j] = (uint32_t)cnt;
        rd->job_hist_base[j] = hbase;
        base += (uint32_t)cnt;
        hbase += cnt * rb;
        cells += cnt * rb;
    }
    rd->n_props = base;
    rd->n_items = 0u;
    rd->queue_head = 0u;
    rd->round_steps = 0ull;
    rd->round_cells = cells;
}

/* ----------------------------------------------------------------------- */
/* First index i < N with !(wcum[i] < u) (std::lower_bound on a
 * non-decreasing array), clamped to N - 1, as pcs_pick: a 32-way search, each
 * lane probing one split point per round (2 dependent loads for N = 1024
 * instead of 10). */
__device__ __forceinline__ uint32_t warp_pick_(const double* wcum, uint32_t N, double u, uint32_t lane)
{
    uint32_t lo = 0, hi = N; /* the answer lies in [lo, hi]; hi == N: none found yet */
    for (int round = 0; round < 8 && hi > lo; ++round) {
        const uint32_t span = hi - lo;
        uint32_t idx;
        bool valid;
        if (span <= 32u) {
            idx = lo + lane;
            valid = lane < span;
        } else {
            idx = lo + (uint32_t)(((uint64_t)(lane + 1u) * span) / 32u) - 1u;
            valid = true;
        }
        const bool ge = valid && !(wcum[idx] < u);
        const unsigned m = __ballot_sync(0xFFFFFFFFu, ge);
        if (m == 0u) {
            lo = hi;
            break;
        }
        const uint32_t f = (uint32_t)(__ffs(m) - 1);
        const uint32_t idx_f = __shfl_sync(0xFFFFFFFFu, idx, f);
        if (span <= 32u) {
            lo = hi = idx_f;
            break;
        }
        const uint32_t prev = __shfl_sync(0xFFFFFFFFu, idx, f > 0u ? f - 1u : 0u);
        lo = f > 0u ? prev + 1u : lo;
        hi = idx_f;
    }
    return lo < N ? lo : N - 1u;
}

/* One warp per proposal.  The FP64 work is spread over the lanes: lane i
 * draws perturbation normal pair i, lane p perturbs and reflects parameter p,
 * lane c computes component c's arguments (10^log10c, step sd); the Poisson
 * constants are computed once and the lanes draw the per-video counts in
 * parallel (each count has its own Philox counter) and scan them into the
 * video prefix.  Every value is the one pcs_build_theta / pcs_build_args /
 * pcs_draw_counts compute (same functions, same operation order). */
constexpr uint32_t kProposeWarps = 8;

__global__ void __launch_bounds__(32 * kProposeWarps) k_propose(PmcArgs a)
{
    RoundDev* rd = a.round;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t q = blockIdx.x * kProposeWarps + (threadIdx.x >> 5);
    if (q >= rd->n_props) return; /* whole warp */
    const uint32_t j = job_of_(rd, q);
    JobPmcDev& pm = a.pmc[j];
    const JobDev& jd = a.jobs[j];
    const uint32_t k = rd->job_k[j];
    const uint32_t local = q - rd->job_base[j];
    const uint32_t pend_idx = local / k, rep = local % k;
    const uint32_t slot = pm.pending[pend_idx];
    const uint32_t trial = pm.next_trial[slot] + rep;
    const uint32_t gen = pm.generation;
    const uint32_t k0 = jd.seed_lo, k1 = jd.seed_hi;
    const uint32_t P = pm.P;
    const uint32_t gt = pcs_ctr_gen_trial(gen, trial);

    /* parameters: lane p holds parameter p */
    double th_l = 0.0;
    if (gen == 0u) {
        if (lane < P) th_l = pm.theta[(uint64_t)slot * P + lane];
    } else {
        const pcs_u4 r = pcs_draw(0u, pcs_ctr_tag(PCS_STREAM_PICK, 0u), slot, gt, k0, k1);
        const uint32_t parent = warp_pick_(pm.wcum, pm.N, pcs_u01_53(r.x, r.y), lane);
        const double* tp = pm.theta + (uint64_t)parent * P;
        double n0 = 0.0, n1 = 0.0;
        if (2u * lane < P) {
            const pcs_u4 rr = pcs_draw(lane, pcs_ctr_tag(PCS_STREAM_PERTURB, 0u), slot, gt, k0, k1);
            pcs_normal2(rr, n0, n1);
        }
        double nrm[PCS_MAX_P];
        for (uint32_t i = 0; i < P; ++i) { /* P is the same on every lane */
            const double a0 = __shfl_sync(0xFFFFFFFFu, n0, i >> 1);
            const double a1 = __shfl_sync(0xFFFFFFFFu, n1, i >> 1);
            nrm[i] = (i & 1u) ? a1 : a0;
        }
        if (lane < P) th_l = pcs_perturb_one(pm, tp, pm.factor, nrm, lane);
    }
    double th[PCS_MAX_P];
    for (uint32_t i = 0; i < P; ++i) th[i] = __shfl_sync(0xFFFFFFFFu, th_l, i);
    if (gen != 0u) pcs_sort_components(pm, th);

    /* per-component arguments: lane c computes component c */
    CompArgs ca_l;
    ca_l.powc = 0.0;
    ca_l.sd_scale = ca_l.sd_shape = 0.0f;
    if (lane < pm.C) ca_l = pcs_comp_args(pm, th, lane);
    CompArgs ca[PCS_MAX_C];
    for (uint32_t i = 0; i < pm.C; ++i) {
        ca[i].powc = __shfl_sync(0xFFFFFFFFu, ca_l.powc, i);
        ca[i].sd_scale = __shfl_sync(0xFFFFFFFFu, ca_l.sd_scale, i);
        ca[i].sd_shape = __shfl_sync(0xFFFFFFFFu, ca_l.sd_shape, i);
    }
    PropDev pd;
    pd.job = j;
    pd.slot = slot;
    pd.trial = trial;
    pd.gen = gen;
    pd.hist_z = 0u;
    const double lambda = pcs_assemble_args(pm, th, ca, gen, pd);
    if (lane == 0u) {
        double* out = a.theta_prop + (uint64_t)q * PCS_MAX_P;
        for (uint32_t p = 0; p < P; ++p) out[p] = th[p];
    }

    PoissonSetup ps = pcs_poisson_setup(lambda);
    ps.logfact = a.logfact;
    ps.logfact_n = a.logfact_n;
    const uint64_t coff = (uint64_t)q * (2u * rd->v_max + 1u);
    uint32_t* cnt = a.counts + coff;
    uint32_t* pre = cnt + jd.V;
    uint64_t run = 0, steps = 0;
    if (lane == 0u) pre[0] = 0u;
    for (uint32_t v0 = 0; v0 < jd.V; v0 += 32u) {
        const uint32_t v = v0 + lane;
        uint32_t c = 0u;
        if (v < jd.V) {
            c = pcs_poisson_draw(ps, v, slot, gt, k0, k1);
            cnt[v] = c;
            steps += (uint64_t)c * jd.frames[v];
        }
        uint64_t incl = c;
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if ((int)lane >= d) incl += t;
        }
        const uint64_t tot = run + incl;
        if (v < jd.V) pre[v + 1] = (uint32_t)(tot < 0xFFFFFFFFull ? tot : 0xFFFFFFFFull);
        run += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    for (int d = 16; d >= 1; d >>= 1) steps += __shfl_xor_sync(0xFFFFFFFFu, steps, d);
    if (lane != 0u) return;
    const uint64_t total = run;
    if (total > 0xFFFFFFFFull) atomicOr(a.err, PCS_ERRBIT_COUNTS);
    pd.total_particles = (uint32_t)min(total, (uint64_t)0xFFFFFFFFu);
    pd.counts_off = coff;
    pd.hist_off = rd->job_hist_base[j] + (uint64_t)local * ((uint64_t)jd.R * jd.B);
    /* the job's histograms start at a multiple of R x B words (k_round_plan) */
    pd.hist_z = (uint32_t)(pd.hist_off / max(1ull, (unsigned long long)jd.R * jd.B));
    pd.item_count = (pd.total_particles + rd->chunk - 1u) / rd->chunk;
    pd.item_begin = 0u;
    a.props[q] = pd;
    atomicAdd((unsigned long long*)&pm.particle_steps, (unsigned long long)steps);
    atomicAdd(&a.round->round_steps, (unsigned long long)steps);
}

/* ----------------------------------------------------------------------- */
/* item scan: one block */
__global__ void __launch_bounds__(1024) k_items(PmcArgs a)
{
    __shared__ uint32_t s_part[1024];
    RoundDev* rd = a.round;
    const uint32_t M = rd->n_props;
    const uint32_t per = (M + blockDim.x - 1) / blockDim.x;
    const uint32_t b = threadIdx.x * per, e = min(b + per, M);
    uint32_t sum = 0;
    for (uint32_t q = b; q < e; ++q) sum += a.props[q].item_count;
    s_part[threadIdx.x] = sum;
    __syncthreads();
    for (uint32_t d = 1; d < blockDim.x; d <<= 1) {
        uint32_t t = (threadIdx.x >= d) ? s_part[threadIdx.x - d] : 0u;
        __syncthreads();
        s_part[threadIdx.x] += t;
        __syncthreads();
    }
    uint32_t run = s_part[threadIdx.x] - sum;
    for (uint32_t q = b; q < e; ++q) {
        a.props[q].item_begin = run;
        run += a.props[q].item_count;
    }
    const uint32_t total = s_part[blockDim.x - 1];
    const uint32_t cap = rd->items_cap;
    __syncthreads(); /* every proposal's item_begin is written */
    if (threadIdx.x == 0) {
        if (total > cap) atomicOr(a.err, PCS_ERRBIT_ITEMS);
        rd->n_items = min(total, cap);
        rd->queue_head = 0u;
    }
    /* the item -> proposal map: a warp per proposal, its lanes on
     * consecutive items (coalesced stores) */
    const uint32_t lane = threadIdx.x & 31u, nw = blockDim.x >> 5;
    for (uint32_t q = threadIdx.x >> 5; q < M; q += nw) {
        const uint32_t ib = a.props[q].item_begin, ic = a.props[q].item_count;
        for (uint32_t i = lane; i < ic; i += 32u)
            if (ib + i < cap) a.item_prop[ib + i] = q;
    }
}

/* ----------------------------------------------------------------------- */
/* accept: one block per job */
__global__ void __launch_bounds__(1024) k_accept(PmcArgs a)
{
    __shared__ uint32_t s_keep, s_exhausted;
    __shared__ unsigned long long s_trials, s_acc;
    const uint32_t j = blockIdx.x;
    RoundDev* rd = a.round;
    if (j >= rd->n_jobs) return;
    JobPmcDev& pm = a.pmc[j];
    if (pm.done) return;
    const uint32_t k = rd->job_k[j];
    const uint32_t cnt = rd->job_count[j];
    const uint32_t base = rd->job_base[j];
    const uint32_t nprop_slots = cnt / k;
    const uint32_t npend = pm.pending_count;
    const uint32_t P = pm.P;
    if (threadIdx.x == 0) {
        s_keep = 0u;
        s_exhausted = 0u;
        s_trials = 0ull;
        s_acc = 0ull;
        pm.gen_ended = 0u;
    }
    __syncthreads();
    /* decide every pending slot; kept slots go to scratch (as u32 bits) */
    uint32_t* keep_list = reinterpret_cast<uint32_t*>(pm.scratch);
    for (uint32_t i = threadIdx.x; i < npend; i += blockDim.x) {
        const uint32_t slot = pm.pending[i];
        bool acc_ok = false;
        if (i < nprop_slots) {
            uint32_t first = k;
            double dsel = 0.0;
            for (uint32_t r = 0; r < k; ++r) {
                const uint32_t q = base + i * k + r;
                const double df = a.use_f64_distance && a.dist_f64 ? a.dist_f64[q] : (double)a.dist_f32[q];
                const double d = log10(df);
                if (pm.generation == 0u || d <= pm.gamma) {
                    first = r;
                    dsel = d;
                    break;
                }
            }
            if (first < k) {
                const uint32_t q = base + i * k + first;
                for (uint32_t p = 0; p < P; ++p)
                    pm.theta_new[(uint64_t)slot * P + p] = a.theta_prop[(uint64_t)q * PCS_MAX_P + p];
                pm.dist_new[slot] = dsel;
                pm.accepted[slot] = 1u;
                acc_ok = true;
                atomicAdd(&s_trials, (unsigned long long)(first + 1u));
                atomicAdd(&s_acc, 1ull);
            } else {
                pm.next_trial[slot] += k;
                atomicAdd(&s_trials, (unsigned long long)k);
                /* the trial ordinal has 20 bits in the random-stream counter:
                 * a slot that exhausts them ends the generation like the
                 * trial cap does (converged) */
                if (pm.next_trial[slot] + rd->max_spec >= (1u << 20)) s_exhausted = 1u;
            }
        }
        if (!acc_ok) keep_list[atomicAdd(&s_keep, 1u)] = slot;
    }
    __syncthreads();
    const uint32_t nk = s_keep;
    for (uint32_t i = threadIdx.x; i < nk; i += blockDim.x) pm.pending[i] = keep_list[i];
    if (threadIdx.x == 0) {
        pm.pending_count = nk;
        pm.trials += s_trials;
        pm.simulations += cnt;
        pm.accepted_total += s_acc;
        pm.accepted_gen += s_acc;
        if (s_exhausted && pm.generation > 0u) pm.trials = (uint64_t)pm.avg_trials * pm.N;
        const bool cap = pm.generation > 0u &&
                         (double)pm.trials >= (double)pm.avg_trials * (double)pm.N;
        if (nk == 0u || cap) pm.gen_ended = 1u;
    }
}

/* ----------------------------------------------------------------------- */
/* whitened coordinates for the kernel density: y = A^-1 (theta - mean),
 * A = diag(tau) or the Cholesky factor; fixed parameters dropped.  Output
 * float [2][N][P] in the job's ybuf (old population, then new). */
__device__ __forceinline__ bool needs_kernel_sum_(const JobPmcDev& pm)
{
    return !(pm.done || !pm.gen_ended || pm.generation == 0u || pm.weighting != 0u) &&
           !((double)pm.trials >= (double)pm.avg_trials * (double)pm.N);
}

/* y_i = L^-1 (theta_i - lo) (Cholesky) or (theta_i - lo) / tau: point i of
 * the committed (i < N) or new (i >= N) population, whitened. */
__device__ __forceinline__ void whiten_one_(const JobPmcDev& pm, uint32_t i)
{
    const uint32_t N = pm.N, P = pm.P;
    const double* th = (i < N) ? pm.theta + (uint64_t)i * P : pm.theta_new + (uint64_t)(i - N) * P;
    float* y = pm.ybuf + (uint64_t)i * P;
    double v[PCS_MAX_P];
    for (uint32_t p = 0; p < P; ++p) v[p] = th[p] - pm.lo[p];
    if (pm.perturbation == 1u) {
        for (uint32_t p = 0; p < P; ++p) {
            if (pm.fixed[p]) {
                v[p] = 0.0;
                continue;
            }
            double s = v[p];
            for (uint32_t q = 0; q < p; ++q)
                if (!pm.fixed[q]) s -= pm.factor[p * P + q] * v[q];
            v[p] = s / pm.factor[p * P + p];
        }
    } else {
        for (uint32_t p = 0; p < P; ++p) v[p] = pm.fixed[p] ? 0.0 : v[p] / pm.factor[p * P + p];
    }
    for (uint32_t p = 0; p < P; ++p) y[p] = (float)v[p];
}

/* The grid covers one job's 2N points and strides over the round's jobs, so
 * rounds that end no generation launch a few blocks that return at once. */
__global__ void k_whiten(PmcArgs a)
{
    const uint32_t n_jobs = a.round->n_jobs;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        const JobPmcDev& pm = a.pmc[j];
        if (!needs_kernel_sum_(pm)) continue;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 2u * pm.N; i += gridDim.x * blockDim.x)
            whiten_one_(pm, i);
    }
}


/* pmc-standard (simulation_impl.inl:832-871): log w*_a = -log sum_i w_i
 * exp(-0.5 |y*_a - y_i|^2) (the Gaussian normalising constants cancel in
 * the normalisation).  One warp per new particle a. */
__device__ __forceinline__ void kernel_sum_one_(const JobPmcDev& pm, uint32_t an, uint32_t lane);

__global__ void __launch_bounds__(256) k_kernel_sum(PmcArgs a)
{
    const uint32_t n_jobs = a.round->n_jobs;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t j = 0; j < n_jobs; ++j) {
        const JobPmcDev& pm = a.pmc[j];
        if (!needs_kernel_sum_(pm)) continue;
        for (uint32_t an = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; an < pm.N; an += warps)
            kernel_sum_one_(pm, an, lane);
    }
}

/* log w*_an for new particle an, one warp */
__device__ __forceinline__ void kernel_sum_one_(const JobPmcDev& pm, uint32_t an, uint32_t lane)
{
    const uint32_t N = pm.N, P = pm.P;
    const float* yb = pm.ybuf;
    const float* ya = yb + (uint64_t)(N + an) * P;
    float yl[PCS_MAX_P];
    for (uint32_t p = 0; p < P; ++p) yl[p] = ya[p];
    /* pass 1: max exponent; pass 2: scaled sum */
    float mx = -INFINITY;
    for (uint32_t i = lane; i < N; i += 32u) {
        if (!(pm.w[i] > 0.0)) continue;
        const float* yi = yb + (uint64_t)i * P;
        float s = 0.0f;
        for (uint32_t p = 0; p < P; ++p) {
            float d = yl[p] - yi[p];
            s = fmaf(d, d, s);
        }
        mx = fmaxf(mx, -0.5f * s);
    }
    for (int d = 16; d >= 1; d >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, d));
    float acc = 0.0f;
    for (uint32_t i = lane; i < N; i += 32u) {
        const float wi = (float)pm.w[i];
        if (!(wi > 0.0f)) continue;
        const float* yi = yb + (uint64_t)i * P;
        float s = 0.0f;
        for (uint32_t p = 0; p < P; ++p) {
            float d = yl[p] - yi[p];
            s = fmaf(d, d, s);
        }
        acc = fmaf(wi, __expf(-0.5f * s - mx), acc);
    }
    for (int d = 16; d >= 1; d >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, d);
    if (lane == 0) pm.scratch[an] = -(double)mx - log((double)acc); /* log w*_a */
}

/* ----------------------------------------------------------------------- */
/* Order-preserving map of a double to an unsigned key (negative values:
 * all bits flipped; others: the sign bit set), and back. */
__device__ __forceinline__ unsigned long long order_key_(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double from_order_key_(unsigned long long k)
{
    const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double((long long)b);
}

struct SelectShared {
    uint32_t hist[256];
    unsigned long long prefix, mask;
    uint32_t target;
};

/* The value at position `target` (0-based) of x[0..N) in ascending order
 * (nth_element's result, simulation_impl.inl:819-829), by one block: a
 * radix select over the order-preserving keys, eight passes of 8-bit
 * digits from the top; each pass counts the candidates' digits in shared
 * memory (warp-aggregated atomics) and keeps the digit whose bucket holds
 * the target rank.  O(8 N) work instead of comparing all pairs. */
__device__ double select_rank_(const double* x, uint32_t N, uint32_t target, SelectShared& sh)
{
    const uint32_t tid = threadIdx.x, bd = blockDim.x, lane = tid & 31u;
    if (tid == 0) {
        sh.prefix = 0ull;
        sh.mask = 0ull;
        sh.target = target;
    }
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (uint32_t b = tid; b < 256u; b += bd) sh.hist[b] = 0u;
        __syncthreads();
        const unsigned long long prefix = sh.prefix, mask = sh.mask;
        for (uint32_t base = 0; base < N; base += bd) { /* the same trip count for every thread */
            const uint32_t i = base + tid;
            uint32_t digit = 256u; /* no candidate */
            if (i < N) {
                const unsigned long long k = order_key_(x[i]);
                if ((k & mask) == prefix) digit = (uint32_t)(k >> shift) & 255u;
            }
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, digit);
            if (digit < 256u && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&sh.hist[digit], (uint32_t)__popc(peers));
        }
        __syncthreads();
        if (tid < 32u) {
            /* warp 0: lane l owns digits 8l .. 8l+7; find the digit holding the target */
            uint32_t c[8], own = 0u;
            for (int t = 0; t < 8; ++t) {
                c[t] = sh.hist[8u * lane + t];
                own += c[t];
            }
            uint32_t incl = own;
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, d);
                if ((int)lane >= d) incl += v;
            }
            const uint32_t tgt = sh.target, excl = incl - own;
            if (tgt >= excl && tgt < incl) { /* exactly one lane */
                uint32_t run = excl, dsel = 8u * lane;
                for (int t = 0; t < 8; ++t) {
                    if (tgt < run + c[t]) {
                        dsel = 8u * lane + (uint32_t)t;
                        break;
                    }
                    run += c[t];
                }
                sh.target = tgt - run;
                sh.prefix |= (unsigned long long)dsel << shift;
                sh.mask |= 255ull << shift;
            }
        }
        __syncthreads();
    }
    return from_order_key_(sh.prefix);
}

__device__ double block_sum_(double v, double* s_red)
{
    for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
    const uint32_t w = threadIdx.x >> 5, l = threadIdx.x & 31u;
    __syncthreads();
    if (l == 0) s_red[w] = v;
    __syncthreads();
    double t = 0.0;
    const uint32_t nw = blockDim.x >> 5;
    if (w == 0) {
        t = (l < nw) ? s_red[l] : 0.0;
        for (int d = 16; d >= 1; d >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, d);
        if (l == 0) s_red[0] = t;
    }
    __syncthreads();
    t = s_red[0];
    __syncthreads();
    return t;
}

__device__ double block_max_(double v, double* s_red)
{
    for (int d = 16; d >= 1; d >>= 1) v = fmax(v, __shfl_xor_sync(0xFFFFFFFFu, v, d));
    const uint32_t w = threadIdx.x >> 5, l = threadIdx.x & 31u;
    __syncthreads();
    if (l == 0) s_red[w] = v;
    __syncthreads();
    const uint32_t nw = blockDim.x >> 5;
    if (w == 0) {
        double t = (l < nw) ? s_red[l] : -INFINITY;
        for (int d = 16; d >= 1; d >>= 1) t = fmax(t, __shfl_xor_sync(0xFFFFFFFFu, t, d));
        if (l == 0) s_red[0] = t;
    }
    __syncthreads();
    double t = s_red[0];
    __syncthreads();
    return t;
}

/* start of a main iteration (simulation_impl.inl:202-222): count it, stop
 * once -S is exceeded (the count then stays at max + 1, as the reference's
 * meta reports), lower gamma on the delta schedule */
__device__ void start_generation_(JobPmcDev& pm)
{
    pm.iterations += 1u;
    if ((pm.max_generations && pm.iterations > pm.max_generations) || pm.generation >= PCS_MAX_GENERATION) {
        pm.done = 1u;
        return;
    }
    if (pm.schedule == 0u) pm.gamma -= pm.delta_gamma;
    pm.generation += 1u;
    pm.pending_count = pm.N;
    pm.trials = 0ull;
    pm.accepted_gen = 0ull;
    pm.gen_ended = 0u;
}

/* finalize: one block per job whose generation ended this round */
constexpr uint32_t kWcumChunk = 1024;

__global__ void __launch_bounds__(1024) k_finalize(PmcArgs a)
{
    __shared__ double s_red[32];
    __shared__ double s_wc[kWcumChunk];
    __shared__ double s_sel;
    __shared__ double s_mean[PCS_MAX_P];
    __shared__ double s_cov[PCS_MAX_P * PCS_MAX_P];
    __shared__ SelectShared s_select;
    const uint32_t j = blockIdx.x;
    RoundDev* rd = a.round;
    if (j >= rd->n_jobs) return;
    JobPmcDev& pm = a.pmc[j];
    if (pm.done || !pm.gen_ended) return;
    const uint32_t N = pm.N, P = pm.P;
    const uint32_t tid = threadIdx.x, bd = blockDim.x;

    bool commit = true;
    if (pm.generation == 0u) {
        /* prior pass: gamma_0 from the median distance (compute_initial_gamma_ :819-829) */
        const uint32_t target = (pm.schedule == 1u) ? min(N - 1u, (uint32_t)floor(pm.quantile * N)) : N / 2u;
        const double g0 = select_rank_(pm.dist_new, N, target, s_select);
        if (tid == 0) pm.gamma = g0;
        /* the reference keeps the prior population as drawn; the quantile
         * schedule keeps its distances as the generation-0 distances */
        for (uint32_t i = tid; i < N; i += bd) pm.dist[i] = (pm.schedule == 1u) ? pm.dist_new[i] : 0.0;
        commit = false;
    } else if ((double)pm.trials >= (double)pm.avg_trials * (double)pm.N) {
        /* trial cap: converged, discard this generation (:425-428) */
        if (tid == 0) {
            pm.converged = 1u;
            pm.done = 1u;
        }
        return;
    }

    if (commit) {
        /* weights */
        if (pm.weighting == 0u) {
            double mx = -INFINITY;
            for (uint32_t i = tid; i < N; i += bd) mx = fmax(mx, pm.scratch[i]);
            mx = block_max_(mx, s_red);
            double s = 0.0;
            for (uint32_t i = tid; i < N; i += bd) {
                const double e = exp(pm.scratch[i] - mx);
                pm.scratch[i] = e;
                s += e;
            }
            s = block_sum_(s, s_red);
            for (uint32_t i = tid; i < N; i += bd) pm.w[i] = pm.scratch[i] / s;
        } else {
            /* inverse-distance-squared (:872-887) */
            double s = 0.0;
            for (uint32_t i = tid; i < N; i += bd) {
                const double d = pm.dist_new[i];
                const double wv = 1.0 / (d * d);
                pm.scratch[i] = wv;
                s += wv;
            }
            s = block_sum_(s, s_red);
            for (uint32_t i = tid; i < N; i += bd) pm.w[i] = pm.scratch[i] / s;
        }
        /* commit the new population (:434-450) */
        for (uint64_t i = tid; i < (uint64_t)N * P; i += bd) pm.theta[i] = pm.theta_new[i];
        for (uint32_t i = tid; i < N; i += bd) pm.dist[i] = pm.dist_new[i];
        __syncthreads();
    }

    /* cumulative weights (partial_sum, :222): one thread adds them in the
     * reference's order, from a shared-memory copy of each 1024-weight chunk
     * (a chain through global memory would wait for every load in turn) */
    {
        double acc = 0.0; /* thread 0's running sum across chunks */
        for (uint32_t base = 0; base < N; base += kWcumChunk) {
            const uint32_t m = min(kWcumChunk, N - base);
            for (uint32_t i = tid; i < m; i += bd) s_wc[i] = pm.w[base + i];
            __syncthreads();
            if (tid == 0) {
                for (uint32_t i = 0; i < m; ++i) {
                    acc += s_wc[i];
                    s_wc[i] = acc;
                }
            }
            __syncthreads();
            for (uint32_t i = tid; i < m; i += bd) pm.wcum[base + i] = s_wc[i];
            __syncthreads();
        }
    }
    /* perturbation factor from the (new) committed population */
    if (pm.perturbation == 0u) {
        /* compute_tau_ (:733-749): tau = sqrt(2 var), uncorrected 1/N variance */
        for (uint32_t p = 0; p < P; ++p) {
            double s = 0.0;
            for (uint32_t i = tid; i < N; i += bd) s += pm.theta[(uint64_t)i * P + p];
            s = block_sum_(s, s_red);
            const double mean = s / (double)N;
            double v = 0.0;
            for (uint32_t i = tid; i < N; i += bd) {
                const double x = pm.theta[(uint64_t)i * P + p] - mean;
                v += x * x;
            }
            v = block_sum_(v, s_red);
            if (tid == 0) {
                for (uint32_t q = 0; q < P; ++q) pm.factor[p * P + q] = 0.0;
                pm.factor[p * P + p] = sqrt(2.0 * (v / (double)N));
            }
        }
    } else {
        /* 2 x weighted covariance and its Cholesky factor (Beaumont et al. 2009) */
        for (uint32_t p = 0; p < P; ++p) {
            double s = 0.0;
            for (uint32_t i = tid; i < N; i += bd) s += pm.w[i] * pm.theta[(uint64_t)i * P + p];
            s = block_sum_(s, s_red);
            if (tid == 0) s_mean[p] = s;
        }
        __syncthreads();
        for (uint32_t p = 0; p < P; ++p)
            for (uint32_t q = 0; q <= p; ++q) {
                double s = 0.0;
                for (uint32_t i = tid; i < N; i += bd) {
                    const double* t = pm.theta + (uint64_t)i * P;
                    s += pm.w[i] * (t[p] - s_mean[p]) * (t[q] - s_mean[q]);
                }
                s = block_sum_(s, s_red);
                if (tid == 0) s_cov[p * P + q] = s_cov[q * P + p] = 2.0 * s;
            }
        __syncthreads();
        if (tid == 0) {
            for (uint32_t x = 0; x < P * P; ++x) pm.factor[x] = 0.0;
            for (uint32_t c = 0; c < P; ++c) {
                if (pm.fixed[c]) continue;
                double d = s_cov[c * P + c];
                for (uint32_t t = 0; t < c; ++t)
                    if (!pm.fixed[t]) d -= pm.factor[c * P + t] * pm.factor[c * P + t];
                const double lv = sqrt(fmax(d, 1e-300));
                pm.factor[c * P + c] = lv;
                for (uint32_t r = c + 1; r < P; ++r) {
                    if (pm.fixed[r]) continue;
                    double s = s_cov[r * P + c];
                    for (uint32_t t = 0; t < c; ++t)
                        if (!pm.fixed[t]) s -= pm.factor[r * P + t] * pm.factor[c * P + t];
                    pm.factor[r * P + c] = s / lv;
                }
            }
        }
    }
    __syncthreads();

    /* epsilon for the next generation */
    if (pm.schedule == 1u && pm.generation > 0u) {
        const uint32_t target = min(N - 1u, (uint32_t)floor(pm.quantile * N));
        const double eps = select_rank_(pm.dist, N, target, s_select);
        if (tid == 0) s_sel = eps;
        __syncthreads();
    }
    if (tid == 0) {
        if (pm.schedule == 1u && pm.generation > 0u) pm.gamma = s_sel;
        start_generation_(pm);
    }
    for (uint32_t i = tid; i < N; i += bd) {
        pm.pending[i] = i;
        pm.next_trial[i] = 0u;
        pm.accepted[i] = 0u;
    }
}

/* ----------------------------------------------------------------------- */
/* observed cumulative histogram (simulation_impl.inl:605-629) */
__global__ void k_observed_bin(const uint32_t* K, const double* DE, size_t n, uint32_t rows,
                               uint32_t bins, double ub_de, uint32_t* sat, uint32_t* err)
{
    const double width = ub_de / (double)bins;
    const uint64_t total = (uint64_t)rows * bins;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double de = DE[i];
        if (de >= ub_de) continue;
        const long long idx = (long long)(de / width);
        const long long flat = (long long)K[i] * bins + idx;
        if (flat < 0 || (unsigned long long)flat >= total) {
            atomicOr(err, PCS_ERRBIT_HIST_BOUNDS);
            continue;
        }
        atomicAdd(sat + flat, 1u);
    }
}

/* the Julia path's observed histogram (src/cpu/estimate.jl:32-40): kmax
 * rows for K = 1..kmax, bin ceil(DE / width) kept when in 1..bins, i.e.
 * (0, w] bins; a K outside 1..kmax sets the bounds bit (Julia throws). */
__global__ void k_observed_bin_julia(const uint32_t* K, const double* DE, size_t n, uint32_t kmax,
                                     uint32_t bins, double ub_de, uint32_t* sat, uint32_t* err)
{
    const double width = ub_de / (double)bins;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double q = ceil(DE[i] / width);
        if (!(q >= 1.0 && q <= (double)bins)) continue;
        const uint32_t k = K[i];
        if (k < 1u || k > kmax) {
            atomicOr(err, PCS_ERRBIT_HIST_BOUNDS);
            continue;
        }
        atomicAdd(sat + (uint64_t)(k - 1u) * bins + (uint64_t)q - 1u, 1u);
    }
}

/* column-wise then row-wise partial sums; also writes the column-major copy
 * (pairs of columns interleaved, pcs_sat_t_index) */
__global__ void k_observed_cols(uint32_t rows, uint32_t bins, uint32_t* sat)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= bins) return;
    uint32_t acc = 0;
    for (uint32_t r = 0; r < rows; ++r) {
        acc += sat[(uint64_t)r * bins + c];
        sat[(uint64_t)r * bins + c] = acc;
    }
}

__global__ void k_observed_rows(uint32_t rows, uint32_t bins, uint32_t* sat, uint32_t* sat_t)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    uint32_t acc = 0;
    for (uint32_t c = 0; c < bins; ++c) {
        acc += sat[(uint64_t)r * bins + c];
        sat[(uint64_t)r * bins + c] = acc;
        if (sat_t) sat_t[pcs_sat_t_index(r, c, rows, bins)] = acc;
    }
}

/* ----------------------------------------------------------------------- */
cudaError_t launch_round_plan(const PmcArgs& a, cudaStream_t st)
{
    k_round_plan<<<1, 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_propose(const PmcArgs& a, uint32_t capacity, cudaStream_t st)
{
    k_propose<<<(capacity + kProposeWarps - 1) / kProposeWarps, 32 * kProposeWarps, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_items(const PmcArgs& a, cudaStream_t st)
{
    k_items<<<1, 1024, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_accept(const PmcArgs& a, uint32_t n_jobs, cudaStream_t st)
{
    k_accept<<<n_jobs, 1024, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const PmcArgs& a, uint32_t n_jobs, uint32_t max_n, cudaStream_t st)
{
    /* grids for one job's points; the kernels stride over the round's jobs */
    k_whiten<<<(2u * max_n + 255) / 256, 256, 0, st>>>(a);
    k_kernel_sum<<<(max_n * 32u + 255) / 256, 256, 0, st>>>(a);
    k_finalize<<<n_jobs, 1024, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_observed_sat(const uint32_t* K, const double* DE, size_t n, uint32_t rows,
                                uint32_t bins, double ub_de, uint32_t* sat, uint32_t* sat_t,
                                uint32_t* err, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(sat, 0, sizeof(uint32_t) * (size_t)rows * bins, st);
    if (e != cudaSuccess) return e;
    if (n) k_observed_bin<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, st>>>(K, DE, n, rows, bins, ub_de, sat, err);
    k_observed_cols<<<(bins + 127) / 128, 128, 0, st>>>(rows, bins, sat);
    k_observed_rows<<<(rows + 127) / 128, 128, 0, st>>>(rows, bins, sat, sat_t);
    return cudaGetLastError();
}

cudaError_t launch_observed_sat_julia(const uint32_t* K, const double* DE, size_t n, uint32_t kmax,
                                      uint32_t bins, double ub_de, uint32_t* sat, uint32_t* err, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(sat, 0, sizeof(uint32_t) * (size_t)kmax * bins, st);
    if (e != cudaSuccess) return e;
    if (n) k_observed_bin_julia<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, st>>>(K, DE, n, kmax, bins, ub_de, sat, err);
    k_observed_cols<<<(bins + 127) / 128, 128, 0, st>>>(kmax, bins, sat);
    k_observed_rows<<<(kmax + 127) / 128, 128, 0, st>>>(kmax, bins, sat, nullptr);
    return cudaGetLastError();
}

} // namespace pcs
