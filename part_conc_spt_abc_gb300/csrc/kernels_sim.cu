/*
 * kernels_sim.cu -- the fused forward model: simulate + summarise.
 *
 * One persistent launch walks the particles of every proposal in a round
 * (cusim::K_simulate_system, src/gpu/cusim/kernel-simulate.inl:106-185, and
 * its unrolled twin kernel-simulate-unroll.inl:69-298, do one proposal per
 * launch with one warp per video).  Work items are (proposal, range of
 * particles) pulled from a device counter, so proposals with uneven Poisson
 * particle counts pack densely onto all SMs.  Per particle the walk state
 * lives in registers; each track's (K, DE) goes to a histogram whose first
 * rows are privatised in shared memory (flushed with red.global.add after
 * each item) and whose remaining rows take global atomics.
 *
 * Arithmetic contract: the walk, DE and binning use explicit round-to-nearest
 * intrinsics (__fmul_rn/__fadd_rn/__fdiv_rn) in the reference's evaluation
 * order, so given the same draws the histogram is bit-exact with the
 * reference kernel built without FMA contraction.
 *
 * Random draws: Philox4x32-10, counter (particle, tag|block, slot,
 * generation|trial) with the job seed folded into words 2 and 3; the rounds'
 * work on the words that stay fixed for a particle is done once per particle
 * (pcs_philox_prepare); block 0 = position and
 * component, block 1 = size, blocks 2+3g..4+3g = the 12 normals of walk steps
 * 4g+1..4g+4 (Box-Muller on word pairs).  In replay mode the same kernel
 * reads pre-generated draws instead.
 */
#include <cuda_runtime.h>

#include <algorithm>

#include "pcs_common.h"
#include "pcs_kernels.h"

namespace pcs {

namespace {

__device__ __forceinline__ float wrap_(float v, float m, float two_m)
{
    /* periodic_bounds_ (kernel-simulate.inl:95-103): one wrap, v -= 2 copysign(m, v) */
    return (fabsf(v) > m) ? __fsub_rn(v, copysignf(two_m, v)) : v;
}

/* The three wraps of one step.  A step is much shorter than the box, so a
 * wrap is rare: one combined test skips the three selects on the common
 * path (same values as three wrap_ calls). */
__device__ __forceinline__ void wrap3_(float& x, float& y, float& z, float hx, float hy, float hz, float tx,
                                       float ty, float tz)
{
    if (__builtin_expect(fabsf(x) > hx || fabsf(y) > hy || fabsf(z) > hz, 0)) {
        x = wrap_(x, hx, tx);
        y = wrap_(y, hy, ty);
        z = wrap_(z, hz, tz);
    }
}

/* The PTX approximate instructions in their flush-to-zero forms.  Box-Muller
 * never gives them a subnormal operand (u >= 2^-33; -2 ln u is 0 or above
 * 5e-8; the angle is 0 or above 1e-7 in magnitude), so they return what the
 * non-flushing forms (__log2f, __sincosf in a build without -ftz) return,
 * without the subnormal handling those carry: ~10% fewer instructions per
 * particle-step for the same normals. */
__device__ __forceinline__ float lg2_ftz_(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float sqrt_ftz_(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float sin_ftz_(float x)
{
    float y;
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float cos_ftz_(float x)
{
    float y;
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

const float kSqrt2Ln2 = 1.1774100225154747f; /* sqrt(2 ln 2): sqrt(-2 ln u) = sqrt(2 ln 2) sqrt(-log2 u) */

/* Box-Muller on two 32-bit words: u1 in (0,1], angle uniform on [-pi, pi);
 * both normals times scale = rscale / sqrt(2 ln 2).  The radius is
 * rscale sqrt(-log2 u): a caller that scales every pair by the same factor
 * (the walk: its particle's step sd, so its steps take the normals as they
 * are) folds sqrt(2 ln 2) into it once, one multiply per pair fewer. */
__device__ __forceinline__ void box_muller_r_(uint32_t ra, uint32_t rb, float& n0, float& n1, float rscale)
{
    float u = __fmaf_rn(__uint2float_rn(ra), 2.3283064365386963e-10f, 1.1641532182693481e-10f);
    float rad = rscale * sqrt_ftz_(-lg2_ftz_(u));
    float t = __fmaf_rn(__uint2float_rn(rb), 1.4629180792671596e-09f, -3.14159265358979f);
    n0 = rad * sin_ftz_(t);
    n1 = rad * cos_ftz_(t);
}

/* unit normals */
__device__ __forceinline__ void box_muller_(uint32_t ra, uint32_t rb, float& n0, float& n1)
{
    box_muller_r_(ra, rb, n0, n1, kSqrt2Ln2);
}

struct Walker {
    float x, y, z, de, sd, haz; /* sd: the step sd, or (fresh-draw walk) sd x sqrt(2 ln 2) for box_muller_r_ */
    uint32_t k, F, n;  /* n: particle index within the proposal */
    pcs_philox_pre ph; /* the particle's stream with its fixed counter words folded in */
};

struct ItemCtx {
    float hlx, hly, hlz, two_hlx, two_hly, two_hlz, hax, hay, four_dt, dde;
    uint32_t kmin, B, RB, tile_words_used, tile_rows;
    uint32_t* hist; /* global histogram of the proposal */
    uint32_t* err;
};

/* HistogramRecorder::record (histogram2d.inl:313-321) into the privatised
 * tile or the global histogram. */
template <bool AGG>
__device__ __noinline__ void record_out_(float four_dt, float dde, uint32_t B, uint32_t RB,
                                         uint32_t tile_rows, uint32_t* hist, uint32_t* err,
                                         uint32_t* tile, uint32_t k, float de)
{
    float denom = __fmul_rn(__uint2float_rn(k - 1u), four_dt);
    float DE = __fdiv_rn(de, denom);
    float q = __fdiv_rn(DE, dde);
    uint32_t bin = __float2uint_rz(q); /* tCount(aDE / mDDE): truncating, saturating, NaN -> 0 */
    if (bin >= B) return;
    uint64_t idx = (uint64_t)k * B + bin;
    if (idx >= RB) {
        atomicOr(err, PCS_ERRBIT_HIST_BOUNDS);
        return;
    }
    if (k < tile_rows) {
        if (AGG) {
            unsigned mask = __activemask();
            unsigned peers = __match_any_sync(mask, (unsigned)idx);
            int leader = __ffs(peers) - 1;
            if ((int)(threadIdx.x & 31u) == leader) atomicAdd(&tile[idx], (uint32_t)__popc(peers));
        } else {
            atomicAdd(&tile[idx], 1u);
        }
    } else {
        atomicAdd(&hist[idx], 1u);
    }
}

template <bool AGG>
__device__ __forceinline__ void record_(const ItemCtx& c, uint32_t* tile, uint32_t k, float de)
{
    record_out_<AGG>(c.four_dt, c.dde, c.B, c.RB, c.tile_rows, c.hist, c.err, tile, k, de);
}

/* One frame of the walk.  CHECK: the frame may lie past the particle's
 * last one (s >= F) and is then skipped; full groups of four frames call it
 * without the test.  SCALED: the normals already carry the step sd (fresh
 * Philox draws); replayed normals are unit normals, scaled here as the
 * reference scales them. */
template <bool AGG, bool CHECK = true, bool SCALED = false>
__device__ __forceinline__ void step_(const ItemCtx& c, uint32_t* tile, Walker& w, uint32_t s,
                                      float n0, float n1, float n2)
{
    if (CHECK && s >= w.F) return;
    float dx = SCALED ? n0 : __fmul_rn(w.sd, n0);
    float dy = SCALED ? n1 : __fmul_rn(w.sd, n1);
    float dz = SCALED ? n2 : __fmul_rn(w.sd, n2);
    w.x = __fadd_rn(w.x, dx);
    w.y = __fadd_rn(w.y, dy);
    w.z = __fadd_rn(w.z, dz);
    wrap3_(w.x, w.y, w.z, c.hlx, c.hly, c.hlz, c.two_hlx, c.two_hly, c.two_hlz);
    /* kernel-simulate.inl:70-93: a detected step extends the track (DE from
     * its second frame on), an undetected one closes it (recorded if K >=
     * kmin).  (Updating the track state by selects instead keeps all lanes
     * together but executes ~6% more instructions: no faster.) */
    bool det = fabsf(w.z) <= w.haz && fabsf(w.x) <= c.hax && fabsf(w.y) <= c.hay;
    if (det) {
        uint32_t kp = w.k + 1u;
        if (kp >= 2u) w.de = __fadd_rn(w.de, __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
        w.k = kp;
    } else {
        if (w.k >= c.kmin) record_<AGG>(c, tile, w.k, w.de);
        w.k = 0u;
        w.de = 0.0f;
    }
}

/* wrand_index (utility.inl:8-57). */
__device__ __forceinline__ uint32_t wrand_index_(float u, uint32_t C, const float* pre)
{
    if (C == 2u) return (pre[0] >= u) ? 0u : 1u;
    uint32_t bot = 0, top = C;
    while (bot != top) {
        uint32_t mid = (top + bot) >> 1;
        if (pre[mid] <= u)
            bot = mid + 1u;
        else
            top = mid;
    }
    return bot;
}

__device__ __forceinline__ uint32_t video_of_(const uint32_t* prefix, uint32_t V, uint32_t n)
{
    /* largest v with prefix[v] <= n (prefix[0] = 0, prefix[V] = total) */
    uint32_t lo = 0, hi = V;
    while (hi - lo > 1u) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= n)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

/* Item context of proposal s_prop (of job s_job). */
__device__ __forceinline__ ItemCtx item_ctx_(const SimArgs& a, const JobDev& s_job, const PropDev& s_prop)
{
    ItemCtx c;
    c.hlx = s_job.half_lx;
    c.hly = s_job.half_ly;
    c.hlz = s_job.half_lz;
    c.two_hlx = 2.0f * s_job.half_lx;
    c.two_hly = 2.0f * s_job.half_ly;
    c.two_hlz = 2.0f * s_job.half_lz;
    c.hax = s_job.half_ax;
    c.hay = s_job.half_ay;
    c.four_dt = s_job.four_delta_t;
    c.dde = s_job.dde;
    c.kmin = s_job.kmin;
    c.B = s_job.B;
    c.RB = s_job.R * s_job.B;
    c.tile_rows = min(s_job.R, a.tile_words / max(s_job.B, 1u));
    c.tile_words_used = c.tile_rows * s_job.B;
    c.hist = a.hist + s_prop.hist_off;
    c.err = a.err;
    return c;
}

/* Loads work item `item`'s proposal and job blocks into shared memory. */
__device__ __forceinline__ void load_item_(const SimArgs& a, uint32_t item, PropDev& s_prop, JobDev& s_job)
{
    const uint32_t tid = threadIdx.x;
    const uint32_t p = a.item_prop[item];
    if (tid < sizeof(PropDev) / 4) reinterpret_cast<uint32_t*>(&s_prop)[tid] = reinterpret_cast<const uint32_t*>(a.props + p)[tid];
    __syncthreads();
    if (tid < sizeof(JobDev) / 4) reinterpret_cast<uint32_t*>(&s_job)[tid] = reinterpret_cast<const uint32_t*>(a.jobs + s_prop.job)[tid];
    __syncthreads();
}

/* Initial state of particle n (make_particle, utility.inl:60-99, and the
 * particle's step sd): position, component, half depth, step sd, K.
 * BM_SD: q.sd carries sd x sqrt(2 ln 2), the scale box_muller_r_ takes. */
template <bool REPLAY, bool BM_SD = false>
__device__ __forceinline__ void init_walker_(const SimArgs& a, const ItemCtx& c, const JobDev& s_job,
                                             const PropDev& s_prop, const uint32_t* prefix, uint32_t n,
                                             uint32_t slot, uint32_t gt, uint32_t k0, uint32_t k1, Walker& q)
{
    const uint32_t V = s_job.V, C = s_job.C, model = s_job.model;
    const uint32_t v = video_of_(prefix, V, n);
    q.F = __ldg(s_job.frames + v);
    float u0, u1, u2, u3;
    if (REPLAY) {
        const float* u = a.rp_uniforms + 4ull * n;
        u0 = u[0];
        u1 = u[1];
        u2 = u[2];
        u3 = u[3];
    } else {
        q.ph = pcs_philox_prepare(n, slot, gt, k0, k1);
        pcs_u4 r = pcs_draw_pre(q.ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, 0u));
        u0 = pcs_u01_24(r.x);
        u1 = pcs_u01_24(r.y);
        u2 = pcs_u01_24(r.z);
        u3 = pcs_u01_24(r.w);
    }
    /* make_particle (utility.inl:60-99): halfL * (2u - 1) */
    q.x = __fmul_rn(c.hlx, __fsub_rn(2.0f * u0, 1.0f));
    q.y = __fmul_rn(c.hly, __fsub_rn(2.0f * u1, 1.0f));
    q.z = __fmul_rn(c.hlz, __fsub_rn(2.0f * u2, 1.0f));
    uint32_t comp = (C > 1u) ? wrand_index_(u3, C, s_prop.pre_comp_prob) : 0u;
    if (comp >= C) {
        atomicOr(a.err, PCS_ERRBIT_COMPONENT);
        comp = C - 1u;
    }
    q.haz = (model == PCS_DEV_MODEL_VARIABLE_Z) ? s_prop.half_az[comp] : s_prop.half_az[0];
    if (model == PCS_DEV_MODEL_LOGNORMAL) {
        if (REPLAY) {
            q.sd = a.rp_sigmas[n];
        } else {
            pcs_u4 r = pcs_draw_pre(q.ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, 1u));
            float z0, z1;
            box_muller_(r.x, r.y, z0, z1);
            q.sd = s_prop.sd_scale[comp] * expf(s_prop.sd_shape[comp] * z0);
        }
    } else {
        q.sd = s_prop.sd_scale[comp];
    }
    if (BM_SD) q.sd = __fmul_rn(q.sd, kSqrt2Ln2);
    const bool det = fabsf(q.z) <= q.haz && fabsf(q.x) <= c.hax && fabsf(q.y) <= c.hay;
    q.k = det ? 1u : 0u;
}

/* The 12 normals of the group of frames s0 .. s0+3: Philox blocks
 * 2+3g .. 4+3g through Box-Muller, times the particle's step sd (q.sd holds
 * sd x sqrt(2 ln 2) on this path); or the replayed unit normals (zeros past
 * F). */
template <bool REPLAY>
__device__ __forceinline__ void group_normals_(const SimArgs& a, const Walker& q, uint32_t s0, float* nn)
{
    if (REPLAY) {
        const float* src = a.rp_normals + ((uint64_t)q.n * a.rp_stride + (s0 - 1u)) * 3u;
        const uint32_t rem = min(4u, q.F - s0);
#pragma unroll
        for (int t = 0; t < 12; ++t) nn[t] = ((uint32_t)t < rem * 3u) ? src[t] : 0.0f;
    } else {
        const uint32_t g = (s0 - 1u) >> 2;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            pcs_u4 r = pcs_draw_pre(q.ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, 2u + 3u * g + (uint32_t)b));
            box_muller_r_(r.x, r.y, nn[4 * b + 0], nn[4 * b + 1], q.sd);
            box_muller_r_(r.z, r.w, nn[4 * b + 2], nn[4 * b + 3], q.sd);
        }
    }
}

/* Frames 1 .. F-1 of one walker, four per group: the full groups skip the
 * per-frame end test, the tail group keeps it. */
template <bool REPLAY, bool AGG>
__device__ __forceinline__ void walk_single_(const SimArgs& a, const ItemCtx& c, uint32_t* tile, Walker& q)
{
    uint32_t s0 = 1;
    for (; s0 + 3u < q.F; s0 += 4u) {
        float nn[12];
        group_normals_<REPLAY>(a, q, s0, nn);
        step_<AGG, false, !REPLAY>(c, tile, q, s0 + 0u, nn[0], nn[1], nn[2]);
        step_<AGG, false, !REPLAY>(c, tile, q, s0 + 1u, nn[3], nn[4], nn[5]);
        step_<AGG, false, !REPLAY>(c, tile, q, s0 + 2u, nn[6], nn[7], nn[8]);
        step_<AGG, false, !REPLAY>(c, tile, q, s0 + 3u, nn[9], nn[10], nn[11]);
    }
    if (s0 < q.F) {
        float nn[12];
        group_normals_<REPLAY>(a, q, s0, nn);
        step_<AGG, true, !REPLAY>(c, tile, q, s0 + 0u, nn[0], nn[1], nn[2]);
        step_<AGG, true, !REPLAY>(c, tile, q, s0 + 1u, nn[3], nn[4], nn[5]);
        step_<AGG, true, !REPLAY>(c, tile, q, s0 + 2u, nn[6], nn[7], nn[8]);
        step_<AGG, true, !REPLAY>(c, tile, q, s0 + 3u, nn[9], nn[10], nn[11]);
    }
}

/* Work without a shared-memory histogram tile (every record a global
 * atomic): nothing ties a CTA's warps to one work item, so each warp takes
 * its own 32-particle slice of an item from the queue (slice s is part
 * s % slices of item s / slices) and no CTA barrier is needed.  Same walkers,
 * same draws, same records as the CTA loop. */
template <bool AGG>
__device__ __noinline__ void simulate_warp_slices_(const SimArgs& a)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t slices = (a.chunk + 31u) / 32u;
    const uint32_t n_slices = *a.n_items * slices;
    for (;;) {
        uint32_t sl = 0u;
        if (lane == 0u) sl = atomicAdd(a.queue_head, 1u);
        sl = __shfl_sync(0xFFFFFFFFu, sl, 0);
        if (sl >= n_slices) break;
        const uint32_t item = sl / slices, part = sl - item * slices;
        const PropDev& prop = a.props[a.item_prop[item]];
        const JobDev& job = a.jobs[prop.job];
        const ItemCtx c = item_ctx_(a, job, prop);
        const uint32_t i0 = (item - prop.item_begin) * a.chunk;
        const uint32_t i1 = min(i0 + a.chunk, prop.total_particles);
        const uint32_t n = i0 + part * 32u + lane;
        if (n < i1) {
            Walker q;
            q.n = n;
            q.F = 0;
            q.k = 0;
            q.de = 0.0f;
            q.x = q.y = q.z = 0.0f;
            q.sd = 0.0f;
            q.haz = 0.0f;
            init_walker_<false, true>(a, c, job, prop, a.counts + prop.counts_off + job.V, n, prop.slot,
                                pcs_ctr_gen_trial(prop.gen, prop.trial), job.seed_lo, job.seed_hi, q);
            walk_single_<false, AGG>(a, c, nullptr, q);
            if (q.F > 0u && q.k >= c.kmin) record_<AGG>(c, nullptr, q.k, q.de);
        }
    }
}

} // namespace

/* Launch bound by walkers per thread: one walker keeps 64 registers for
 * 1024-thread CTAs; 2, 4 and 8 interleaved walkers get 128 (512 threads) and
 * 255 (256 threads) registers, so their walk state stays out of local
 * memory. */
template <int PPT, bool REPLAY, bool AGG>
__global__ void __launch_bounds__(sim_max_block(PPT)) k_simulate(SimArgs a)
{
    extern __shared__ uint32_t s_tile[];
    __shared__ uint32_t s_item;
    __shared__ PropDev s_prop;
    __shared__ JobDev s_job;

    if (!REPLAY && PPT == 1 && a.tile_words == 0u) {
        simulate_warp_slices_<AGG>(a);
        return;
    }
    const uint32_t tid = threadIdx.x, bd = blockDim.x;
    for (uint32_t i = tid; i < a.tile_words; i += bd) s_tile[i] = 0u;
    const uint32_t n_items = *a.n_items;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(a.queue_head, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= n_items) break;
        load_item_(a, item, s_prop, s_job);
        const ItemCtx c = item_ctx_(a, s_job, s_prop);

        const uint32_t V = s_job.V;
        const uint32_t* prefix = a.counts + s_prop.counts_off + V; /* [V+1] */
        const uint32_t k0 = s_job.seed_lo, k1 = s_job.seed_hi;
        const uint32_t slot = s_prop.slot;
        const uint32_t gt = pcs_ctr_gen_trial(s_prop.gen, s_prop.trial);

        const uint32_t chunk_idx = item - s_prop.item_begin;
        const uint32_t a0 = chunk_idx * a.chunk;
        const uint32_t a1 = min(a0 + a.chunk, s_prop.total_particles);

        for (uint32_t base = a0; base < a1; base += bd * PPT) {
            Walker w[PPT];
            uint32_t fmax = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                const uint32_t n = base + tid + (uint32_t)j * bd;
                Walker& q = w[j];
                q.n = n;
                q.F = 0;
                q.k = 0;
                q.de = 0.0f;
                q.x = q.y = q.z = 0.0f;
                q.sd = 0.0f;
                q.haz = 0.0f;
                if (n < a1) {
                    init_walker_<REPLAY, !REPLAY>(a, c, s_job, s_prop, prefix, n, slot, gt, k0, k1, q);
                    fmax = max(fmax, q.F);
                }
            }

            /* frames 1 .. F-1, four per group; one walker per thread: the
             * full groups skip the per-frame end test, the tail group keeps it */
            if (PPT == 1) {
                walk_single_<REPLAY, AGG>(a, c, s_tile, w[0]);
            } else
            for (uint32_t s0 = 1; s0 < fmax; s0 += 4u) {
#pragma unroll
                for (int j = 0; j < PPT; ++j) {
                    Walker& q = w[j];
                    if (s0 >= q.F) continue;
                    float nn[12];
                    group_normals_<REPLAY>(a, q, s0, nn);
                    step_<AGG, true, !REPLAY>(c, s_tile, q, s0 + 0u, nn[0], nn[1], nn[2]);
                    step_<AGG, true, !REPLAY>(c, s_tile, q, s0 + 1u, nn[3], nn[4], nn[5]);
                    step_<AGG, true, !REPLAY>(c, s_tile, q, s0 + 2u, nn[6], nn[7], nn[8]);
                    step_<AGG, true, !REPLAY>(c, s_tile, q, s0 + 3u, nn[9], nn[10], nn[11]);
                }
            }
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                if (w[j].F > 0u && w[j].k >= c.kmin) record_<AGG>(c, s_tile, w[j].k, w[j].de);
            }
        }

        __syncthreads();
        /* flush the privatised rows into the proposal's histogram */
        for (uint32_t i = tid; i < c.tile_words_used; i += bd) {
            const uint32_t v = s_tile[i];
            if (v) {
                atomicAdd(c.hist + i, v);
                s_tile[i] = 0u;
            }
        }
    }
}

/* ----------------------------------------------------------------------- */
/* The slab-split walk (k_simulate_split).
 *
 * Same model as k_simulate, fewer draws: a particle can only be detected
 * while its z lies in the detection slab (|z| <= half depth), and the x, y
 * steps taken while z is outside it matter only through their sum.  Steps
 * go in groups of four (m <= 4 in the last group).  The CTA (256 threads,
 * one particle each) works in chunks of kSplitG groups, in three phases
 * separated by barriers:
 *   Z  every thread walks z step by step exactly (four normals per group)
 *      and moves x, y by the group's summed displacement S = sd sqrt(m) n;
 *      a group with any z in the slab becomes a task in the CTA's queue;
 *   T  the CTA's threads take the queued tasks densely: a task draws its
 *      group's x, y steps conditioned on their sum (Gaussian bridge,
 *      d_i = S/m + sd (n_i - mean n), exactly i.i.d. N(0, sd^2) again),
 *      walks them from the group's start and stores each step's detection
 *      bit and dx^2 + dy^2;
 *   S  each thread runs the reference's track bookkeeping
 *      (kernel-simulate.inl:70-93) over its groups in time order; a group
 *      without a task is undetected from its first step.
 * The joint law of the positions at every frame is the per-step walk's, so
 * the histograms have the same distribution (from different draws); the
 * CPU oracle's orc_simulate_philox_split follows the same blocks and
 * arithmetic.  Philox blocks of particle n per group pair h (groups 2h,
 * 2h+1): 2+8h z(2h), 3+8h z(2h+1), 4+8h both groups' sums, 5+8h..6+8h the
 * x, y steps of group 2h, 7+8h..8+8h those of group 2h+1. */

constexpr uint32_t kSplitThreads = 256;
constexpr uint32_t kSplitG = 6; /* groups per chunk: even, so group pairs stay in one chunk */
constexpr uint32_t kSplitCap = kSplitThreads * kSplitG;

struct SplitShared {
    float xs[kSplitCap], ys[kSplitCap], sx[kSplitCap], sy[kSplitCap]; /* in; out: dx^2 + dy^2 per step */
    float sd[kSplitCap];
    uint32_t meta[kSplitCap]; /* owner << 16 | group-in-chunk << 8 | m << 4 | in-slab bits (detection bits out) */
    uint16_t idx[kSplitG][kSplitThreads]; /* task of (group-in-chunk, thread) */
    uint32_t count;
};

namespace {

__device__ __forceinline__ float split_sqrt_m_(uint32_t m)
{
    return m == 4u ? 2.0f : (m == 3u ? 1.73205080757f : (m == 2u ? 1.41421356237f : 1.0f));
}

__device__ __forceinline__ float split_inv_m_(uint32_t m)
{
    return m == 4u ? 0.25f : (m == 3u ? 0.333333333333f : (m == 2u ? 0.5f : 1.0f));
}

template <bool AGG>
__device__ __forceinline__ void close_track_(const ItemCtx& c, uint32_t* tile, Walker& q)
{
    if (q.k >= c.kmin) record_<AGG>(c, tile, q.k, q.de);
    q.k = 0u;
    q.de = 0.0f;
}

} // namespace

template <bool AGG>
__global__ void __launch_bounds__(kSplitThreads, 4) k_simulate_split(SimArgs a)
{
    extern __shared__ uint32_t s_tile[];
    __shared__ uint32_t s_item, s_gmax;
    __shared__ PropDev s_prop;
    __shared__ JobDev s_job;

    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    SplitShared& sh = *reinterpret_cast<SplitShared*>(s_tile + a.tile_words);
    for (uint32_t i = tid; i < a.tile_words; i += kSplitThreads) s_tile[i] = 0u;
    const uint32_t n_items = *a.n_items;
    unsigned long long tasks_total = 0ull;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(a.queue_head, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= n_items) break;
        load_item_(a, item, s_prop, s_job);
        const ItemCtx c = item_ctx_(a, s_job, s_prop);
        const uint32_t* prefix = a.counts + s_prop.counts_off + s_job.V; /* [V+1] */
        const uint32_t k0 = s_job.seed_lo, k1 = s_job.seed_hi;
        const uint32_t slot = s_prop.slot;
        const uint32_t gt = pcs_ctr_gen_trial(s_prop.gen, s_prop.trial);
        const uint32_t chunk_idx = item - s_prop.item_begin;
        const uint32_t a0 = chunk_idx * a.chunk;
        const uint32_t a1 = min(a0 + a.chunk, s_prop.total_particles);

        for (uint32_t base = a0; base < a1; base += kSplitThreads) {
            const uint32_t n = base + tid;
            Walker q;
            q.n = n;
            q.F = 0u;
            q.k = 0u;
            q.de = 0.0f;
            q.x = q.y = q.z = 0.0f;
            q.sd = 0.0f;
            q.haz = 0.0f;
            if (n < a1) init_walker_<false>(a, c, s_job, s_prop, prefix, n, slot, gt, k0, k1, q);
            const uint32_t steps = q.F > 0u ? q.F - 1u : 0u;
            const uint32_t groups = (steps + 3u) >> 2;
            if (tid == 0) {
                s_gmax = 0u;
                sh.count = 0u;
            }
            __syncthreads();
            atomicMax(&s_gmax, groups);
            __syncthreads();
            const uint32_t gmax = s_gmax;

            for (uint32_t g0 = 0; g0 < gmax; g0 += kSplitG) {
                /* ---- phase Z: z per step, x, y per group, tasks queued ---- */
                uint32_t fullmask = 0u;
#pragma unroll 1
                for (uint32_t gl = 0; gl < kSplitG; gl += 2u) {
                    const uint32_t g = g0 + gl; /* even */
                    float nz[8], ag[4];
                    if (g < groups) {
                        const uint32_t blk0 = 2u + 8u * (g >> 1);
                        const pcs_u4 r0 = pcs_draw_pre(q.ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, blk0));
                        const pcs_u4 r1 = pcs_draw_pre(q.ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, blk0 + 1u));
                        const pcs_u4 r2 = pcs_draw_pre(q.ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, blk0 + 2u));
                        box_muller_(r0.x, r0.y, nz[0], nz[1]);
                        box_muller_(r0.z, r0.w, nz[2], nz[3]);
                        box_muller_(r1.x, r1.y, nz[4], nz[5]);
                        box_muller_(r1.z, r1.w, nz[6], nz[7]);
                        box_muller_(r2.x, r2.y, ag[0], ag[1]);
                        box_muller_(r2.z, r2.w, ag[2], ag[3]);
                    }
#pragma unroll
                    for (uint32_t h = 0; h < 2u; ++h) {
                        const uint32_t gg = g + h;
                        uint32_t zbits = 0u, m = 0u;
                        float xs = 0.0f, ys = 0.0f, sx = 0.0f, sy = 0.0f;
                        if (gg < groups) {
                            m = min(4u, steps - 4u * gg);
#pragma unroll
                            for (uint32_t i = 0; i < 4u; ++i) {
                                if (i < m) {
                                    const float dz = __fmul_rn(q.sd, nz[4u * h + i]);
                                    q.z = wrap_(__fadd_rn(q.z, dz), c.hlz, c.two_hlz);
                                    if (fabsf(q.z) <= q.haz) zbits |= 1u << i;
                                }
                            }
                            const float sds = __fmul_rn(q.sd, split_sqrt_m_(m));
                            sx = __fmul_rn(sds, ag[2u * h]);
                            sy = __fmul_rn(sds, ag[2u * h + 1u]);
                            xs = q.x;
                            ys = q.y;
                            q.x = wrap_(__fadd_rn(q.x, sx), c.hlx, c.two_hlx);
                            q.y = wrap_(__fadd_rn(q.y, sy), c.hly, c.two_hly);
                        }
                        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, zbits != 0u);
                        if (bal) {
                            uint32_t wbase = 0u;
                            if (lane == 0u) wbase = atomicAdd(&sh.count, (uint32_t)__popc(bal));
                            wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0);
                            if (zbits) {
                                const uint32_t e = wbase + (uint32_t)__popc(bal & lt_mask);
                                sh.xs[e] = xs;
                                sh.ys[e] = ys;
                                sh.sx[e] = sx;
                                sh.sy[e] = sy;
                                sh.sd[e] = q.sd;
                                sh.meta[e] = (tid << 16) | ((gl + h) << 8) | (m << 4) | zbits;
                                sh.idx[gl + h][tid] = (uint16_t)e;
                                fullmask |= 1u << (gl + h);
                            }
                        }
                    }
                }
                __syncthreads();
                /* ---- phase T: the queued tasks, densely ---- */
                const uint32_t cnt = sh.count;
                for (uint32_t e = tid; e < cnt; e += kSplitThreads) {
                    const uint32_t meta = sh.meta[e];
                    const uint32_t owner = meta >> 16, gl = (meta >> 8) & 0xFFu, m = (meta >> 4) & 7u;
                    const uint32_t zbits = meta & 15u, g = g0 + gl;
                    const float xs = sh.xs[e], ys = sh.ys[e], sxv = sh.sx[e], syv = sh.sy[e], sd = sh.sd[e];
                    const pcs_philox_pre ph = pcs_philox_prepare(base + owner, slot, gt, k0, k1);
                    const uint32_t blk = 2u + 8u * (g >> 1) + 3u + 2u * (g & 1u);
                    float nx[4], ny[4];
                    pcs_u4 r = pcs_draw_pre(ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, blk));
                    box_muller_(r.x, r.y, nx[0], ny[0]);
                    box_muller_(r.z, r.w, nx[1], ny[1]);
                    r = pcs_draw_pre(ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, blk + 1u));
                    box_muller_(r.x, r.y, nx[2], ny[2]);
                    box_muller_(r.z, r.w, nx[3], ny[3]);
                    const float im = split_inv_m_(m);
                    float mx = 0.0f, my = 0.0f;
#pragma unroll
                    for (uint32_t i = 0; i < 4u; ++i) {
                        if (i < m) {
                            mx = __fadd_rn(mx, nx[i]);
                            my = __fadd_rn(my, ny[i]);
                        }
                    }
                    mx = __fmul_rn(mx, im);
                    my = __fmul_rn(my, im);
                    const float cx = __fmul_rn(sxv, im), cy = __fmul_rn(syv, im);
                    float xx = xs, yy = ys, dv[4];
                    uint32_t det = 0u;
#pragma unroll
                    for (uint32_t i = 0; i < 4u; ++i) {
                        dv[i] = 0.0f;
                        if (i < m) {
                            const float dx = __fadd_rn(cx, __fmul_rn(sd, __fsub_rn(nx[i], mx)));
                            const float dy = __fadd_rn(cy, __fmul_rn(sd, __fsub_rn(ny[i], my)));
                            xx = wrap_(__fadd_rn(xx, dx), c.hlx, c.two_hlx);
                            yy = wrap_(__fadd_rn(yy, dy), c.hly, c.two_hly);
                            if (((zbits >> i) & 1u) && fabsf(xx) <= c.hax && fabsf(yy) <= c.hay) det |= 1u << i;
                            dv[i] = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
                        }
                    }
                    sh.xs[e] = dv[0];
                    sh.ys[e] = dv[1];
                    sh.sx[e] = dv[2];
                    sh.sy[e] = dv[3];
                    sh.meta[e] = (meta & ~15u) | det;
                }
                tasks_total += cnt;
                __syncthreads();
                if (tid == 0) sh.count = 0u;
                /* ---- phase S: track bookkeeping over this thread's groups ---- */
                const uint32_t have = groups > g0 ? min(groups - g0, kSplitG) : 0u; /* groups of this chunk */
                uint32_t bits = fullmask, pos = 0u;
                while (bits) {
                    const uint32_t gl = (uint32_t)__ffs(bits) - 1u;
                    bits &= bits - 1u;
                    if (gl > pos) close_track_<AGG>(c, s_tile, q); /* groups without a task before it */
                    const uint32_t e = sh.idx[gl][tid];
                    const uint32_t meta = sh.meta[e];
                    const uint32_t m = (meta >> 4) & 7u;
                    const float dv[4] = {sh.xs[e], sh.ys[e], sh.sx[e], sh.sy[e]};
#pragma unroll
                    for (uint32_t i = 0; i < 4u; ++i) {
                        if (i < m) {
                            if ((meta >> i) & 1u) {
                                const uint32_t kp = q.k + 1u;
                                if (kp >= 2u) q.de = __fadd_rn(q.de, dv[i]);
                                q.k = kp;
                            } else {
                                close_track_<AGG>(c, s_tile, q);
                            }
                        }
                    }
                    pos = gl + 1u;
                }
                if (have > pos) close_track_<AGG>(c, s_tile, q); /* groups without a task after the last */
                __syncthreads();
            }
            if (q.F > 0u && q.k >= c.kmin) record_<AGG>(c, s_tile, q.k, q.de);
        }

        __syncthreads();
        /* flush the privatised rows into the proposal's histogram */
        for (uint32_t i = tid; i < c.tile_words_used; i += kSplitThreads) {
            const uint32_t v = s_tile[i];
            if (v) {
                atomicAdd(c.hist + i, v);
                s_tile[i] = 0u;
            }
        }
    }
    if (a.tasks && tid == 0u && tasks_total) atomicAdd(a.tasks, tasks_total);
}

/* ----------------------------------------------------------------------- */

namespace {
template <int PPT, bool REPLAY, bool AGG>
cudaError_t launch_sim_(const SimArgs& a, uint32_t grid, uint32_t block, size_t smem, cudaStream_t st)
{
    auto fn = k_simulate<PPT, REPLAY, AGG>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

template <int PPT, bool REPLAY, bool AGG>
int occupancy_(uint32_t block, size_t smem)
{
    int n = 0;
    auto fn = k_simulate<PPT, REPLAY, AGG>;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, (int)block, smem) != cudaSuccess) return 0;
    return n;
}

template <bool AGG>
cudaError_t launch_split_(const SimArgs& a, uint32_t grid, size_t smem, cudaStream_t st)
{
    auto fn = k_simulate_split<AGG>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<grid, kSplitThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <bool AGG>
int occupancy_split_(size_t smem)
{
    int n = 0;
    auto fn = k_simulate_split<AGG>;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, (int)kSplitThreads, smem) != cudaSuccess) return 0;
    return n;
}

/* The split walk's task queue follows the histogram tile in shared memory;
 * the tile gives way so that both fit in 220 KB. */
uint32_t split_tile_words_(uint32_t tile_words)
{
    const size_t cap = (220u * 1024u - sizeof(SplitShared)) / 4u;
    return (uint32_t)(tile_words < cap ? tile_words : cap);
}
} // namespace

cudaError_t launch_simulate(const SimArgs& a_in, const SimLaunch& l, cudaStream_t st)
{
    if (l.split) {
        if (l.replay) return cudaErrorInvalidValue;
        SimArgs a = a_in;
        a.tile_words = split_tile_words_(a.tile_words);
        const size_t smem = (size_t)a.tile_words * 4u + sizeof(SplitShared);
        return l.aggregate ? launch_split_<true>(a, l.grid, smem, st) : launch_split_<false>(a, l.grid, smem, st);
    }
    const SimArgs& a = a_in;
    const size_t smem = (size_t)a.tile_words * 4u;
#define PCS_SIM_CASE(P, R, G)                                                               \
    if (l.ppt == P && l.replay == R && l.aggregate == G) return launch_sim_<P, R, G>(a, l.grid, l.block, smem, st);
    PCS_SIM_CASE(1, false, false)
    PCS_SIM_CASE(1, false, true)
    PCS_SIM_CASE(2, false, false)
    PCS_SIM_CASE(2, false, true)
    PCS_SIM_CASE(4, false, false)
    PCS_SIM_CASE(4, false, true)
    PCS_SIM_CASE(8, false, false)
    PCS_SIM_CASE(8, false, true)
    PCS_SIM_CASE(1, true, false)
    PCS_SIM_CASE(1, true, true)
#undef PCS_SIM_CASE
    return cudaErrorInvalidValue;
}

int simulate_occupancy(const SimLaunch& l, uint32_t tile_words)
{
    if (l.split) {
        const size_t smem = (size_t)split_tile_words_(tile_words) * 4u + sizeof(SplitShared);
        return l.aggregate ? occupancy_split_<true>(smem) : occupancy_split_<false>(smem);
    }
    const size_t smem = (size_t)tile_words * 4u;
#define PCS_SIM_OCC(P, R, G) \
    if (l.ppt == P && l.replay == R && l.aggregate == G) return occupancy_<P, R, G>(l.block, smem);
    PCS_SIM_OCC(1, false, false)
    PCS_SIM_OCC(1, false, true)
    PCS_SIM_OCC(2, false, false)
    PCS_SIM_OCC(2, false, true)
    PCS_SIM_OCC(4, false, false)
    PCS_SIM_OCC(4, false, true)
    PCS_SIM_OCC(8, false, false)
    PCS_SIM_OCC(8, false, true)
    PCS_SIM_OCC(1, true, false)
    PCS_SIM_OCC(1, true, true)
#undef PCS_SIM_OCC
    return 0;
}

/* Raw stream words for the counter-layout check. */
__global__ void k_debug_stream(uint32_t k0, uint32_t k1, uint32_t slot, uint32_t gt, uint32_t n,
                               uint32_t j, uint32_t* out)
{
    pcs_u4 r = pcs_draw(n, pcs_ctr_tag(PCS_STREAM_PARTICLE, j), slot, gt, k0, k1);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}

cudaError_t launch_debug_stream(uint64_t seed, uint32_t slot, uint32_t gen, uint32_t trial,
                                uint32_t particle, uint32_t block, uint32_t* d_out, cudaStream_t st)
{
    uint32_t m0 = 0, m1 = 0;
    pcs_seed_masks(seed, &m0, &m1);
    k_debug_stream<<<1, 1, 0, st>>>(m0, m1, slot, pcs_ctr_gen_trial(gen, trial), particle, block, d_out);
    return cudaGetLastError();
}

} // namespace pcs
