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

#include "pcs_common.h"
#include "pcs_kernels.h"

namespace pcs {

namespace {

__device__ __forceinline__ float wrap_(float v, float m, float two_m)
{
    /* periodic_bounds_ (kernel-simulate.inl:95-103): one wrap, v -= 2 copysign(m, v) */
    return (fabsf(v) > m) ? __fsub_rn(v, copysignf(two_m, v)) : v;
}

/* Box-Muller on two 32-bit words: u1 in (0,1], angle uniform on [-pi, pi). */
__device__ __forceinline__ void box_muller_(uint32_t ra, uint32_t rb, float& n0, float& n1)
{
    float u = __fmaf_rn(__uint2float_rn(ra), 2.3283064365386963e-10f, 1.1641532182693481e-10f);
    float x = -1.3862943611198906f * __log2f(u); /* -2 ln u */
    float rad = x * rsqrtf(fmaxf(x, 1e-30f));
    float t = __fmaf_rn(__uint2float_rn(rb), 1.4629180792671596e-09f, -3.14159265358979f);
    float s, c;
    __sincosf(t, &s, &c);
    n0 = rad * s;
    n1 = rad * c;
}

struct Walker {
    float x, y, z, de, sd, haz;
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

template <bool AGG>
__device__ __forceinline__ void step_(const ItemCtx& c, uint32_t* tile, Walker& w, uint32_t s,
                                      float n0, float n1, float n2)
{
    if (s >= w.F) return;
    float dx = __fmul_rn(w.sd, n0);
    w.x = wrap_(__fadd_rn(w.x, dx), c.hlx, c.two_hlx);
    float dy = __fmul_rn(w.sd, n1);
    w.y = wrap_(__fadd_rn(w.y, dy), c.hly, c.two_hly);
    float dz = __fmul_rn(w.sd, n2);
    w.z = wrap_(__fadd_rn(w.z, dz), c.hlz, c.two_hlz);
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

} // namespace

template <int PPT, bool REPLAY, bool AGG>
__global__ void __launch_bounds__(1024) k_simulate(SimArgs a)
{
    extern __shared__ uint32_t s_tile[];
    __shared__ uint32_t s_item;
    __shared__ PropDev s_prop;
    __shared__ JobDev s_job;

    const uint32_t tid = threadIdx.x, bd = blockDim.x;
    for (uint32_t i = tid; i < a.tile_words; i += bd) s_tile[i] = 0u;
    const uint32_t n_items = *a.n_items;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(a.queue_head, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= n_items) break;
        const uint32_t p = a.item_prop[item];
        if (tid < sizeof(PropDev) / 4) reinterpret_cast<uint32_t*>(&s_prop)[tid] = reinterpret_cast<const uint32_t*>(a.props + p)[tid];
        __syncthreads();
        if (tid < sizeof(JobDev) / 4) reinterpret_cast<uint32_t*>(&s_job)[tid] = reinterpret_cast<const uint32_t*>(a.jobs + s_prop.job)[tid];
        __syncthreads();

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

        const uint32_t V = s_job.V;
        const uint32_t C = s_job.C;
        const uint32_t model = s_job.model;
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
                    bool det = fabsf(q.z) <= q.haz && fabsf(q.x) <= c.hax && fabsf(q.y) <= c.hay;
                    q.k = det ? 1u : 0u;
                    fmax = max(fmax, q.F);
                }
            }

            /* frames 1 .. F-1, four per group */
            for (uint32_t s0 = 1; s0 < fmax; s0 += 4u) {
                const uint32_t g = (s0 - 1u) >> 2;
#pragma unroll
                for (int j = 0; j < PPT; ++j) {
                    Walker& q = w[j];
                    if (s0 >= q.F) continue;
                    float nn[12];
                    if (REPLAY) {
                        const float* src = a.rp_normals + ((uint64_t)q.n * a.rp_stride + (s0 - 1u)) * 3u;
                        const uint32_t rem = min(4u, q.F - s0);
#pragma unroll
                        for (int t = 0; t < 12; ++t) nn[t] = ((uint32_t)t < rem * 3u) ? src[t] : 0.0f;
                    } else {
#pragma unroll
                        for (int b = 0; b < 3; ++b) {
                            pcs_u4 r = pcs_draw_pre(q.ph, pcs_ctr_tag(PCS_STREAM_PARTICLE, 2u + 3u * g + (uint32_t)b));
                            box_muller_(r.x, r.y, nn[4 * b + 0], nn[4 * b + 1]);
                            box_muller_(r.z, r.w, nn[4 * b + 2], nn[4 * b + 3]);
                        }
                    }
                    step_<AGG>(c, s_tile, q, s0 + 0u, nn[0], nn[1], nn[2]);
                    step_<AGG>(c, s_tile, q, s0 + 1u, nn[3], nn[4], nn[5]);
                    step_<AGG>(c, s_tile, q, s0 + 2u, nn[6], nn[7], nn[8]);
                    step_<AGG>(c, s_tile, q, s0 + 3u, nn[9], nn[10], nn[11]);
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
} // namespace

cudaError_t launch_simulate(const SimArgs& a, const SimLaunch& l, cudaStream_t st)
{
    const size_t smem = (size_t)a.tile_words * 4u;
#define PCS_SIM_CASE(P, R, G)                                                               \
    if (l.ppt == P && l.replay == R && l.aggregate == G) return launch_sim_<P, R, G>(a, l.grid, l.block, smem, st);
    PCS_SIM_CASE(1, false, false)
    PCS_SIM_CASE(1, false, true)
    PCS_SIM_CASE(2, false, false)
    PCS_SIM_CASE(2, false, true)
    PCS_SIM_CASE(4, false, false)
    PCS_SIM_CASE(4, false, true)
    PCS_SIM_CASE(1, true, false)
    PCS_SIM_CASE(1, true, true)
#undef PCS_SIM_CASE
    return cudaErrorInvalidValue;
}

int simulate_occupancy(const SimLaunch& l, uint32_t tile_words)
{
    const size_t smem = (size_t)tile_words * 4u;
#define PCS_SIM_OCC(P, R, G) \
    if (l.ppt == P && l.replay == R && l.aggregate == G) return occupancy_<P, R, G>(l.block, smem);
    PCS_SIM_OCC(1, false, false)
    PCS_SIM_OCC(1, false, true)
    PCS_SIM_OCC(2, false, false)
    PCS_SIM_OCC(2, false, true)
    PCS_SIM_OCC(4, false, false)
    PCS_SIM_OCC(4, false, true)
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
