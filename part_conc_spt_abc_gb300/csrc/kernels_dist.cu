/*
 * kernels_dist.cu -- fused 2-D prefix sum + cumulative distance.
 *
 * Follows cusim::K_distance (src/gpu/cusim/kernel-distance.inl:81-241), which
 * runs one 32x32 block per proposal over the whole R x B histogram twice
 * (row scans, then column scans accumulating (cum - ref)^2) and zeroes the
 * histogram for reuse.  Here one CTA per proposal streams the histogram in
 * strips of 32 DE columns through a shared-memory tile (row pitch 33 words,
 * so row-wise and column-wise accesses are both conflict-free):
 *   k_distance_strip (up to ~1650 rows, 512 threads): the whole strip
 *            height sits in the tile; phase A builds its 2-D prefix sums
 *            (coalesced 128-byte loads, zeros written back, per-lane column
 *            and row passes, per-row carry across strips in shared memory),
 *            phase B
 *            reads column c0+w for logical warp w while lane l accumulates
 *            (float(cum) - float(ref))^2 for rows l, l+32, ..., the observed
 *            cumulative histogram read from its transposed copy (coalesced);
 *   k_distance (taller histograms, 1024 threads): the same in blocks of
 *            256 rows, with the column carry in a register.
 * Warp w / lane l therefore own exactly the columns and rows they own in the
 * reference launch, so the per-lane sums, the shfl_down trees of reduce0
 * (:69-78) and the final per-warp tree reproduce the reference's float
 * result bit for bit (each operation is an explicit round-to-nearest
 * intrinsic, as in a build without FMA contraction).  The exact integer sum
 * of squares and a double-precision sum are accumulated alongside on request.
 */
#include <cuda_runtime.h>

#include "pcs_common.h"
#include "pcs_kernels.h"

namespace pcs {

namespace {

const uint32_t kPad = 33; /* shared tile row pitch: conflict-free column reads */

__device__ __forceinline__ uint32_t warp_scan_(uint32_t v, uint32_t lane)
{
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

__device__ __forceinline__ float reduce0_(float v)
{
    v = __fadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 16));
    v = __fadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 8));
    v = __fadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 4));
    v = __fadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 2));
    v = __fadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 1));
    return v;
}

__device__ __forceinline__ double reduce0_(double v)
{
    v = __dadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 16));
    v = __dadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 8));
    v = __dadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 4));
    v = __dadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 2));
    v = __dadd_rn(v, __shfl_down_sync(0xFFFFFFFFu, v, 1));
    return v;
}

__device__ __forceinline__ void add128_(uint64_t& hi, uint64_t& lo, uint64_t bhi, uint64_t blo)
{
    uint64_t n = lo + blo;
    hi += bhi + (n < lo ? 1u : 0u);
    lo = n;
}

} // namespace

template <bool F64>
__global__ void __launch_bounds__(1024, 1) k_distance(DistArgs a)
{
    extern __shared__ uint32_t s_mem[];
    uint32_t* carry = s_mem;            /* [max_rows] */
    uint32_t* T = s_mem + a.max_rows;   /* [kDistRowBlock][kPad] */
    __shared__ float s_tot[32];
    __shared__ double s_tot64[32];
    __shared__ uint64_t s_hi[32], s_lo[32];

    const uint32_t tid = threadIdx.x;
    const uint32_t w = tid >> 5, l = tid & 31u;
    const uint32_t M = *a.n_props;

    for (uint32_t p = blockIdx.x; p < M; p += gridDim.x) {
        const uint32_t job = a.props[p].job;
        const uint64_t hoff = a.props[p].hist_off;
        const uint32_t R = a.jobs[job].R, B = a.jobs[job].B;
        const uint32_t* refT = a.jobs[job].ref_sat_t;
        uint32_t* hist = a.hist + hoff;
        uint32_t* cum = a.cum_out ? a.cum_out + hoff : nullptr;
        if (R > a.max_rows) {
            if (tid == 0) {
                atomicOr(a.err, PCS_ERRBIT_ROWS);
                a.dist_f32[p] = __int_as_float(0x7fc00000);
            }
            continue;
        }
        for (uint32_t r = tid; r < R; r += blockDim.x) carry[r] = 0u;
        __syncthreads();

        float acc = 0.0f;
        double acc64 = 0.0;
        uint64_t shi = 0, slo = 0;
        for (uint32_t c0 = 0; c0 < B; c0 += 32u) {
            const uint32_t col = c0 + w;
            uint32_t colcarry = 0u;
            float a2 = 0.0f;
            double a2d = 0.0;
            for (uint32_t r0 = 0; r0 < R; r0 += kDistRowBlock) {
                const uint32_t rows = min(kDistRowBlock, R - r0);
                /* phase A: prefix along DE within each row of the strip */
                for (uint32_t rr = w; rr < rows; rr += 32u) {
                    const uint32_t r = r0 + rr;
                    const uint32_t c = c0 + l;
                    uint32_t v = 0u;
                    if (c < B) {
                        uint32_t* h = hist + (uint64_t)r * B + c;
                        v = *h;
                        *h = 0u;
                    }
                    const uint32_t cr = carry[r];
                    const uint32_t s = warp_scan_(v, l) + cr;
                    T[rr * kPad + l] = s;
                    __syncwarp();
                    if (l == 31u) carry[r] = s;
                }
                __syncthreads();
                /* phase B: prefix along K down column c0 + w, distance terms */
                if (col < B) {
                    for (uint32_t rr0 = 0; rr0 < rows; rr0 += 32u) {
                        const uint32_t rr = rr0 + l;
                        const bool valid = rr < rows;
                        const uint32_t v = valid ? T[rr * kPad + w] : 0u;
                        const uint32_t s = warp_scan_(v, l) + colcarry;
                        colcarry = __shfl_sync(0xFFFFFFFFu, s, 31);
                        if (valid) {
                            const uint32_t r = r0 + rr;
                            const uint32_t ref = __ldg(refT + (uint64_t)col * R + r);
                            const float dd = __fsub_rn(__uint2float_rn(s), __uint2float_rn(ref));
                            a2 = __fadd_rn(a2, __fmul_rn(dd, dd));
                            if (F64) {
                                const double d64 = __dsub_rn((double)s, (double)ref);
                                a2d = __dadd_rn(a2d, __dmul_rn(d64, d64));
                            }
                            const uint64_t ad = (s >= ref) ? (uint64_t)(s - ref) : (uint64_t)(ref - s);
                            add128_(shi, slo, 0u, ad * ad);
                            if (cum) cum[(uint64_t)r * B + col] = s;
                        }
                    }
                }
                __syncthreads();
            }
            if (col < B) {
                acc = __fadd_rn(acc, a2);
                if (F64) acc64 = __dadd_rn(acc64, a2d);
            }
        }

        /* reduce0 per warp, then over the 32 warp totals (kernel-distance.inl:210-229) */
        const float wsum = reduce0_(acc);
        double wsum64 = 0.0;
        if (F64) wsum64 = reduce0_(acc64);
        for (uint32_t d = 16; d >= 1; d >>= 1) {
            uint64_t ohi = __shfl_down_sync(0xFFFFFFFFu, shi, d);
            uint64_t olo = __shfl_down_sync(0xFFFFFFFFu, slo, d);
            if (l + d < 32u) add128_(shi, slo, ohi, olo);
        }
        if (l == 0) {
            s_tot[w] = wsum;
            s_tot64[w] = wsum64;
            s_hi[w] = shi;
            s_lo[w] = slo;
        }
        __syncthreads();
        if (w == 0) {
            const float fin = reduce0_(s_tot[l]);
            double fin64 = 0.0;
            if (F64) fin64 = reduce0_(s_tot64[l]);
            uint64_t thi = s_hi[l], tlo = s_lo[l];
            for (uint32_t d = 16; d >= 1; d >>= 1) {
                uint64_t ohi = __shfl_down_sync(0xFFFFFFFFu, thi, d);
                uint64_t olo = __shfl_down_sync(0xFFFFFFFFu, tlo, d);
                if (l + d < 32u) add128_(thi, tlo, ohi, olo);
            }
            if (l == 0) {
                a.dist_f32[p] = fin;
                if (F64 && a.dist_f64) a.dist_f64[p] = fin64;
                if (a.ssd) {
                    a.ssd[2 * (uint64_t)p] = thi;
                    a.ssd[2 * (uint64_t)p + 1] = tlo;
                }
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ uint32_t pick4_(const uint4& v, uint32_t i)
{
    return i == 0u ? v.x : (i == 1u ? v.y : (i == 2u ? v.z : v.w));
}

/* Strip kernel: 16 warps, full-height strips of 32 DE columns, a persistent
 * CTA walking the (proposal, strip) sequence blockIdx.x, blockIdx.x + grid,
 * ... strip by strip.
 *
 * Copy: warp w owns a contiguous segment of ceil(R/16) rows, lane i the
 * rows rb+i, rb+i+32, ... of it.  A row's 32 cells (128 bytes) move with
 * one bulk copy (cp.async.bulk, the TMA unit) completing on the tile's
 * mbarrier, when source, destination and size are 16-byte aligned (B a
 * multiple of 4 and an aligned histogram; every copy is checked before it
 * is issued); cells past B are zero-filled with plain stores.  Other rows
 * take 4-byte cp.async per cell (any B, any offset).  Every thread arrives
 * on the tile's mbarrier once per fill with the bytes of its bulk copies,
 * so a waiter passes only when all copies of the strip have landed; the
 * wait is bounded (error bit 0x80 and a clean exit when it runs out).  With
 * two tiles (db) the copies of the next strip -- or of the next proposal's
 * first strip -- are in flight while the current strip is computed; with
 * one tile (tall histograms) the copies of a strip are issued together.
 * Phase A1: each lane sums column c0+l of its warp's segment (column totals
 * of the segment) and writes zeros back to the histogram, as K_distance
 * does.
 * Phase A2: lane l runs down column c0+l of the segment from the totals of
 * the segments above (column prefix), then lane j runs across row rb+j from
 * the row's carry of the strips to its left (row prefix, 128-bit shared
 * loads and stores): the tile holds the 2-D prefix sums after per-lane
 * chains through shared memory, no shuffles.
 * Phase B: warp w reads two columns of the strip, c0+w for logical warp w
 * and c0+w+16 for logical warp w+16 of the reference's 32x32 launch, so
 * every lane keeps the reference's per-lane sums in two accumulators; the
 * observed cumulative histogram of four 32-row groups is requested at once.
 * SSD: also accumulate the exact integer sum of squares (128-bit per lane);
 * the PMC rounds do not ask for it, the parity entry point does.
 * Tile rows are 36 words (144 bytes): 16-byte aligned for the bulk copies,
 * and with 128-bit shared accesses (row pass, and the 16-byte chunk holding
 * a column in phase B) eight consecutive rows fall in eight different
 * bank groups, so both passes are free of bank conflicts.  R x 36 words per
 * tile: two tiles and two CTAs per SM up to ~385 rows. */
const uint32_t kStripThreads = 512;
const int kStripRefGroups = 4;
const uint32_t kSPitch = 36;                 /* strip tile row pitch (words) */
const uint32_t kMbarWaitLimit = 1u << 22;    /* try_wait rounds before a wait is given up */

__device__ __forceinline__ uint32_t smem_u32_(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init_(uint64_t* m, uint32_t count)
{
    asm volatile("mbarrier.init.shared.b64 [%0], %1;\n" ::"r"(smem_u32_(m)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence_() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx_(uint64_t* m, uint32_t bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(smem_u32_(m)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait_(uint64_t* m, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(done)
                 : "r"(smem_u32_(m)), "r"(parity)
                 : "memory");
    return done != 0u;
}

/* bounded wait for a phase of the mbarrier */
__device__ __forceinline__ bool mbar_wait_(uint64_t* m, uint32_t parity)
{
    for (uint32_t it = 0; it < kMbarWaitLimit; ++it)
        if (mbar_try_wait_(m, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_copy_(void* dst, const void* src, uint32_t bytes, uint64_t* m)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32_(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32_(m))
                 : "memory");
}

/* orders this thread's earlier generic shared-memory accesses before later
 * async-proxy (bulk copy) writes to the same memory */
__device__ __forceinline__ void fence_proxy_async_() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void cp_async4_(uint32_t* dst, const uint32_t* src, bool valid)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = valid ? 4 : 0; /* 0: the destination is zero-filled, src is not read */
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
}

__device__ __forceinline__ void cp_async_commit_() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait_() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ bool aligned16_(const void* p) { return ((uintptr_t)p & 15u) == 0u; }

/* This thread's copies of strip c0 of proposal p into tile T, and its one
 * arrival on the tile's mbarrier (with the bytes of its bulk copies). */
__device__ __forceinline__ void strip_copy_(const DistArgs& a, uint32_t p, uint32_t c0, uint32_t* T, uint32_t w,
                                            uint32_t l, uint64_t* mbar)
{
    const uint32_t job = a.props[p].job;
    const uint32_t R = a.jobs[job].R, B = a.jobs[job].B;
    const bool ok = R <= a.max_rows;
    const uint32_t* hist = a.hist + a.props[p].hist_off;
    const uint32_t seg = (R + 15u) / 16u;
    const uint32_t rb = ok ? min(R, w * seg) : 0u, re = ok ? min(R, rb + seg) : 0u;
    const uint32_t n = B > c0 ? min(32u, B - c0) : 0u; /* cells of this strip in a row */
    const bool bulk_shape = n > 0u && (n & 3u) == 0u;
    uint32_t bytes = 0u;
    if (bulk_shape)
        for (uint32_t r = rb + l; r < re; r += 32u)
            if (aligned16_(hist + (uint64_t)r * B + c0) && aligned16_(T + r * kSPitch)) bytes += 4u * n;
    mbar_arrive_expect_tx_(mbar, bytes);
    for (uint32_t r = rb + l; r < re; r += 32u) {
        const uint32_t* src = hist + (uint64_t)r * B + c0;
        uint32_t* dst = T + r * kSPitch;
        if (bulk_shape && aligned16_(src) && aligned16_(dst)) {
            bulk_copy_(dst, src, 4u * n, mbar);
            for (uint32_t c = n; c < 32u; ++c) dst[c] = 0u;
        } else {
            for (uint32_t c = 0; c < 32u; ++c) cp_async4_(dst + c, c < n ? src + c : hist, c < n);
        }
    }
}

template <bool F64, bool SSD>
__global__ void __launch_bounds__(512, 2) k_distance_strip(DistArgs a, uint32_t db)
{
    extern __shared__ __align__(16) uint32_t s_mem[];
    const uint32_t tile_words = a.max_rows * kSPitch;
    /* 16-byte aligned tiles (the launch reserves 16 bytes for this) */
    uint32_t* tiles = s_mem + ((16u - (smem_u32_(s_mem) & 15u)) & 15u) / 4u; /* [1 + db][max_rows][kSPitch] */
    uint32_t* carry = s_mem + (1u + db) * tile_words;     /* [max_rows] */
    __shared__ float s_tot[32];
    __shared__ double s_tot64[32];
    __shared__ uint64_t s_hi[32], s_lo[32];
    __shared__ uint32_t s_col[16][32]; /* column totals of each warp's row segment */
    __shared__ __align__(8) uint64_t s_mbar[2];
    __shared__ uint32_t s_abort;

    const uint32_t tid = threadIdx.x;
    const uint32_t w = tid >> 5, l = tid & 31u;
    const uint32_t M = *a.n_props;
    uint32_t p = blockIdx.x;
    if (p >= M) return;
    if (tid == 0) {
        mbar_init_(&s_mbar[0], kStripThreads);
        mbar_init_(&s_mbar[1], kStripThreads);
        mbar_init_fence_();
        s_abort = 0u;
    }
    __syncthreads();

    uint32_t c0 = 0, cur = 0, parity = 0u; /* parity bit b: the phase of tile b's next fill */
    uint32_t pending = 1u;                  /* bit b: tile b has a fill in flight */
    strip_copy_(a, p, 0u, tiles, w, l, &s_mbar[0]);
    cp_async_commit_();

    float acc0 = 0.0f, acc1 = 0.0f;
    double accd0 = 0.0, accd1 = 0.0;
    uint64_t shi = 0, slo = 0;
    for (;;) {
        const uint32_t job = a.props[p].job;
        const uint64_t hoff = a.props[p].hist_off;
        const uint32_t R = a.jobs[job].R, B = a.jobs[job].B;
        const bool ok = R <= a.max_rows;
        /* the (proposal, strip) after this one */
        uint32_t pn = p, cn = c0 + 32u;
        if (!ok || cn >= B) {
            pn = p + gridDim.x;
            cn = 0u;
        }
        const bool has_next = pn < M;
        if (db) {
            if (has_next) {
                strip_copy_(a, pn, cn, tiles + (cur ^ 1u) * tile_words, w, l, &s_mbar[cur ^ 1u]);
                pending |= 1u << (cur ^ 1u);
            }
            cp_async_commit_();
            cp_async_wait_<1>(); /* this thread's 4-byte copies of the current strip have landed */
        } else {
            cp_async_wait_<0>();
        }
        /* the current strip's bulk copies (all threads' arrivals and bytes) */
        if (!mbar_wait_(&s_mbar[cur], (parity >> cur) & 1u)) {
            atomicOr(a.err, PCS_ERRBIT_TIMEOUT);
            s_abort = 1u;
        }
        parity ^= 1u << cur;
        pending &= ~(1u << cur);
        __syncwarp(); /* rows copied by other lanes of this warp (4-byte copies, zero fills) */
        uint32_t* T = tiles + cur * tile_words;
        if (!ok) {
            if (tid == 0) {
                atomicOr(a.err, PCS_ERRBIT_ROWS);
                a.dist_f32[p] = __int_as_float(0x7fc00000);
            }
        } else {
            const uint32_t* __restrict__ refT = a.jobs[job].ref_sat_t;
            uint32_t* hist = a.hist + hoff;
            uint32_t* cum = a.cum_out ? a.cum_out + hoff : nullptr;
            const uint32_t seg = (R + 15u) / 16u;
            const uint32_t rb = min(R, w * seg), re = min(R, rb + seg);
            const uint32_t c = c0 + l;
            const bool cin = c < B;
            /* phase A1: this lane's cells -> column total, zeros written back */
            uint32_t coltot = 0u;
#pragma unroll 4
            for (uint32_t r = rb; r < re; ++r) {
                coltot += T[r * kSPitch + l];
                if (cin) __stcs(hist + (uint64_t)r * B + c, 0u);
            }
            s_col[w][l] = coltot;
            __syncthreads();
            if (s_abort) break; /* a copy wait ran out (error word set) */
            /* phase A2: column prefix down the segment, then row prefix across
             * the strip: the tile holds the 2-D prefix sums */
            uint32_t run = 0u;
            for (uint32_t q = 0; q < w; ++q) run += s_col[q][l];
#pragma unroll 4
            for (uint32_t r = rb; r < re; ++r) {
                run += T[r * kSPitch + l];
                T[r * kSPitch + l] = run;
            }
            __syncwarp();
            for (uint32_t r = rb + l; r < re; r += 32u) {
                uint4* row4 = reinterpret_cast<uint4*>(T + r * kSPitch);
                uint32_t acc = c0 ? carry[r] : 0u;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    uint4 v = row4[j];
                    v.x += acc;
                    v.y += v.x;
                    v.z += v.y;
                    v.w += v.z;
                    acc = v.w;
                    row4[j] = v;
                }
                carry[r] = acc;
            }
            __syncthreads();
            /* phase B: columns c0 + w and c0 + w + 16 */
            const uint32_t colA = c0 + w, colB = c0 + w + 16u;
            const bool inA = colA < B, inB = colB < B;
            if (inA) {
                float a2A = 0.0f, a2B = 0.0f;
                double a2dA = 0.0, a2dB = 0.0;
                for (uint32_t rg = 0; rg < R; rg += 32u * kStripRefGroups) {
                    uint32_t refAv[kStripRefGroups], refBv[kStripRefGroups];
#pragma unroll
                    for (int g = 0; g < kStripRefGroups; ++g) {
                        const uint32_t r = rg + 32u * (uint32_t)g + l;
                        refAv[g] = r < R ? __ldg(refT + (uint64_t)colA * R + r) : 0u;
                        refBv[g] = (r < R && inB) ? __ldg(refT + (uint64_t)colB * R + r) : 0u;
                    }
#pragma unroll
                    for (int g = 0; g < kStripRefGroups; ++g) {
                        const uint32_t r = rg + 32u * (uint32_t)g + l;
                        if (r < R) {
                            const uint4 chA = reinterpret_cast<const uint4*>(T + r * kSPitch)[w >> 2];
                            const uint32_t sA = pick4_(chA, w & 3u);
                            const uint32_t refA = refAv[g];
                            const float ddA = __fsub_rn(__uint2float_rn(sA), __uint2float_rn(refA));
                            a2A = __fadd_rn(a2A, __fmul_rn(ddA, ddA));
                            if (SSD) {
                                const uint64_t adA = (sA >= refA) ? (uint64_t)(sA - refA) : (uint64_t)(refA - sA);
                                add128_(shi, slo, 0u, adA * adA);
                            }
                            if (F64) {
                                const double d64 = __dsub_rn((double)sA, (double)refA);
                                a2dA = __dadd_rn(a2dA, __dmul_rn(d64, d64));
                            }
                            if (cum) cum[(uint64_t)r * B + colA] = sA;
                            if (inB) {
                                const uint4 chB = reinterpret_cast<const uint4*>(T + r * kSPitch)[(w >> 2) + 4u];
                                const uint32_t sB = pick4_(chB, w & 3u);
                                const uint32_t refB = refBv[g];
                                const float ddB = __fsub_rn(__uint2float_rn(sB), __uint2float_rn(refB));
                                a2B = __fadd_rn(a2B, __fmul_rn(ddB, ddB));
                                if (SSD) {
                                    const uint64_t adB = (sB >= refB) ? (uint64_t)(sB - refB) : (uint64_t)(refB - sB);
                                    add128_(shi, slo, 0u, adB * adB);
                                }
                                if (F64) {
                                    const double d64 = __dsub_rn((double)sB, (double)refB);
                                    a2dB = __dadd_rn(a2dB, __dmul_rn(d64, d64));
                                }
                                if (cum) cum[(uint64_t)r * B + colB] = sB;
                            }
                        }
                    }
                }
                acc0 = __fadd_rn(acc0, a2A);
                if (F64) accd0 = __dadd_rn(accd0, a2dA);
                if (inB) {
                    acc1 = __fadd_rn(acc1, a2B);
                    if (F64) accd1 = __dadd_rn(accd1, a2dB);
                }
            }
        }
        fence_proxy_async_(); /* this tile's generic accesses before its next bulk fill */
        __syncthreads();      /* the tile is free for the copies issued next */

        if (ok && c0 + 32u >= B) {
            /* last strip: reduce0 per logical warp (w and w + 16), then over
             * the 32 totals */
            const float ws0 = reduce0_(acc0), ws1 = reduce0_(acc1);
            double wd0 = 0.0, wd1 = 0.0;
            if (F64) {
                wd0 = reduce0_(accd0);
                wd1 = reduce0_(accd1);
            }
            if (SSD) {
                for (uint32_t d = 16; d >= 1; d >>= 1) {
                    uint64_t ohi = __shfl_down_sync(0xFFFFFFFFu, shi, d);
                    uint64_t olo = __shfl_down_sync(0xFFFFFFFFu, slo, d);
                    if (l + d < 32u) add128_(shi, slo, ohi, olo);
                }
            }
            if (l == 0) {
                s_tot[w] = ws0;
                s_tot[w + 16] = ws1;
                s_tot64[w] = wd0;
                s_tot64[w + 16] = wd1;
                s_hi[w] = shi;
                s_lo[w] = slo;
                s_hi[w + 16] = 0u;
                s_lo[w + 16] = 0u;
            }
            __syncthreads();
            if (w == 0) {
                const float fin = reduce0_(s_tot[l]);
                double fin64 = 0.0;
                if (F64) fin64 = reduce0_(s_tot64[l]);
                uint64_t thi = s_hi[l], tlo = s_lo[l];
                if (SSD) {
                    for (uint32_t d = 16; d >= 1; d >>= 1) {
                        uint64_t ohi = __shfl_down_sync(0xFFFFFFFFu, thi, d);
                        uint64_t olo = __shfl_down_sync(0xFFFFFFFFu, tlo, d);
                        if (l + d < 32u) add128_(thi, tlo, ohi, olo);
                    }
                }
                if (l == 0) {
                    a.dist_f32[p] = fin;
                    if (F64 && a.dist_f64) a.dist_f64[p] = fin64;
                    if (SSD && a.ssd) {
                        a.ssd[2 * (uint64_t)p] = thi;
                        a.ssd[2 * (uint64_t)p + 1] = tlo;
                    }
                }
            }
            __syncthreads();
            acc0 = acc1 = 0.0f;
            accd0 = accd1 = 0.0;
            shi = slo = 0u;
        }
        if (!has_next) break;
        if (!db) {
            strip_copy_(a, pn, cn, tiles, w, l, &s_mbar[0]);
            pending |= 1u;
            cp_async_commit_();
        } else {
            cur ^= 1u;
        }
        p = pn;
        c0 = cn;
    }
    cp_async_wait_<0>();
    /* after a given-up wait: let the fills still in flight land (bounded) */
    for (uint32_t b = 0; b < 2u; ++b)
        if ((pending >> b) & 1u) mbar_wait_(&s_mbar[b], (parity >> b) & 1u);
}

static const size_t kStripSmemMax = 220u * 1024u;

/* one or two tiles + carry + 16 bytes to align the tiles */
static size_t strip_smem_bytes(uint32_t max_rows, bool db)
{
    return ((size_t)max_rows * (1u + (db ? 2u : 1u) * kSPitch)) * sizeof(uint32_t) + 16u;
}

static bool use_strip(uint32_t max_rows) { return strip_smem_bytes(max_rows, false) <= kStripSmemMax; }
static bool strip_db(uint32_t max_rows) { return strip_smem_bytes(max_rows, true) <= kStripSmemMax; }

size_t distance_smem_bytes(uint32_t max_rows)
{
    if (use_strip(max_rows)) return strip_smem_bytes(max_rows, strip_db(max_rows));
    return ((size_t)max_rows + (size_t)kDistRowBlock * kPad) * sizeof(uint32_t);
}

uint32_t distance_block_threads(uint32_t max_rows) { return use_strip(max_rows) ? kStripThreads : 1024u; }

int distance_ctas_per_sm(uint32_t max_rows)
{
    const size_t smem = distance_smem_bytes(max_rows);
    int n = 0;
    if (use_strip(max_rows)) {
        cudaFuncSetAttribute(k_distance_strip<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_distance_strip<false, false>, (int)kStripThreads, smem);
    } else {
        cudaFuncSetAttribute(k_distance<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_distance<false>, 1024, smem);
    }
    return n > 0 ? n : 1;
}

cudaError_t launch_distance(const DistArgs& a, uint32_t grid, cudaStream_t st)
{
    const size_t smem = distance_smem_bytes(a.max_rows);
    if (use_strip(a.max_rows)) {
        void (*k)(DistArgs, uint32_t);
        if (a.dist_f64) k = a.ssd ? k_distance_strip<true, true> : k_distance_strip<true, false>;
        else k = a.ssd ? k_distance_strip<false, true> : k_distance_strip<false, false>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, kStripThreads, smem, st>>>(a, strip_db(a.max_rows) ? 1u : 0u);
        return cudaGetLastError();
    }
    if (a.dist_f64) {
        cudaError_t e = cudaFuncSetAttribute(k_distance<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_distance<true><<<grid, 1024, smem, st>>>(a);
    } else {
        cudaError_t e = cudaFuncSetAttribute(k_distance<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_distance<false><<<grid, 1024, smem, st>>>(a);
    }
    return cudaGetLastError();
}

} // namespace pcs
