/*
 * kernels_dist.cu -- fused 2-D prefix sum + cumulative distance.
 *
 * Follows cusim::K_distance (src/gpu/cusim/kernel-distance.inl:81-241), which
 * runs one 32x32 block per proposal over the whole R x B histogram twice
 * (row scans, then column scans accumulating (cum - ref)^2) and zeroes the
 * histogram for reuse.  Here one CTA per proposal streams the histogram in
 * strips of 32 DE columns through a shared-memory tile:
 *   k_distance_strip (up to 1664 rows, 512 threads): the whole strip height
 *            sits in a swizzled tile filled by TMA box copies; phase A
 *            builds its 2-D prefix sums (zeros written back by box stores,
 *            per-lane column and row passes, per-row carry across strips
 *            in shared memory), phase B reads columns c0+2w, c0+2w+1 for
 *            logical warps 2w, 2w+1 while lane l accumulates
 *            (float(cum) - float(ref))^2 for rows l, l+32, ..., the observed
 *            cumulative histogram read from its column-major copy (coalesced);
 *   k_distance_cluster (histograms of up to 256 bins, where they are tall
 *            or each has a cluster): a thread-block cluster per histogram,
 *            one strip per CTA, the row carries and per-lane sums
 *            exchanged through distributed shared memory;
 *   k_distance (taller histograms, 1024 threads): the same in blocks of
 *            256 rows (tile row pitch 33 words), with the column carry in a
 *            register.
 * Warp w / lane l therefore own exactly the columns and rows they own in the
 * reference launch, so the per-lane sums, the shfl_down trees of reduce0
 * (:69-78) and the final per-warp tree reproduce the reference's float
 * result bit for bit (each operation is an explicit round-to-nearest
 * intrinsic, as in a build without FMA contraction).  The exact integer sum
 * of squares and a double-precision sum are accumulated alongside on request.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

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
                            const uint32_t ref = __ldg(refT + pcs_sat_t_index(r, col, R, B));
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

/* Strip kernel: 16 warps, full-height strips of 32 DE columns, a persistent
 * CTA walking the (proposal, strip) sequence blockIdx.x, blockIdx.x + grid,
 * ... strip by strip.
 *
 * Tile: rows of 32 cells (128 bytes) whose 16-byte chunks are permuted by
 * XOR with (row mod 8) -- the TMA 128-byte swizzle -- so row-wise 128-bit
 * accesses by lanes on consecutive rows, and column-wise accesses, are free
 * of bank conflicts; 1024-byte aligned; rows up to the next multiple of 32.
 * Copy: with a tensor map for the job (B x R x histograms, boxes of 32 x 32
 * cells), one thread issues ceil(R/32) box copies (cp.async.bulk.tensor, the
 * TMA unit) completing on the tile's mbarrier; rows past R and columns past
 * B are outside the tensor and arrive as zeros.  Without one (B not a
 * multiple of 4, R or B below 32, callers without maps), every lane copies
 * its cells with 4-byte cp.async into the swizzled positions, zero-filling
 * past R and B.  Every thread arrives on the tile's mbarrier once per fill,
 * so a waiter passes only when all copies of the strip have landed; the
 * wait is bounded (error bit 0x80 and a clean exit when it runs out).  With
 * two tiles (db) the copies of the next strip -- or of the next proposal's
 * first strip -- are issued after the current strip's first barrier (every
 * warp is then past the strip before, whose tile they fill) and are in
 * flight while the current strip is computed: two CTA barriers per strip.
 * With one tile (tall histograms) the copies of a strip are issued together
 * after a third barrier.
 * Rows are split into 16 warp segments of a multiple of 8 rows (the
 * segments reach the next multiple of 8 past R; those rows hold zeros), so
 * a lane's swizzled column offset within each group of 8 rows is fixed.
 * Phase A1: lane l runs down column c0+l of its warp's segment (column
 * prefix within the segment, in place) and keeps the segment's column total;
 * the strip is zeroed in the histogram, as K_distance does, by box stores
 * of a zero box (one thread), or by the lanes cell by cell without a map.
 * Phase A2: lane l adds the totals of the segments above (the column carry
 * into the segment) and a warp scan turns the 32 carries into their prefix
 * across the strip; lane j then runs across row rb+j from the row's carry
 * of the strips to its left (128-bit shared loads and stores), adding the
 * scanned column carry: the tile holds the 2-D prefix sums.
 * Phase B: warp w reads columns c0+2w and c0+2w+1 -- logical warps 2w and
 * 2w+1 of the reference's 32x32 launch -- with one 8-byte shared load per
 * row, and the observed cumulative histogram of the same two columns with
 * one coalesced 8-byte load per row (pair-interleaved copy), so every lane
 * keeps the reference's per-lane sums in two accumulators.  When every
 * cumulative count of the strip and of the observed histogram is below
 * 2^22 (the largest is the last row's last cell: prefix sums of counts
 * are monotone), float(s) - float(o) is the exact integer s - o, and it is
 * formed as the float whose bits are 0x4B400000 + s - o (1.5 * 2^23 + s - o,
 * exact in [2^23, 2^24)) minus 1.5 * 2^23: the same value the reference's
 * two conversions and subtraction give, in two instructions.
 * SSD: also accumulate the exact integer sum of squares (128-bit per lane);
 * the PMC rounds do not ask for it, the parity entry point does. */
const uint32_t kStripThreads = 512;
const uint32_t kBox = 32;                     /* rows and columns of a tensor-map box */
const uint32_t kBoxBytes = kBox * kBox * 4u;  /* 4096 */
const uint32_t kMbarWaitLimit = 1u << 22;     /* try_wait rounds before a wait is given up */
const uint32_t kExactBelow = 1u << 22;        /* cumulative counts below this take the integer difference */

__host__ __device__ __forceinline__ uint32_t strip_cap_rows(uint32_t max_rows) { return (max_rows + 31u) & ~31u; }

__device__ __forceinline__ uint32_t round8_(uint32_t x) { return (x + 7u) & ~7u; }

/* word of (row r, column c) in a swizzled strip tile */
__device__ __forceinline__ uint32_t sw_(uint32_t r, uint32_t c)
{
    return (r << 5) | ((((c >> 2) ^ (r & 7u)) << 2) | (c & 3u));
}

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

/* the tensor map as written through global memory, for this thread's box copies */
__device__ __forceinline__ void tmap_acquire_(const TmapDev* map)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(map) : "memory");
}

/* box (x, y, z) of a 3-D tensor map -> shared memory, completing on an mbarrier */
__device__ __forceinline__ void tma_load_3d_(uint32_t* dst, const TmapDev* map, uint32_t x, uint32_t y, uint32_t z,
                                             uint64_t* m)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
            smem_u32_(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32_(m))
        : "memory");
}

/* shared memory -> box (x, y, z) of a 3-D tensor map (cells outside the tensor are dropped) */
__device__ __forceinline__ void tma_store_3d_(const TmapDev* map, uint32_t x, uint32_t y, uint32_t z, const uint32_t* src)
{
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(map),
                 "r"(x), "r"(y), "r"(z), "r"(smem_u32_(src))
                 : "memory");
}

__device__ __forceinline__ void bulk_commit_() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }

/* this thread's box stores have completed */
__device__ __forceinline__ void bulk_wait_all_() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

/* orders this thread's earlier generic shared-memory accesses before later
 * async-proxy (tensor copy) accesses to the same memory */
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

/* thread-block cluster: this CTA's rank, the cluster's index and count */
__device__ __forceinline__ uint32_t cluster_rank_()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cluster_id_()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;\n" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cluster_count_()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;\n" : "=r"(r));
    return r;
}

/* every thread of every CTA of the cluster; shared-memory writes before it
 * are visible to shared::cluster reads after it */
__device__ __forceinline__ void cluster_sync_()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

/* the word at `p` (this CTA's shared memory) in the shared memory of the
 * cluster's CTA `rank` */
__device__ __forceinline__ uint32_t ld_cluster_(const void* p, uint32_t rank)
{
    uint32_t ra, v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(ra) : "r"(smem_u32_(p)), "r"(rank));
    asm volatile("ld.shared::cluster.u32 %0, [%1];\n" : "=r"(v) : "r"(ra) : "memory");
    return v;
}

/* warp w's segment of rows: [rb, re), multiples of 8, up to round8(R) */
struct Seg {
    uint32_t rb, re;
};

__device__ __forceinline__ Seg seg_(uint32_t R, uint32_t w)
{
    const uint32_t R8 = round8_(R);
    const uint32_t n = round8_((R8 + 15u) / 16u);
    Seg s;
    s.rb = min(R8, w * n);
    s.re = min(R8, s.rb + n);
    return s;
}

/* proposal p's tensor map and its index along the map, or null (cell-by-cell copies) */
__device__ __forceinline__ const TmapDev* prop_tmap_(const DistArgs& a, uint32_t p, uint32_t job, uint32_t& z)
{
    z = 0u;
    if (!a.tmaps) return nullptr;
    const uint32_t depth = a.jobs[job].tmap_depth;
    z = a.props[p].hist_z;
    return (depth != 0u && z < depth) ? a.tmaps + job : nullptr;
}

/* This thread's part of filling tile T with strip c0 of proposal p, and its
 * one arrival on the tile's mbarrier. */
__device__ __forceinline__ void strip_fill_(const DistArgs& a, uint32_t p, uint32_t c0, uint32_t* T, uint32_t tid,
                                            uint64_t* mbar)
{
    const uint32_t job = a.props[p].job;
    const uint32_t R = a.jobs[job].R, B = a.jobs[job].B;
    if (R > a.max_rows) {
        mbar_arrive_expect_tx_(mbar, 0u);
        return;
    }
    uint32_t z;
    const TmapDev* map = prop_tmap_(a, p, job, z);
    if (map) {
        if (tid == 0u) {
            const uint32_t nbox = (R + kBox - 1u) / kBox;
            tmap_acquire_(map);
            mbar_arrive_expect_tx_(mbar, nbox * kBoxBytes);
            for (uint32_t b = 0; b < nbox; ++b) tma_load_3d_(T + b * kBox * 32u, map, c0, b * kBox, z, mbar);
        } else {
            mbar_arrive_expect_tx_(mbar, 0u);
        }
        return;
    }
    mbar_arrive_expect_tx_(mbar, 0u);
    const uint32_t w = tid >> 5, l = tid & 31u;
    const Seg sg = seg_(R, w);
    const uint32_t* hist = a.hist + a.props[p].hist_off;
    const uint32_t c = c0 + l, lc = l >> 2, lo = l & 3u;
    for (uint32_t r8 = sg.rb; r8 < sg.re; r8 += 8u)
#pragma unroll
        for (uint32_t k = 0; k < 8u; ++k) {
            const uint32_t r = r8 + k;
            const bool v = r < R && c < B;
            cp_async4_(T + (r << 5) + (((lc ^ k) << 2) | lo), v ? hist + (uint64_t)r * B + c : hist, v);
        }
}

/* one distance term, general form: the reference's conversions, and on
 * request the FP64 and exact integer sums and the prefix-sum output */
template <bool F64, bool SSD>
__device__ __forceinline__ void term_(uint32_t s, uint32_t o, float& a2, double& a2d, uint64_t& shi,
                                      uint64_t& slo, uint32_t* cum, uint64_t at)
{
    const float dd = __fsub_rn(__uint2float_rn(s), __uint2float_rn(o));
    a2 = __fadd_rn(a2, __fmul_rn(dd, dd));
    if (SSD) {
        const uint64_t ad = (s >= o) ? (uint64_t)(s - o) : (uint64_t)(o - s);
        add128_(shi, slo, 0u, ad * ad);
    }
    if (F64) {
        const double d64 = __dsub_rn((double)s, (double)o);
        a2d = __dadd_rn(a2d, __dmul_rn(d64, d64));
    }
    if (cum) cum[at] = s;
}

/* float(s) - float(o) for s, o < 2^22 (exact integer difference) */
__device__ __forceinline__ float exact_diff_(uint32_t s, uint32_t o)
{
    return __fsub_rn(__uint_as_float(0x4B400000u + s - o), 12582912.0f);
}

/* Cluster mode (k_distance_cluster), for launches where walking each
 * histogram's strips one after another in one CTA leaves SMs idle or takes
 * long: few histograms, or tall ones.  A cluster of `cl` CTAs takes one
 * histogram at a time, CTA k its strip k (columns
 * 32k..32k+31; cl is at least the strips of every job).  Each CTA builds
 * its strip's 2-D prefix sums as if the strip stood alone (row carry 0) and
 * publishes the last column, P_k(r) = the cells of rows <= r in the strip;
 * after a cluster barrier CTA k's row carry is sum_{j<k} P_j(r), read from
 * the other CTAs' shared memory (integers, so the prefix sums are the strip
 * walk's exactly).  Each CTA then forms its strip's per-lane sums for
 * logical warps 2w, 2w+1 as the strip walk does and publishes them; after
 * the next barrier CTA 0 adds each (logical warp, lane)'s strip sums in
 * strip order -- the strip walk's per-lane accumulation, operation for
 * operation -- and reduces them with the same trees: the same float, bit
 * for bit.  One barrier per histogram: P and the per-lane sums alternate
 * between two buffers, and CTA 0 reduces histogram i while the cluster
 * computes histogram i + 1.  The next histogram's strip is copied in while
 * the current one is computed (two tiles), or, with one tile (tall
 * histograms), as soon as phase B has read it.  A copy wait that runs out ends
 * the loop on every CTA of the cluster together (each reads all CTAs' flags
 * after the barrier), so no CTA is left waiting at a cluster barrier. */
__device__ __forceinline__ void cluster_fill_(const DistArgs& a, uint32_t p, uint32_t k, uint32_t cl, uint32_t* T,
                                              uint32_t tid, uint64_t* mbar)
{
    const uint32_t ns = (a.jobs[a.props[p].job].B + 31u) / 32u;
    if (k < ns && ns <= cl) strip_fill_(a, p, 32u * k, T, tid, mbar);
    else mbar_arrive_expect_tx_(mbar, 0u);
}

/* CTA 0: histogram p's distance from every strip's per-lane sums */
__device__ __forceinline__ void cluster_reduce_(const DistArgs& a, uint32_t p, uint32_t cl, const float* part,
                                                float* s_tot)
{
    const uint32_t tid = threadIdx.x, w = tid >> 5, l = tid & 31u;
    const uint32_t job = a.props[p].job;
    const uint32_t B = a.jobs[job].B;
    if (!(a.jobs[job].R <= a.max_rows && (B + 31u) / 32u <= cl)) {
        if (tid == 0u) {
            atomicOr(a.err, PCS_ERRBIT_ROWS);
            a.dist_f32[p] = __int_as_float(0x7fc00000);
        }
        return;
    }
    const uint32_t ns = (B + 31u) / 32u;
#pragma unroll
    for (uint32_t h = 0; h < 2u; ++h) {
        const uint32_t lw = 2u * w + h;
        float acc = 0.0f;
        for (uint32_t j = 0; j < ns; ++j)
            if (32u * j + lw < B) acc = __fadd_rn(acc, __uint_as_float(ld_cluster_(part + lw * 32u + l, j)));
        const float ws = reduce0_(acc);
        if (l == 0u) s_tot[lw] = ws;
    }
    __syncthreads();
    if (w == 0u) {
        const float fin = reduce0_(s_tot[l]);
        if (l == 0u) a.dist_f32[p] = fin;
    }
}

__device__ __forceinline__ void strip_cluster_(const DistArgs& a, uint32_t db, uint32_t cl, uint32_t M,
                                               uint32_t* tiles, uint32_t tile_words, const uint32_t* zero,
                                               uint32_t* carry, uint32_t* P2, float* part2, float* s_tot,
                                               uint32_t (*s_col)[32], uint32_t (*s_K)[32], uint64_t* s_mbar,
                                               uint32_t* s_abort)
{
    const uint32_t tid = threadIdx.x;
    const uint32_t w = tid >> 5, l = tid & 31u;
    const uint32_t k = cluster_rank_(), ncl = cluster_count_();
    const uint32_t prow = strip_cap_rows(a.max_rows);
    uint32_t p = cluster_id_();
    cluster_sync_(); /* every CTA of the cluster runs before shared::cluster reads */
    uint32_t cur = 0, parity = 0u, pending = 1u, it = 0u, ab = 0u;
    uint32_t p_prev = 0u;
    cluster_fill_(a, p, k, cl, tiles, tid, &s_mbar[0]);
    cp_async_commit_();
    for (;;) {
        const uint32_t job = a.props[p].job;
        const uint32_t R = a.jobs[job].R, B = a.jobs[job].B;
        const uint32_t ns = (B + 31u) / 32u;
        const bool ok = R <= a.max_rows && ns <= cl;
        const bool act = ok && k < ns;
        const uint32_t c0 = 32u * k;
        const uint32_t pn = p + ncl;
        const bool has_next = pn < M;
        uint32_t* P = P2 + (it & 1u) * prow;
        float* part = part2 + (it & 1u) * 1024u;
        cp_async_wait_<0>();
        if (!mbar_wait_(&s_mbar[cur], (parity >> cur) & 1u)) {
            atomicOr(a.err, PCS_ERRBIT_TIMEOUT);
            *s_abort = 1u;
        }
        parity ^= 1u << cur;
        pending &= ~(1u << cur);
        __syncwarp();
        uint32_t* T = tiles + cur * tile_words;
        const Seg sg = seg_(R, w);
        const uint32_t lc = l >> 2, lo = l & 3u;
        if (act) {
            /* phase A1 as in the strip walk, and the strip zeroed */
            uint32_t run = 0u;
            for (uint32_t r8 = sg.rb; r8 < sg.re; r8 += 8u) {
                uint32_t* t = T + (r8 << 5);
#pragma unroll
                for (uint32_t j = 0; j < 8u; ++j) {
                    uint32_t* q = t + (j << 5) + (((lc ^ j) << 2) | lo);
                    run += *q;
                    *q = run;
                }
            }
            s_col[w][l] = run;
            uint32_t z;
            const TmapDev* map = prop_tmap_(a, p, job, z);
            if (map) {
                if (tid == 0u) {
                    const uint32_t nbox = (R + kBox - 1u) / kBox;
                    for (uint32_t b = 0; b < nbox; ++b) tma_store_3d_(map, c0, b * kBox, z, zero);
                    bulk_commit_();
                }
            } else if (c0 + l < B) {
                uint32_t* hist = a.hist + a.props[p].hist_off;
                for (uint32_t r = sg.rb; r < min(sg.re, R); ++r) __stcs(hist + (uint64_t)r * B + c0 + l, 0u);
            }
        }
        __syncthreads();
        if (db && has_next && !*s_abort) {
            cluster_fill_(a, pn, k, cl, tiles + (cur ^ 1u) * tile_words, tid, &s_mbar[cur ^ 1u]);
            pending |= 1u << (cur ^ 1u);
            cp_async_commit_();
        }
        if (act) {
            /* phase A2 with row carry 0: the strip's own 2-D prefix sums */
            uint32_t cc = 0u;
            for (uint32_t q = 0; q < w; ++q) cc += s_col[q][l];
            s_K[w][l] = warp_scan_(cc, l);
            __syncwarp();
            const uint4* K4 = reinterpret_cast<const uint4*>(s_K[w]);
            for (uint32_t r = sg.rb + l; r < sg.re; r += 32u) {
                uint4* row4 = reinterpret_cast<uint4*>(T + (r << 5));
                const uint32_t m = r & 7u;
                uint32_t acc = 0u;
                uint4 o = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (uint32_t j = 0; j < 8u; ++j) {
                    const uint4 v = row4[j ^ m];
                    const uint4 kk = K4[j];
                    acc += v.x;
                    o.x = acc + kk.x;
                    acc += v.y;
                    o.y = acc + kk.y;
                    acc += v.z;
                    o.z = acc + kk.z;
                    acc += v.w;
                    o.w = acc + kk.w;
                    row4[j ^ m] = o;
                }
                P[r] = o.w;
            }
        }
        /* this histogram's last columns, and the previous one's per-lane sums, published */
        cluster_sync_();
        for (uint32_t j = 0; j < cl; ++j) ab |= ld_cluster_(s_abort, j);
        if (ab) break; /* a copy wait ran out somewhere in the cluster (error word set) */
        if (act) {
            /* row carry from the strips to the left */
            for (uint32_t r = tid; r < R; r += kStripThreads) {
                uint32_t c = 0u;
                for (uint32_t j = 0; j < k; ++j) c += ld_cluster_(P + r, j);
                carry[r] = c;
            }
            __syncthreads();
            /* phase B as in the strip walk, the row carry added to each cell */
            const uint32_t colA = c0 + 2u * w;
            float a2A = 0.0f, a2B = 0.0f;
            if (colA < B) {
                const bool inB = colA + 1u < B;
                const uint32_t* Tl = T + ((((w >> 1) ^ (l & 7u)) << 2) | ((2u * w) & 3u));
                const uint32_t* __restrict__ refT = a.jobs[job].ref_sat_t;
                const uint32_t* refc = refT + (uint64_t)colA * R;
                const bool exact = T[sw_(R - 1u, 31u)] + carry[R - 1u] < kExactBelow &&
                                   __ldg(refT + pcs_sat_t_index(R - 1u, B - 1u, R, B)) < kExactBelow;
                if (exact && inB) {
                    const uint2* ref2 = reinterpret_cast<const uint2*>(refc);
#pragma unroll 4
                    for (uint32_t r = l; r < R; r += 32u) {
                        const uint2 v = *reinterpret_cast<const uint2*>(Tl + (r << 5));
                        const uint32_t c = carry[r];
                        const uint2 o = __ldg(ref2 + r);
                        const float dA = exact_diff_(v.x + c, o.x);
                        const float dB = exact_diff_(v.y + c, o.y);
                        a2A = __fadd_rn(a2A, __fmul_rn(dA, dA));
                        a2B = __fadd_rn(a2B, __fmul_rn(dB, dB));
                    }
                } else if (exact) {
                    for (uint32_t r = l; r < R; r += 32u) {
                        const float dA = exact_diff_(Tl[r << 5] + carry[r], __ldg(refc + r));
                        a2A = __fadd_rn(a2A, __fmul_rn(dA, dA));
                    }
                } else {
                    for (uint32_t r = l; r < R; r += 32u) {
                        const uint32_t c = carry[r];
                        if (inB) {
                            const uint2 v = *reinterpret_cast<const uint2*>(Tl + (r << 5));
                            const uint2 o = __ldg(reinterpret_cast<const uint2*>(refc) + r);
                            const float dA = __fsub_rn(__uint2float_rn(v.x + c), __uint2float_rn(o.x));
                            const float dB = __fsub_rn(__uint2float_rn(v.y + c), __uint2float_rn(o.y));
                            a2A = __fadd_rn(a2A, __fmul_rn(dA, dA));
                            a2B = __fadd_rn(a2B, __fmul_rn(dB, dB));
                        } else {
                            const float dA = __fsub_rn(__uint2float_rn(Tl[r << 5] + c), __uint2float_rn(__ldg(refc + r)));
                            a2A = __fadd_rn(a2A, __fmul_rn(dA, dA));
                        }
                    }
                }
            }
            part[(2u * w) * 32u + l] = a2A;
            part[(2u * w + 1u) * 32u + l] = a2B;
        }
        /* this tile's generic accesses before its next box fill */
        fence_proxy_async_();
        if (!db && has_next) {
            __syncthreads(); /* the one tile is free: refill it before CTA 0's reduction */
            cluster_fill_(a, pn, k, cl, tiles, tid, &s_mbar[0]);
            pending |= 1u;
            cp_async_commit_();
        }
        /* CTA 0: the previous histogram, whose sums every CTA published before the barrier */
        if (k == 0u && it > 0u) cluster_reduce_(a, p_prev, cl, part2 + ((it - 1u) & 1u) * 1024u, s_tot);
        if (!has_next) break;
        if (db) cur ^= 1u;
        p_prev = p;
        p = pn;
        ++it;
    }
    cluster_sync_(); /* the last histogram's per-lane sums published */
    if (!ab && k == 0u) cluster_reduce_(a, p, cl, part2 + (it & 1u) * 1024u, s_tot);
    cluster_sync_(); /* no CTA leaves while CTA 0 reads its sums */
    cp_async_wait_<0>();
    for (uint32_t b = 0; b < 2u; ++b)
        if ((pending >> b) & 1u) mbar_wait_(&s_mbar[b], (parity >> b) & 1u);
    bulk_wait_all_();
}

/* Cluster mode (float distance only), clusters of cl CTAs. */
__global__ void __launch_bounds__(512, 2) k_distance_cluster(DistArgs a, uint32_t db, uint32_t cl)
{
    extern __shared__ __align__(16) uint32_t s_mem[];
    const uint32_t M = *a.n_props;
    if (cluster_id_() >= M) return; /* whole clusters return */
    const uint32_t prow = strip_cap_rows(a.max_rows), tile_words = prow * 32u;
    /* [1 + db][cap rows][32] tiles (1024-byte aligned), a zero box, the row
     * carries, two last-column arrays, two 32 x 32 per-lane sum arrays */
    uint32_t* tiles = s_mem + ((1024u - (smem_u32_(s_mem) & 1023u)) & 1023u) / 4u;
    uint32_t* zero = tiles + (1u + db) * tile_words;
    uint32_t* carry = zero + kBox * kBox;
    uint32_t* P2 = carry + prow;
    float* part2 = reinterpret_cast<float*>(P2 + 2u * prow);
    __shared__ float s_tot[32];
    __shared__ uint32_t s_col[16][32];
    __shared__ __align__(16) uint32_t s_K[16][32];
    __shared__ __align__(8) uint64_t s_mbar[2];
    __shared__ uint32_t s_abort;
    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        mbar_init_(&s_mbar[0], kStripThreads);
        mbar_init_(&s_mbar[1], kStripThreads);
        mbar_init_fence_();
        s_abort = 0u;
    }
    for (uint32_t i = tid; i < kBox * kBox; i += kStripThreads) zero[i] = 0u;
    fence_proxy_async_(); /* the zero box, before box stores read it */
    __syncthreads();
    strip_cluster_(a, db, cl, M, tiles, tile_words, zero, carry, P2, part2, s_tot, s_col, s_K, s_mbar, &s_abort);
}

template <bool F64, bool SSD>
__global__ void __launch_bounds__(512, 2) k_distance_strip(DistArgs a, uint32_t db)
{
    extern __shared__ __align__(16) uint32_t s_mem[];
    const uint32_t tile_words = strip_cap_rows(a.max_rows) * 32u;
    /* [1 + db][cap rows][32] tiles, 1024-byte aligned (the launch reserves
     * 1024 bytes for this), a zero box, the row carries */
    uint32_t* tiles = s_mem + ((1024u - (smem_u32_(s_mem) & 1023u)) & 1023u) / 4u;
    uint32_t* zero = tiles + (1u + db) * tile_words;
    uint32_t* carry = zero + kBox * kBox;
    __shared__ float s_tot[32];
    __shared__ double s_tot64[32];
    __shared__ uint64_t s_hi[32], s_lo[32];
    __shared__ uint32_t s_col[16][32];             /* column totals of each warp's row segment */
    __shared__ __align__(16) uint32_t s_K[16][32]; /* per segment: prefix across the strip of its column carries */
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
    for (uint32_t i = tid; i < kBox * kBox; i += kStripThreads) zero[i] = 0u;
    fence_proxy_async_(); /* the zero box, before box stores read it */
    __syncthreads();

    uint32_t c0 = 0, cur = 0, parity = 0u; /* parity bit b: the phase of tile b's next fill */
    uint32_t pending = 1u;                  /* bit b: tile b has a fill in flight */
    strip_fill_(a, p, 0u, tiles, tid, &s_mbar[0]);
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
        cp_async_wait_<0>(); /* this thread's cell copies of the current strip have landed */
        /* the current strip's box copies (all threads' arrivals and bytes) */
        if (!mbar_wait_(&s_mbar[cur], (parity >> cur) & 1u)) {
            atomicOr(a.err, PCS_ERRBIT_TIMEOUT);
            s_abort = 1u;
        }
        parity ^= 1u << cur;
        pending &= ~(1u << cur);
        __syncwarp(); /* cells copied by other lanes of this warp */
        uint32_t* T = tiles + cur * tile_words;
        if (!ok) {
            if (tid == 0) {
                atomicOr(a.err, PCS_ERRBIT_ROWS);
                a.dist_f32[p] = __int_as_float(0x7fc00000);
            }
            __syncthreads();
            if (s_abort) break; /* a copy wait ran out (error word set) */
            if (db && has_next) {
                strip_fill_(a, pn, cn, tiles + (cur ^ 1u) * tile_words, tid, &s_mbar[cur ^ 1u]);
                pending |= 1u << (cur ^ 1u);
                cp_async_commit_();
            }
        } else {
            const uint32_t* __restrict__ refT = a.jobs[job].ref_sat_t;
            uint32_t* hist = a.hist + hoff;
            uint32_t* cum = a.cum_out ? a.cum_out + hoff : nullptr;
            const Seg sg = seg_(R, w);
            const uint32_t lc = l >> 2, lo = l & 3u;
            /* phase A1: column prefix within the segment, segment totals */
            uint32_t run = 0u;
            for (uint32_t r8 = sg.rb; r8 < sg.re; r8 += 8u) {
                uint32_t* t = T + (r8 << 5);
#pragma unroll
                for (uint32_t k = 0; k < 8u; ++k) {
                    uint32_t* q = t + (k << 5) + (((lc ^ k) << 2) | lo);
                    run += *q;
                    *q = run;
                }
            }
            s_col[w][l] = run;
            /* ... and the strip is zeroed in the histogram */
            uint32_t z;
            const TmapDev* map = prop_tmap_(a, p, job, z);
            if (map) {
                if (tid == 0u) {
                    const uint32_t nbox = (R + kBox - 1u) / kBox;
                    for (uint32_t b = 0; b < nbox; ++b) tma_store_3d_(map, c0, b * kBox, z, zero);
                    bulk_commit_();
                }
            } else if (c0 + l < B) {
                for (uint32_t r = sg.rb; r < min(sg.re, R); ++r) __stcs(hist + (uint64_t)r * B + c0 + l, 0u);
            }
            __syncthreads();
            if (s_abort) break; /* a copy wait ran out (error word set) */
            /* every warp is past the previous strip, whose tile the next
             * strip's copies now fill (with two tiles) */
            if (db && has_next) {
                strip_fill_(a, pn, cn, tiles + (cur ^ 1u) * tile_words, tid, &s_mbar[cur ^ 1u]);
                pending |= 1u << (cur ^ 1u);
                cp_async_commit_();
            }
            /* phase A2: column carry into the segment, scanned across the
             * strip; then the row prefix from the left strips' row carry */
            uint32_t cc = 0u;
            for (uint32_t q = 0; q < w; ++q) cc += s_col[q][l];
            s_K[w][l] = warp_scan_(cc, l);
            __syncwarp();
            const uint4* K4 = reinterpret_cast<const uint4*>(s_K[w]);
            for (uint32_t r = sg.rb + l; r < sg.re; r += 32u) {
                uint4* row4 = reinterpret_cast<uint4*>(T + (r << 5));
                const uint32_t m = r & 7u;
                uint32_t acc = c0 ? carry[r] : 0u;
                uint4 o = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (uint32_t j = 0; j < 8u; ++j) {
                    const uint4 v = row4[j ^ m];
                    const uint4 k = K4[j];
                    acc += v.x;
                    o.x = acc + k.x;
                    acc += v.y;
                    o.y = acc + k.y;
                    acc += v.z;
                    o.z = acc + k.z;
                    acc += v.w;
                    o.w = acc + k.w;
                    row4[j ^ m] = o;
                }
                carry[r] = o.w;
            }
            __syncthreads();
            /* phase B: columns c0 + 2w and c0 + 2w + 1; lane l reads rows
             * l, l + 32, ..., all congruent to l mod 8, so its swizzled
             * offset within a row is fixed */
            const uint32_t colA = c0 + 2u * w;
            if (colA < B) {
                const bool inB = colA + 1u < B;
                const uint32_t* Tl = T + ((((w >> 1) ^ (l & 7u)) << 2) | ((2u * w) & 3u));
                const uint32_t* refc = refT + (uint64_t)colA * R; /* this column pair (or lone last column) */
                float a2A = 0.0f, a2B = 0.0f;
                double a2dA = 0.0, a2dB = 0.0;
                /* the largest cumulative counts: the strip's and the observed histogram's last cells */
                const bool exact = !F64 && !SSD && !cum && T[sw_(R - 1u, 31u)] < kExactBelow &&
                                   __ldg(refT + pcs_sat_t_index(R - 1u, B - 1u, R, B)) < kExactBelow;
                if (exact && inB) {
                    const uint2* ref2 = reinterpret_cast<const uint2*>(refc);
#pragma unroll 4
                    for (uint32_t r = l; r < R; r += 32u) {
                        const uint2 s = *reinterpret_cast<const uint2*>(Tl + (r << 5));
                        const uint2 o = __ldg(ref2 + r);
                        const float dA = exact_diff_(s.x, o.x);
                        const float dB = exact_diff_(s.y, o.y);
                        a2A = __fadd_rn(a2A, __fmul_rn(dA, dA));
                        a2B = __fadd_rn(a2B, __fmul_rn(dB, dB));
                    }
                } else if (exact) {
#pragma unroll 4
                    for (uint32_t r = l; r < R; r += 32u) {
                        const float dA = exact_diff_(Tl[r << 5], __ldg(refc + r));
                        a2A = __fadd_rn(a2A, __fmul_rn(dA, dA));
                    }
                } else {
                    for (uint32_t r = l; r < R; r += 32u) {
                        const uint64_t at = (uint64_t)r * B + colA;
                        if (inB) {
                            const uint2 s = *reinterpret_cast<const uint2*>(Tl + (r << 5));
                            const uint2 o = __ldg(reinterpret_cast<const uint2*>(refc) + r);
                            term_<F64, SSD>(s.x, o.x, a2A, a2dA, shi, slo, cum, at);
                            term_<F64, SSD>(s.y, o.y, a2B, a2dB, shi, slo, cum, at + 1u);
                        } else {
                            term_<F64, SSD>(Tl[r << 5], __ldg(refc + r), a2A, a2dA, shi, slo, cum, at);
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
        /* this tile's generic accesses before its next box fill, which
         * follows the next strip's first barrier (with one tile, the
         * barrier before the refill below) */
        fence_proxy_async_();

        if (ok && c0 + 32u >= B) {
            /* last strip: reduce0 per logical warp (2w and 2w + 1), then over
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
                s_tot[2u * w] = ws0;
                s_tot[2u * w + 1u] = ws1;
                s_tot64[2u * w] = wd0;
                s_tot64[2u * w + 1u] = wd1;
                s_hi[2u * w] = shi;
                s_lo[2u * w] = slo;
                s_hi[2u * w + 1u] = 0u;
                s_lo[2u * w + 1u] = 0u;
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
            __syncthreads(); /* the one tile is free */
            strip_fill_(a, pn, cn, tiles, tid, &s_mbar[0]);
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
    bulk_wait_all_(); /* the zero box stores have read the zero box before the CTA's shared memory goes */
}

static const size_t kStripSmemMax = 220u * 1024u;

/* 1024 bytes to align the tiles, one or two tiles, the zero box, the row
 * carries; for cluster launches two of each strip's last column and of its
 * 32 x 32 per-lane sums */
static size_t strip_smem_bytes(uint32_t max_rows, bool db, uint32_t cl)
{
    const size_t rows = strip_cap_rows(max_rows);
    size_t n = 1024u + (db ? 2u : 1u) * rows * 32u * sizeof(uint32_t) + kBoxBytes + rows * sizeof(uint32_t);
    if (cl > 1u) n += 2u * (rows * sizeof(uint32_t) + 32u * 32u * sizeof(float));
    return n;
}

static bool use_strip(uint32_t max_rows, uint32_t cl) { return strip_smem_bytes(max_rows, false, cl) <= kStripSmemMax; }
static bool strip_db(uint32_t max_rows, uint32_t cl) { return strip_smem_bytes(max_rows, true, cl) <= kStripSmemMax; }

uint32_t distance_cluster_size(uint32_t max_rows, uint32_t max_bins)
{
    const uint32_t strips = (max_bins + 31u) / 32u;
    if (strips < 2u || strips > kMaxDistCluster) return 0u;
    return use_strip(max_rows, strips) ? strips : 0u;
}

size_t distance_smem_bytes(uint32_t max_rows, uint32_t cl)
{
    if (use_strip(max_rows, cl)) return strip_smem_bytes(max_rows, strip_db(max_rows, cl), cl);
    return ((size_t)max_rows + (size_t)kDistRowBlock * kPad) * sizeof(uint32_t);
}

uint32_t distance_block_threads(uint32_t max_rows) { return use_strip(max_rows, 0u) ? kStripThreads : 1024u; }

int distance_ctas_per_sm(uint32_t max_rows, uint32_t cl)
{
    const size_t smem = distance_smem_bytes(max_rows, cl);
    int n = 0;
    if (use_strip(max_rows, cl)) {
        cudaFuncSetAttribute(k_distance_strip<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_distance_strip<false, false>, (int)kStripThreads, smem);
    } else {
        cudaFuncSetAttribute(k_distance<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_distance<false>, 1024, smem);
    }
    return n > 0 ? n : 1;
}

/* Clusters of cl CTAs of k_distance_cluster that fit at once with `smem`
 * bytes of shared memory each, on the current device; queried once per
 * (device, cl, smem), since the plain form launches per proposal. */
static cudaError_t cluster_fit_(cudaLaunchConfig_t& cfg, uint32_t cl, size_t smem, int& fit)
{
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, size_t>, int> cache;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_tuple(dev, cl, smem);
    {
        std::lock_guard<std::mutex> g(mu);
        const auto it = cache.find(key);
        if (it != cache.end()) {
            fit = it->second;
            return cudaSuccess;
        }
    }
    e = cudaOccupancyMaxActiveClusters(&fit, (void*)k_distance_cluster, &cfg);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    cache[key] = fit;
    return cudaSuccess;
}

cudaError_t launch_distance(const DistArgs& a, uint32_t grid, cudaStream_t st, uint32_t cl)
{
    if (cl > 1u && (a.dist_f64 || a.ssd || a.cum_out || !use_strip(a.max_rows, cl) || cl > kMaxDistCluster)) cl = 0u;
    if (cl > 1u) {
        /* clusters of cl CTAs where the histograms are tall, or where every
         * histogram of the launch has a cluster to itself; as many clusters
         * as fit at once, at most one per histogram slot */
        const size_t smem = distance_smem_bytes(a.max_rows, cl);
        cudaError_t e = cudaFuncSetAttribute(k_distance_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cl;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.blockDim = dim3(kStripThreads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cfg.gridDim = dim3(cl);
        int fit = 0;
        e = cluster_fit_(cfg, cl, smem, fit);
        if (e != cudaSuccess) return e;
        if (fit > 0 && (strip_cap_rows(a.max_rows) >= kClusterRowsMin || grid <= (uint32_t)fit)) {
            cfg.gridDim = dim3(std::min<uint32_t>(grid, (uint32_t)fit) * cl);
            return cudaLaunchKernelEx(&cfg, k_distance_cluster, a, strip_db(a.max_rows, cl) ? 1u : 0u, cl);
        }
        cl = 0u;
    }
    const size_t smem = distance_smem_bytes(a.max_rows, 0u);
    if (use_strip(a.max_rows, 0u)) {
        void (*k)(DistArgs, uint32_t);
        if (a.dist_f64) k = a.ssd ? k_distance_strip<true, true> : k_distance_strip<true, false>;
        else k = a.ssd ? k_distance_strip<false, true> : k_distance_strip<false, false>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, kStripThreads, smem, st>>>(a, strip_db(a.max_rows, 0u) ? 1u : 0u);
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
