/*
 * kernels_dist.cu -- fused 2-D prefix sum + cumulative distance.
 *
 * Follows cusim::K_distance (src/gpu/cusim/kernel-distance.inl:81-241), which
 * runs one 32x32 block per proposal over the whole R x B histogram twice
 * (row scans, then column scans accumulating (cum - ref)^2) and zeroes the
 * histogram for reuse.  Here one 1024-thread CTA per proposal streams the
 * histogram in strips of 32 DE columns and blocks of rows through shared
 * memory:
 *   phase A  warp w scans rows w, w+32, ... of the strip (coalesced 128-byte
 *            loads, warp shuffle scan, per-row carry across strips kept in
 *            shared memory) and writes zeros back;
 *   phase B  warp w scans column c0+w down the rows (shuffle scan, carry in a
 *            register), reads the observed cumulative histogram from its
 *            transposed copy (coalesced), and lane l accumulates
 *            (float(cum) - float(ref))^2 for rows l, l+32, ...
 * Warp w / lane l therefore own exactly the columns and rows they own in the
 * reference launch, so the per-lane sums, the shfl_down trees of reduce0
 * (:69-78) and the final per-warp tree reproduce the reference's float
 * result bit for bit (each operation is an explicit round-to-nearest
 * intrinsic, as in a build without FMA contraction).  The exact integer sum
 * of squares is accumulated alongside.
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

/* Strip kernel: 16 warps, full-height strips of 32 DE columns.
 *
 * Phase A: warp w scans rows w, w+16, ... of the strip, eight rows' loads in
 * flight at a time (8 x 128 B per warp, 32 KB per SM at two CTAs: about the
 * bandwidth-latency product of one SM's share of HBM), carry per row in
 * shared memory, zeros written back.
 * Phase B: warp w scans two columns of the strip at once, c0+w for logical
 * warp w and c0+w+16 for logical warp w+16 of the reference's 32x32 launch,
 * so every lane keeps the reference's per-lane sums in two accumulators.
 * SSD: also accumulate the exact integer sum of squares (128-bit per lane);
 * the PMC rounds do not ask for it, the parity entry point does.
 * Two CTAs fit per SM up to ~830 rows; the tile takes R x 33 words. */
const uint32_t kStripThreads = 512;
const int kStripRowsInFlight = 8;

template <bool F64, bool SSD>
__global__ void __launch_bounds__(512, 2) k_distance_strip(DistArgs a)
{
    extern __shared__ uint32_t s_mem[];
    uint32_t* carry = s_mem;            /* [max_rows] */
    uint32_t* T = s_mem + a.max_rows;   /* [max_rows][kPad] */
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
        const uint32_t* __restrict__ refT = a.jobs[job].ref_sat_t;
        uint32_t* hist = a.hist + hoff;
        uint32_t* cum = a.cum_out ? a.cum_out + hoff : nullptr;
        if (R > a.max_rows) {
            if (tid == 0) {
                atomicOr(a.err, PCS_ERRBIT_ROWS);
                a.dist_f32[p] = __int_as_float(0x7fc00000);
            }
            continue;
        }
        for (uint32_t r = tid; r < R; r += kStripThreads) carry[r] = 0u;
        __syncthreads();

        float acc0 = 0.0f, acc1 = 0.0f;
        double accd0 = 0.0, accd1 = 0.0;
        uint64_t shi = 0, slo = 0;
        for (uint32_t c0 = 0; c0 < B; c0 += 32u) {
            const uint32_t c = c0 + l;
            const bool cin = c < B;
            /* phase A */
            for (uint32_t r = w; r < R; r += 16u * kStripRowsInFlight) {
                uint32_t v[kStripRowsInFlight];
#pragma unroll
                for (int i = 0; i < kStripRowsInFlight; ++i) {
                    const uint32_t ri = r + 16u * (uint32_t)i;
                    v[i] = (ri < R && cin) ? __ldcs(hist + (uint64_t)ri * B + c) : 0u;
                }
#pragma unroll
                for (int i = 0; i < kStripRowsInFlight; ++i) {
                    const uint32_t ri = r + 16u * (uint32_t)i;
                    if (ri < R) {
                        const uint32_t cr = carry[ri];
                        const uint32_t s = warp_scan_(v[i], l) + cr;
                        T[ri * kPad + l] = s;
                        if (cin) __stcs(hist + (uint64_t)ri * B + c, 0u);
                        __syncwarp();
                        if (l == 31u) carry[ri] = s;
                    }
                }
            }
            __syncthreads();
            /* phase B: columns c0 + w and c0 + w + 16 */
            const uint32_t colA = c0 + w, colB = c0 + w + 16u;
            const bool inA = colA < B, inB = colB < B;
            uint32_t carA = 0u, carB = 0u;
            float a2A = 0.0f, a2B = 0.0f;
            double a2dA = 0.0, a2dB = 0.0;
            if (inA) {
                for (uint32_t r0 = 0; r0 < R; r0 += 32u) {
                    const uint32_t r = r0 + l;
                    const bool valid = r < R;
                    const uint32_t vA = valid ? T[r * kPad + w] : 0u;
                    const uint32_t vB = (valid && inB) ? T[r * kPad + w + 16u] : 0u;
                    const uint32_t refA = valid ? __ldg(refT + (uint64_t)colA * R + r) : 0u;
                    const uint32_t refB = (valid && inB) ? __ldg(refT + (uint64_t)colB * R + r) : 0u;
                    const uint32_t sA = warp_scan_(vA, l) + carA;
                    const uint32_t sB = warp_scan_(vB, l) + carB;
                    carA = __shfl_sync(0xFFFFFFFFu, sA, 31);
                    carB = __shfl_sync(0xFFFFFFFFu, sB, 31);
                    if (valid) {
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
                acc0 = __fadd_rn(acc0, a2A);
                if (F64) accd0 = __dadd_rn(accd0, a2dA);
                if (inB) {
                    acc1 = __fadd_rn(acc1, a2B);
                    if (F64) accd1 = __dadd_rn(accd1, a2dB);
                }
            }
            __syncthreads();
        }

        /* reduce0 per logical warp (w and w + 16), then over the 32 totals */
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
    }
}

static size_t strip_smem_bytes(uint32_t max_rows)
{
    return ((size_t)max_rows * (1u + kPad)) * sizeof(uint32_t);
}

static bool use_strip(uint32_t max_rows) { return strip_smem_bytes(max_rows) <= 220u * 1024u; }

size_t distance_smem_bytes(uint32_t max_rows)
{
    if (use_strip(max_rows)) return strip_smem_bytes(max_rows);
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
        void (*k)(DistArgs);
        if (a.dist_f64) k = a.ssd ? k_distance_strip<true, true> : k_distance_strip<true, false>;
        else k = a.ssd ? k_distance_strip<false, true> : k_distance_strip<false, false>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, kStripThreads, smem, st>>>(a);
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
