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

size_t distance_smem_bytes(uint32_t max_rows)
{
    return ((size_t)max_rows + (size_t)kDistRowBlock * kPad) * sizeof(uint32_t);
}

cudaError_t launch_distance(const DistArgs& a, uint32_t grid, cudaStream_t st)
{
    const size_t smem = distance_smem_bytes(a.max_rows);
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
