/*
 * tmap.cpp -- TMA tensor maps over histogram areas (host side).
 *
 * The distance kernel moves each 32-column strip of a histogram into shared
 * memory with tensor-map box copies (32 x 32 cells, 128-byte swizzle) and
 * zeroes it in global memory with box stores from a zero box.  A map spans
 * `depth` histograms of R x B cells laid one after another, as a job's
 * histograms are in a round; rows past R and columns past B lie outside the
 * tensor, so loads there read zeros and stores there are dropped.  The
 * encoder is the driver's cuTensorMapEncodeTiled, found through the runtime
 * (no link against the driver library).
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "pcs_kernels.h"

namespace pcs {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

} // namespace

bool encode_hist_tmap(TmapDev* out, const uint32_t* base, uint32_t R, uint32_t B, uint64_t depth)
{
    static_assert(sizeof(CUtensorMap) == sizeof(TmapDev), "a tensor map is 128 bytes");
    std::memset(out, 0, sizeof *out);
    /* boxes of 32 x 32 cells within the tensor's extent; strides of whole
     * 16-byte units; a 16-byte aligned base */
    if (R < 32u || B < 32u || (B & 3u) != 0u || depth == 0u || depth > 0xFFFFFFFFull ||
        (reinterpret_cast<uintptr_t>(base) & 15u) != 0u)
        return false;
    const PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return false;
    CUtensorMap m;
    const cuuint64_t dims[3] = {B, R, depth};
    const cuuint64_t strides[2] = {(cuuint64_t)B * 4u, (cuuint64_t)R * B * 4u};
    const cuuint32_t box[3] = {32u, 32u, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    const CUresult e = fn(&m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<uint32_t*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (e != CUDA_SUCCESS) return false;
    std::memcpy(out, &m, sizeof m);
    return true;
}

} // namespace pcs
