/*
 * noalloc.cu -- pcs_scan_distance_noalloc: the cumulative-distance kernel
 * for callers that cannot allocate device memory.
 *
 * pcs_scan_distance stages its inputs and its working buffers (the observed
 * cumulative histogram's column-major copy for coalesced column sweeps, one
 * descriptor per histogram, a proposal counter) in memory it allocates per
 * call.  Some callers cannot let a library call cudaMalloc: a host
 * framework whose caching allocator owns all device memory and must not be
 * bypassed, a service running under a fixed device-memory budget, or a
 * real-time loop where an allocation may block on device synchronisation.  This entry
 * point takes device pointers for its inputs and outputs and keeps its
 * working buffers in one file-scope __device__ array of fixed size, so it
 * allocates nothing.
 *
 * Limits: rows * bins <= PCS_NOALLOC_MAX_CELLS (1,048,576 cells, 4 MiB of
 * column-major histogram copy) and count <= PCS_NOALLOC_MAX_COUNT (4096 histograms);
 * larger requests are rejected with PCS_ERR_INVALID_ARGUMENT.  The array
 * (about 4.7 MiB) is reserved on every GPU that loads the library, until the
 * process exits.
 *
 * The array's address is looked up once per device with cudaGetSymbolAddress
 * (the host-side name of a __device__ variable is only a stand-in): the first
 * call on a device does that lookup, so make the first call before any stream
 * capture.  The address is kept for the life of the process, so the entry
 * point does not survive cudaDeviceReset (or another release of the device's
 * primary context), after which the array is reloaded at another address.
 * Every call reuses the same array and overwrites what the previous call left
 * there; two calls whose work overlaps on the GPU (different streams, not
 * ordered) race on it and must not be issued.  Each call waits for its work
 * on the caller's stream, reads the kernel's error word back and reports a
 * raised word as PCS_ERR_DEVICE.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/pcs.h"
#include "pcs_common.h"
#include "pcs_kernels.h"

namespace pcs {
void set_last_error(const std::string& m);
}

namespace {

struct NoallocHeader {
    JobDev job;
    uint32_t n_props;
    uint32_t err;
};

constexpr size_t kHeaderBytes = (sizeof(NoallocHeader) + 255) / 256 * 256;
constexpr size_t kPropBytes = ((size_t)PCS_NOALLOC_MAX_COUNT * sizeof(PropDev) + 255) / 256 * 256;
constexpr size_t kScratchBytes = kHeaderBytes + kPropBytes + (size_t)PCS_NOALLOC_MAX_CELLS * sizeof(uint32_t);

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

/* Fills the scratch for one call: job descriptor, one descriptor per
 * histogram (consecutive R x B blocks of the caller's buffer), the proposal
 * count, a cleared error word, and the observed histogram's column-major
 * copy (pairs of columns interleaved, pcs_sat_t_index). */
__global__ void k_noalloc_setup(const uint32_t* __restrict__ ref_sat, uint32_t rows, uint32_t bins,
                                uint32_t count)
{
    NoallocHeader* h = reinterpret_cast<NoallocHeader*>(g_scratch);
    PropDev* props = reinterpret_cast<PropDev*>(g_scratch + kHeaderBytes);
    uint32_t* ref_t = reinterpret_cast<uint32_t*>(g_scratch + kHeaderBytes + kPropBytes);
    const uint64_t cells = (uint64_t)rows * bins;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (tid == 0) {
        JobDev j;
        memset(&j, 0, sizeof j);
        j.R = rows;
        j.B = bins;
        j.ref_sat = ref_sat;
        j.ref_sat_t = ref_t;
        h->job = j;
        h->n_props = count;
        h->err = 0u;
    }
    for (uint64_t q = tid; q < count; q += stride) {
        PropDev p;
        memset(&p, 0, sizeof p);
        p.hist_off = q * cells;
        props[q] = p;
    }
    for (uint64_t i = tid; i < cells; i += stride) {
        const uint64_t r = i / bins, b = i % bins;
        ref_t[pcs_sat_t_index((uint32_t)r, (uint32_t)b, rows, bins)] = ref_sat[i];
    }
}

std::mutex g_mu;
void* g_addr[64] = {};

/* Device address of the scratch array on the current device (looked up once). */
cudaError_t scratch_address(int device, void** out)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (!g_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        g_addr[device] = p;
    }
    *out = g_addr[device];
    return cudaSuccess;
}

pcs_status fail_(pcs_status s, const std::string& m)
{
    pcs::set_last_error(m);
    return s;
}

} // namespace

extern "C" pcs_status pcs_scan_distance_noalloc(uint32_t* d_hist, const uint32_t* d_ref_sat,
                                                uint32_t rows, uint32_t bins, uint32_t count,
                                                float* d_dist_f32, void* stream)
{
    if (!d_hist || !d_ref_sat || !d_dist_f32) return fail_(PCS_ERR_INVALID_ARGUMENT, "d_hist, d_ref_sat and d_dist_f32 must be device pointers");
    if (count == 0) return fail_(PCS_OK, "");
    if (rows == 0 || bins == 0) return fail_(PCS_ERR_INVALID_ARGUMENT, "rows and bins must be positive");
    if ((uint64_t)rows * bins > PCS_NOALLOC_MAX_CELLS)
        return fail_(PCS_ERR_INVALID_ARGUMENT, "rows * bins = " + std::to_string((uint64_t)rows * bins) +
                                                   " exceeds the allocation-free limit of " +
                                                   std::to_string(PCS_NOALLOC_MAX_CELLS) + " cells");
    if (count > PCS_NOALLOC_MAX_COUNT)
        return fail_(PCS_ERR_INVALID_ARGUMENT, "count = " + std::to_string(count) + " exceeds the allocation-free limit of " +
                                                   std::to_string(PCS_NOALLOC_MAX_COUNT) + " histograms");
    if (pcs::distance_smem_bytes(rows) > 227u * 1024u)
        return fail_(PCS_ERR_UNSUPPORTED, "too many histogram rows for one CTA");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    void* base = nullptr;
    if (e == cudaSuccess) e = scratch_address(device, &base);
    if (e != cudaSuccess) return fail_(PCS_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const uint64_t cells = (uint64_t)rows * bins;
    const uint32_t threads = 256;
    uint64_t blocks = (cells + threads - 1) / threads;
    if (blocks < (count + threads - 1) / threads) blocks = (count + threads - 1) / threads;
    if (blocks > 4096) blocks = 4096;
    k_noalloc_setup<<<(unsigned)blocks, threads, 0, st>>>(d_ref_sat, rows, bins, count);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_(PCS_ERR_CUDA, std::string("setup launch: ") + cudaGetErrorString(e));

    unsigned char* b = static_cast<unsigned char*>(base);
    NoallocHeader* h = reinterpret_cast<NoallocHeader*>(b);
    pcs::DistArgs d{};
    d.jobs = &h->job;
    d.props = reinterpret_cast<const PropDev*>(b + kHeaderBytes);
    d.n_props = &h->n_props;
    d.hist = d_hist;
    d.cum_out = nullptr;
    d.dist_f32 = d_dist_f32;
    d.dist_f64 = nullptr;
    d.ssd = nullptr;
    d.err = &h->err;
    d.max_rows = rows;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const uint32_t cap = (uint32_t)(pcs::distance_ctas_per_sm(rows) * sms);
    const uint32_t grid = count < cap ? count : cap;
    e = pcs::launch_distance(d, grid ? grid : 1u, st);
    if (e != cudaSuccess) return fail_(PCS_ERR_CUDA, std::string("distance launch: ") + cudaGetErrorString(e));
    /* wait for the work and read the kernel's error word back (a plain copy
     * into this stack variable: the runtime stages pageable copies itself) */
    uint32_t word = 0;
    e = cudaMemcpyAsync(&word, &h->err, sizeof word, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_(PCS_ERR_CUDA, std::string("distance kernel: ") + cudaGetErrorString(e));
    if (word) {
        char buf[96];
        snprintf(buf, sizeof buf, "distance kernel raised device error word 0x%x (32: histogram rows, 128: copy wait)", word);
        return fail_(PCS_ERR_DEVICE, buf);
    }
    return fail_(PCS_OK, "");
}
