// TEST INFRASTRUCTURE ONLY.  Runs the reference's own distance kernel,
// cusim::K_distance (src/gpu/cusim/kernel-distance.inl:81-241), on the GPU so
// that the distance fixtures are the reference kernel's outputs.  Built by
// oracle/build_ref_kdist.sh against the copy of kernel-distance.inl it
// prepares under oracle/_ref/kdist/ (one change there: the legacy
// `shfl.up.b32` of warp_prefix becomes `shfl.sync.up.b32` with a full-warp
// member mask, which ptxas requires for sm_70 and newer and which behaves the
// same for a full warp).  Called only by tests/golden/make_distance_golden.py.
//
// The kernel is launched exactly as the reference launches it: one block of
// 32 x 32 threads per histogram (src/gpu/detail/simulation_impl.inl:1090-1096),
// in place on the histogram, which it resets to zero.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <vector>

#include "kernel-distance.inl"

namespace {

template <typename tReal>
int run(const uint32_t* hist, const uint32_t* ref, unsigned rows, unsigned bins, unsigned count, tReal* out,
        int* zeroed, char* err, size_t errcap) {
    const size_t cells = size_t(rows) * bins;
    uint32_t *d_cur = nullptr, *d_ref = nullptr;
    tReal* d_out = nullptr;
    int rc = 0;
    auto fail = [&](cudaError_t e, const char* what) {
        if (err && errcap) snprintf(err, errcap, "%s: %s", what, cudaGetErrorString(e));
        rc = 1;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&d_cur, cells * count * sizeof(uint32_t))) != cudaSuccess) { fail(e, "cudaMalloc"); goto done; }
    if ((e = cudaMalloc(&d_ref, cells * sizeof(uint32_t))) != cudaSuccess) { fail(e, "cudaMalloc"); goto done; }
    if ((e = cudaMalloc(&d_out, count * sizeof(tReal))) != cudaSuccess) { fail(e, "cudaMalloc"); goto done; }
    if ((e = cudaMemcpy(d_cur, hist, cells * count * sizeof(uint32_t), cudaMemcpyHostToDevice)) != cudaSuccess) {
        fail(e, "cudaMemcpy"); goto done;
    }
    if ((e = cudaMemcpy(d_ref, ref, cells * sizeof(uint32_t), cudaMemcpyHostToDevice)) != cudaSuccess) {
        fail(e, "cudaMemcpy"); goto done;
    }
    for (unsigned q = 0; q < count; ++q)
        cusim::K_distance<tReal, unsigned><<<1, dim3(32, 32)>>>(d_out + q, rows, bins, d_cur + q * cells, d_ref);
    if ((e = cudaGetLastError()) != cudaSuccess) { fail(e, "launch"); goto done; }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) { fail(e, "K_distance"); goto done; }
    if ((e = cudaMemcpy(out, d_out, count * sizeof(tReal), cudaMemcpyDeviceToHost)) != cudaSuccess) {
        fail(e, "cudaMemcpy"); goto done;
    }
    if (zeroed) {
        std::vector<uint32_t> back(cells * count);
        if ((e = cudaMemcpy(back.data(), d_cur, back.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost)) != cudaSuccess) {
            fail(e, "cudaMemcpy"); goto done;
        }
        *zeroed = 1;
        for (uint32_t v : back)
            if (v != 0) { *zeroed = 0; break; }
    }
done:
    cudaFree(d_cur);
    cudaFree(d_ref);
    cudaFree(d_out);
    return rc;
}

}  // namespace

extern "C" int ref_kdist_f32(const uint32_t* hist, const uint32_t* ref, unsigned rows, unsigned bins, unsigned count,
                             float* out, int* zeroed, char* err, size_t errcap) {
    return run<float>(hist, ref, rows, bins, count, out, zeroed, err, errcap);
}

extern "C" int ref_kdist_f64(const uint32_t* hist, const uint32_t* ref, unsigned rows, unsigned bins, unsigned count,
                             double* out, int* zeroed, char* err, size_t errcap) {
    return run<double>(hist, ref, rows, bins, count, out, zeroed, err, errcap);
}
