/*
 * ref_harness.cpp -- runs the reference's OWN source on the host, to pin the
 * oracle.  TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh from the
 * reference sources where they lie (nothing is copied), output goes to
 * oracle/_ref/ (git-ignored), and only tests/golden/make_golden.py and the
 * CPU tests load it.
 *
 * What it exposes:
 *   ref_simulate_replay  cusim::K_simulate_system (src/gpu/cusim/kernel-simulate.inl:106-185)
 *                        instantiated with the reference's SimulateSetup/SimulateRun
 *                        (kernel-simulate.cuh:13-63) and HistogramRecorder
 *                        (cusim/histogram2d.inl:306-321), fed by a replay
 *                        random source that satisfies the reference's Random
 *                        interface (src/gpu/random.cuh:50-142).  "Launched" as
 *                        the reference launches it: ceil(V/4) blocks x 128 threads
 *                        (detail/simulation_impl.inl:655-656), one warp per video.
 *   ref_input_load       input::load (src/gpu/shared/input.cpp:101-235)
 *   ref_output_write     output::write (src/gpu/shared/output.cpp:184-258)
 *
 * Built with -ffp-contract=off so every float operation in the kernel
 * template is a single rounded IEEE operation.
 */
#include "cuda_runtime.h" /* host stand-in from oracle/ref_shim */

#include <cxxabi.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <exception>
#include <limits>
#include <string>
#include <typeinfo>
#include <vector>

#include "shared/common.hpp"
#include "shared/input.hpp"
#include "shared/output.hpp"
#include "cusim/histogram2d.cuh"
#include "cusim/kernel-simulate.cuh"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

namespace {

/* Random source replaying pre-generated draws.  Thread gtid belongs to video
 * gtid/32 and walks particles gtid%32, +32, ... (kernel-simulate.inl:123-136);
 * each particle first draws its uniforms (make_particle) and then three
 * normals per frame, so a new particle begins at the first uniform draw after
 * the previous particle's uniforms were used up. */
struct ReplayData {
    using result_type = float;
    const float* uniforms;
    const float* normals;
    unsigned stride;
    const std::uint64_t* videoBase;
    unsigned nU;
    struct Factory;
};

struct ReplayData::Factory {
    struct Instance {
        unsigned v, p, u, n;
        bool started;
        Instance(unsigned gtid, ReplayData&) : v(gtid / 32), p(gtid % 32), u(0), n(0), started(false) {}
        float uniform01(unsigned, ReplayData& d)
        {
            if (started && u == d.nU) {
                p += 32;
                u = 0;
                n = 0;
            }
            started = true;
            std::uint64_t idx = d.videoBase[v] + p;
            return d.uniforms[idx * 4 + u++];
        }
        float normal01(unsigned, ReplayData& d)
        {
            std::uint64_t idx = d.videoBase[v] + p;
            float r = d.normals[(idx * d.stride + n / 3) * 3 + n % 3];
            ++n;
            return r;
        }
        void store(unsigned, ReplayData&) {}
    };
};

template <class Setup, class Run>
void launch_(Setup const& setup, Run const& run, cusim::HistogramRecorder<std::uint32_t, float> rec,
             ReplayData rd, unsigned V)
{
    unsigned const blocks = (V + 4 - 1) / 4;
    blockDim = dim3(128, 1, 1);
    gridDim = dim3(blocks, 1, 1);
    for (unsigned b = 0; b < blocks; ++b)
        for (unsigned t = 0; t < 128; ++t) {
            blockIdx = uint3{b, 0, 0};
            threadIdx = uint3{t, 0, 0};
            cusim::K_simulate_system(setup, run, rec, rd);
        }
}

template <EModel kModel, class CC, class ZC>
void run_model_(unsigned C, unsigned V, unsigned kmin, float fourDeltaT, const float* halfL,
                const float* halfA, const std::uint32_t* frames, const std::uint32_t* particles,
                const float* halfAz, const float* preCompProb, const float* rwsd,
                cusim::HistogramRecorder<std::uint32_t, float> rec, ReplayData rd,
                std::vector<float>& dynHalfAz, std::vector<float>& dynPre, std::vector<float>& dynRw)
{
    using Setup = cusim::SimulateSetup<std::uint32_t, float, kModel, CC>;
    using Run = cusim::SimulateRun<std::uint32_t, float, ZC, CC>;
    Setup setup{CC(C)};
    setup.jobCount = V;
    setup.kmin = kmin;
    setup.fourDeltaT = fourDeltaT;
    setup.halfLx = halfL[0];
    setup.halfLy = halfL[1];
    setup.halfLz = halfL[2];
    setup.halfAx = halfA[0];
    setup.halfAy = halfA[1];

    Run run;
    run.frames = frames;
    run.particles = particles;
    unsigned const Z = (kModel == EModel::discreteFixedZ) ? 1u : C;
    float* hz = cusim::acquire_host_ptr(run.halfAz, ZC(Z));
    float* pc = cusim::acquire_host_ptr(run.preCompProb, CC(C));
    float* rw = cusim::acquire_host_ptr(run.randWalkStddev, CC(C));
    for (unsigned i = 0; i < Z; ++i) hz[i] = halfAz[i];
    for (unsigned i = 0; i < C; ++i) {
        pc[i] = preCompProb[i];
        rw[i] = rwsd[i];
    }
    /* Dynamic counts hold device pointers; in the shim device memory is host memory. */
    dynHalfAz.assign(hz, hz + Z);
    dynPre.assign(pc, pc + C);
    dynRw.assign(rw, rw + C);
    cusim::upload_from_host_ptr(run.halfAz, hz, ZC(Z), [&] { return dynHalfAz.data(); });
    cusim::upload_from_host_ptr(run.preCompProb, pc, CC(C), [&] { return dynPre.data(); });
    cusim::upload_from_host_ptr(run.randWalkStddev, rw, CC(C), [&] { return dynRw.data(); });

    launch_(setup, run, rec, rd, V);

    cusim::release_host_ptr(run.halfAz, hz);
    cusim::release_host_ptr(run.preCompProb, pc);
    cusim::release_host_ptr(run.randWalkStddev, rw);
}

std::string describe_(std::exception const& e)
{
    int status = 0;
    char* name = abi::__cxa_demangle(typeid(e).name(), nullptr, nullptr, &status);
    std::string out = (status == 0 && name) ? name : typeid(e).name();
    std::free(name);
    out += ": ";
    out += e.what();
    try {
        std::rethrow_if_nested(e);
    } catch (std::exception const& n) {
        out += " | nested " + describe_(n);
    } catch (...) {
    }
    return out;
}

void copy_err_(std::string const& s, char* err, std::size_t cap)
{
    if (!err || !cap) return;
    std::snprintf(err, cap, "%s", s.c_str());
}

} // namespace

extern "C" {

/* model: 0 discrete-fixed-depth, 1 discrete-variable-depth.  hist (R x B) is
 * overwritten.  Returns 0 on success. */
int ref_simulate_replay(int model, unsigned C, unsigned V, unsigned kmin, float fourDeltaT,
                        const float* halfL, const float* halfA, const std::uint32_t* frames,
                        const std::uint32_t* particles, const float* halfAz,
                        const float* preCompProb, const float* rwsd, float dde, unsigned R,
                        unsigned B, const float* uniforms, const float* normals, unsigned stride,
                        std::uint32_t* hist, char* err, std::size_t errcap)
{
    try {
        cusim::Histogram2D<std::uint32_t> h(R, B);
        h.clear();
        cusim::HistogramRecorder<std::uint32_t, float> rec(h, dde);

        std::vector<std::uint64_t> base(V + 1, 0);
        for (unsigned v = 0; v < V; ++v) base[v + 1] = base[v] + particles[v];
        ReplayData rd{uniforms, normals, stride, base.data(), C == 1 ? 3u : 4u};

        std::vector<float> a, b, c;
        using S1 = StaticValue<unsigned, 1>;
        using S2 = StaticValue<unsigned, 2>;
        using D = DynamicValue<unsigned>;
        if (model == 0) {
            if (C == 1)
                run_model_<EModel::discreteFixedZ, S1, S1>(C, V, kmin, fourDeltaT, halfL, halfA, frames, particles, halfAz, preCompProb, rwsd, rec, rd, a, b, c);
            else if (C == 2)
                run_model_<EModel::discreteFixedZ, S2, S1>(C, V, kmin, fourDeltaT, halfL, halfA, frames, particles, halfAz, preCompProb, rwsd, rec, rd, a, b, c);
            else
                run_model_<EModel::discreteFixedZ, D, S1>(C, V, kmin, fourDeltaT, halfL, halfA, frames, particles, halfAz, preCompProb, rwsd, rec, rd, a, b, c);
        } else {
            if (C == 1)
                run_model_<EModel::discreteVariableZ, S1, S1>(C, V, kmin, fourDeltaT, halfL, halfA, frames, particles, halfAz, preCompProb, rwsd, rec, rd, a, b, c);
            else if (C == 2)
                run_model_<EModel::discreteVariableZ, S2, S2>(C, V, kmin, fourDeltaT, halfL, halfA, frames, particles, halfAz, preCompProb, rwsd, rec, rd, a, b, c);
            else
                run_model_<EModel::discreteVariableZ, D, D>(C, V, kmin, fourDeltaT, halfL, halfA, frames, particles, halfAz, preCompProb, rwsd, rec, rd, a, b, c);
        }
        std::memcpy(hist, h.device_ptr(), sizeof(std::uint32_t) * std::size_t(R) * B);
        return 0;
    } catch (std::exception const& e) {
        copy_err_(describe_(e), err, errcap);
        return -1;
    }
}

struct ref_params {
    int model;
    int weighting_scheme;
    std::uint64_t component_count, kmin, de_bin_count, abc_sample_count, avg_trial_count;
    double Lx, Ly, Lz, gamma, delta_gamma;
    int adaptive_gamma;
    double de_lower, de_upper, m_lower, m_upper, s_lower, s_upper, c_lower, c_upper, az_lower,
        az_upper;
    double ax, ay, delta_t;
    std::uint64_t n_frames, n_K, n_DE;
    char output_file_path[1024];
};

int ref_input_load(const char* input, const char* data, ref_params* out, std::uint64_t* frames,
                   std::size_t frames_cap, std::uint64_t* K, std::size_t K_cap, double* DE,
                   std::size_t DE_cap, char* err, std::size_t errcap)
{
    try {
        input::Parameters p = input::load(input, data);
        out->model = int(p.model);
        out->weighting_scheme = int(p.weightingScheme);
        out->component_count = p.componentCount;
        out->kmin = p.kmin;
        out->de_bin_count = p.deBinCount;
        out->abc_sample_count = p.abcSampleCount;
        out->avg_trial_count = p.avgTrialCount;
        out->Lx = p.Lx;
        out->Ly = p.Ly;
        out->Lz = p.Lz;
        out->gamma = p.gamma;
        out->delta_gamma = p.deltaGamma;
        out->adaptive_gamma = p.adaptiveGamma ? 1 : 0;
        out->de_lower = p.de.lower;
        out->de_upper = p.de.upper;
        out->m_lower = p.m.lower;
        out->m_upper = p.m.upper;
        out->s_lower = p.s.lower;
        out->s_upper = p.s.upper;
        out->c_lower = p.c.lower;
        out->c_upper = p.c.upper;
        out->az_lower = p.az.lower;
        out->az_upper = p.az.upper;
        out->ax = p.ax;
        out->ay = p.ay;
        out->delta_t = p.deltaT;
        out->n_frames = p.frameCounts.size();
        out->n_K = p.Ks.size();
        out->n_DE = p.DEs.size();
        std::snprintf(out->output_file_path, sizeof out->output_file_path, "%s", p.outputFilePath.c_str());
        for (std::size_t i = 0; i < p.frameCounts.size() && i < frames_cap; ++i) frames[i] = p.frameCounts[i];
        for (std::size_t i = 0; i < p.Ks.size() && i < K_cap; ++i) K[i] = p.Ks[i];
        for (std::size_t i = 0; i < p.DEs.size() && i < DE_cap; ++i) DE[i] = p.DEs[i];
        return 0;
    } catch (std::exception const& e) {
        copy_err_(describe_(e), err, errcap);
        return -1;
    }
}

int ref_output_write(const char* path, int model, int weighting_scheme, std::uint64_t abc,
                     std::uint64_t C, std::uint64_t Z, const double* m, std::size_t nm,
                     const double* c, std::size_t nc, const double* az, std::size_t naz,
                     const double* dist, std::size_t nd, const double* w, std::size_t nw,
                     int converged, double gamma, const char* const* meta_keys,
                     const char* const* meta_values, std::size_t nmeta)
{
    try {
        output::Output o;
        o.model = EModel(model);
        o.weightingScheme = EWeightingScheme(weighting_scheme);
        o.abcSampleCount = abc;
        o.componentCount = C;
        o.zComponentCount = Z;
        o.m.assign(m, m + nm);
        o.c.assign(c, c + nc);
        o.az.assign(az, az + naz);
        o.dist.assign(dist, dist + nd);
        o.w.assign(w, w + nw);
        o.converged = converged != 0;
        o.gamma = gamma;
        for (std::size_t i = 0; i < nmeta; ++i) o.meta[meta_keys[i]] = meta_values[i];
        output::write(path, o);
        return 0;
    } catch (...) {
        return -1;
    }
}

} // extern "C"
