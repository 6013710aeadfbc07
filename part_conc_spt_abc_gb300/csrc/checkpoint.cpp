/*
 * checkpoint.cpp -- exact checkpoint / resume of an estimation job.
 *
 * Every random draw of a job is a pure function of (seed, generation, slot,
 * trial, ...) (Philox counters, pcs_common.h), so the whole future of a job
 * is fixed by its population state between two rounds: the committed and
 * running populations, weights, distances, perturbation factor, the per-slot
 * search state and the generation's counters.  Saving exactly that and
 * loading it into a fresh job created with the same parameters, observed
 * data and seed continues bit for bit as the original would have; the
 * round capacity and which other jobs share the rounds do not matter, as
 * for an uninterrupted run.  The reference has no counterpart (its host
 * std::mt19937 stream and in-flight queues make a resume inexact).
 *
 * Blob layout (little-endian, as the host stores it): a header
 * {magic, version, N, P, C, Z, V, R, B, model, fingerprint, seed, bytes},
 * the scalar counters, then theta, theta_new [N*P], w, wcum, dist, dist_new
 * [N] (f64), factor [P*P] (f64), next_trial, pending, accepted [N] (u32).
 * The fingerprint is a 32-bit FNV-1a hash of every job parameter that
 * shapes the job's future (all of pcs_params but max_generations, which a
 * resumed job takes from its own parameters) and of the observed data
 * (detection area, frame interval, frame counts, K and DE); a checkpoint
 * whose fingerprint differs from the loading job's is refused.
 */
#include <cstring>
#include <vector>

#include "engine.h"

namespace pcs {

namespace {

const uint64_t kMagic = 0x31544B4353435000ull; /* "\0PCSCKT1" */
const uint32_t kVersion = 2;

struct CkptHeader {
    uint64_t magic;
    uint32_t version, N, P, C, Z, V, R, B, model, fingerprint;
    uint64_t seed;
    uint64_t bytes;
};

/* FNV-1a, 32 bits, over explicit fields (no struct padding bytes) */
struct Fnv {
    uint32_t h = 2166136261u;
    void bytes(const void* p, size_t n)
    {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) {
            h ^= c[i];
            h *= 16777619u;
        }
    }
    template <class T> void add(const T& v) { bytes(&v, sizeof v); }
};

uint32_t job_fingerprint(const pcs_params& p, double ax, double ay, double deltat, const std::vector<uint32_t>& frames,
                         const std::vector<uint32_t>& K, const std::vector<double>& DE)
{
    Fnv f;
    f.add(p.model);
    f.add(p.weighting_scheme);
    f.add(p.component_count);
    f.add(p.kmin);
    f.add(p.de_bin_count);
    f.add(p.abc_sample_count);
    f.add(p.avg_trial_count);
    f.add(p.gamma_adaptive);
    const double d[] = {p.Lx, p.Ly, p.Lz, p.gamma_initial, p.delta_gamma, p.ub_de, p.lb_m, p.ub_m, p.lb_s, p.ub_s,
                        p.lb_c, p.ub_c, p.lb_az, p.ub_az, p.temperature, p.viscosity, p.quantile, ax, ay, deltat};
    f.bytes(d, sizeof d);
    f.add(p.schedule);
    f.add(p.perturbation);
    f.add(p.reference_initial_gamma);
    f.add(p.distance_double);
    f.bytes(frames.data(), frames.size() * sizeof(uint32_t));
    f.bytes(K.data(), K.size() * sizeof(uint32_t));
    f.bytes(DE.data(), DE.size() * sizeof(double));
    return f.h;
}

struct CkptScalars {
    double gamma;
    uint64_t trials, simulations, accepted_total, accepted_gen, particle_steps;
    uint32_t generation, pending_count, iterations, converged, done, pad;
};

struct Span {
    void* dev;
    size_t bytes;
};

void spans(const JobPmcDev& pm, uint32_t N, uint32_t P, Span out[11])
{
    const size_t nP = (size_t)N * P;
    out[0] = {pm.theta, nP * 8};
    out[1] = {pm.theta_new, nP * 8};
    out[2] = {pm.w, (size_t)N * 8};
    out[3] = {pm.wcum, (size_t)N * 8};
    out[4] = {pm.dist, (size_t)N * 8};
    out[5] = {pm.dist_new, (size_t)N * 8};
    out[6] = {pm.factor, (size_t)P * P * 8};
    out[7] = {pm.next_trial, (size_t)N * 4};
    out[8] = {pm.pending, (size_t)N * 4};
    out[9] = {pm.accepted, (size_t)N * 4};
    out[10] = {nullptr, 0};
}

} // namespace

size_t Job::checkpoint_bytes() const
{
    const size_t nP = (size_t)N * P;
    return sizeof(CkptHeader) + sizeof(CkptScalars) + 2 * nP * 8 + 4 * (size_t)N * 8 + (size_t)P * P * 8 +
           3 * (size_t)N * 4;
}

void Job::save_state(void* buf) const
{
    if (!initialised) throw Error(PCS_ERR_INVALID_ARGUMENT, "job has no state yet (no generation has run)");
    char* p8 = static_cast<char*>(buf);
    CkptHeader h{};
    h.magic = kMagic;
    h.version = kVersion;
    h.N = N;
    h.P = P;
    h.C = C;
    h.Z = Z;
    h.V = V;
    h.R = R;
    h.B = B;
    h.model = (uint32_t)p.model;
    h.fingerprint = job_fingerprint(p, ax, ay, deltat, frames, K, DE);
    h.seed = seed;
    h.bytes = checkpoint_bytes();
    std::memcpy(p8, &h, sizeof h);
    p8 += sizeof h;
    const JobPmcDev& s = status;
    CkptScalars c{};
    c.gamma = s.gamma;
    c.trials = s.trials;
    c.simulations = s.simulations;
    c.accepted_total = s.accepted_total;
    c.accepted_gen = s.accepted_gen;
    c.particle_steps = s.particle_steps;
    c.generation = s.generation;
    c.pending_count = s.pending_count;
    c.iterations = s.iterations;
    c.converged = s.converged;
    c.done = s.done;
    std::memcpy(p8, &c, sizeof c);
    p8 += sizeof c;
    Span sp[11];
    spans(pm, N, P, sp);
    PCS_CUDA(cudaSetDevice(ctx->device));
    PCS_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; sp[i].dev; ++i) {
        PCS_CUDA(cudaMemcpy(p8, sp[i].dev, sp[i].bytes, cudaMemcpyDeviceToHost));
        p8 += sp[i].bytes;
    }
}

void Job::load_state(const void* buf, size_t bytes)
{
    if (initialised || slot >= 0)
        throw Error(PCS_ERR_INVALID_ARGUMENT, "a checkpoint loads only into a job that has not run yet");
    if (bytes < sizeof(CkptHeader)) throw Error(PCS_ERR_INVALID_ARGUMENT, "checkpoint too short");
    const char* p8 = static_cast<const char*>(buf);
    CkptHeader h;
    std::memcpy(&h, p8, sizeof h);
    if (h.magic != kMagic || h.version != kVersion)
        throw Error(PCS_ERR_INVALID_ARGUMENT, "not a checkpoint of this library version");
    if (h.N != N || h.P != P || h.C != C || h.Z != Z || h.V != V || h.R != R || h.B != B ||
        h.model != (uint32_t)p.model || h.seed != seed)
        throw Error(PCS_ERR_INVALID_ARGUMENT,
                    "checkpoint was taken from a job with other parameters, observed data shape or seed");
    if (h.fingerprint != job_fingerprint(p, ax, ay, deltat, frames, K, DE))
        throw Error(PCS_ERR_INVALID_ARGUMENT,
                    "checkpoint was taken from a job with other parameters or observed data");
    if (h.bytes != checkpoint_bytes() || bytes < h.bytes) throw Error(PCS_ERR_INVALID_ARGUMENT, "checkpoint size mismatch");
    p8 += sizeof h;
    CkptScalars c;
    std::memcpy(&c, p8, sizeof c);
    p8 += sizeof c;
    PCS_CUDA(cudaSetDevice(ctx->device));
    build_device_state(); /* arena, observed histogram, descriptors */
    Span sp[11];
    spans(pm, N, P, sp);
    for (int i = 0; sp[i].dev; ++i) {
        PCS_CUDA(cudaMemcpy(sp[i].dev, p8, sp[i].bytes, cudaMemcpyHostToDevice));
        p8 += sp[i].bytes;
    }
    pm.gamma = c.gamma;
    pm.trials = c.trials;
    pm.simulations = c.simulations;
    pm.accepted_total = c.accepted_total;
    pm.accepted_gen = c.accepted_gen;
    pm.particle_steps = c.particle_steps;
    pm.generation = c.generation;
    pm.pending_count = c.pending_count;
    pm.iterations = c.iterations;
    pm.converged = c.converged;
    pm.done = c.done;
    pm.gen_ended = 0u;
    pm.status = 0u;
    /* a resumed job obeys the cap of the parameters it was created with */
    if (!pm.done && pm.max_generations && pm.iterations > pm.max_generations) pm.done = 1u;
    status = pm;
    finished = pm.done != 0u;
}

} // namespace pcs
