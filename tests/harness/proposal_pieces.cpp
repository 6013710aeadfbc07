/*
 * proposal_pieces.cpp -- test harness: exposes the library's host copy of the
 * proposal's pieces (pcs_proposal.h, shared with k_propose: the Poisson
 * sampler, the Box-Muller normal pair, the reflection into the prior box, the
 * parent pick) to the CPU tests, which check them against the distributions
 * and semantics they implement.  Built by tests/test_proposal_pieces.py into
 * a temporary directory; not part of the library.
 */
#include <stdint.h>

#include <cmath>
#include <vector>

#include "pcs_kernels.h"
#include "pcs_proposal.h"

extern "C" void draw_poisson(double lam, uint32_t n, uint64_t seed, uint32_t* out)
{
    uint32_t m0, m1;
    pcs_seed_masks(seed, &m0, &m1);
    const pcs::PoissonSetup ps = pcs::pcs_poisson_setup(lam);
    for (uint32_t i = 0; i < n; ++i) {
        /* distinct counters: video i mod 4096, slot i / 4096, generation 1 trial 0 */
        out[i] = pcs::pcs_poisson_draw(ps, i & 4095u, i >> 12, pcs_ctr_gen_trial(1u, 0u), m0, m1);
    }
}

extern "C" uint32_t draw_poisson_one(double lam, uint32_t video, uint32_t slot, uint64_t seed)
{
    uint32_t m0, m1;
    pcs_seed_masks(seed, &m0, &m1);
    return pcs::pcs_poisson(lam, video, slot, pcs_ctr_gen_trial(1u, 0u), m0, m1);
}

/* log(k!) for k below the device table's length, as the library's context
 * builds it */
static const double* logfact_table()
{
    static std::vector<double> t;
    if (t.empty()) {
        t.resize(pcs::kLogFactEntries);
        for (uint32_t k = 0; k < pcs::kLogFactEntries; ++k) t[k] = std::lgamma((double)k + 1.0);
    }
    return t.data();
}

/* PTRS iterations on n Philox draws (counters: index i, generation 1 trial
 * it): out[0] iterations the FP32 filter decided, out[1] of those decided
 * differently from the FP64 iteration (decision or k), out[2] the FP64
 * iteration's accepts, out[3] accepts the filter decided.  The draws come
 * from the low-order counter blocks and from a set with U's and V's top bits
 * placed near the tests' thresholds (every fourth). */
extern "C" void ptrs_check(double lam, uint32_t n, uint64_t seed, int with_table, uint64_t* out)
{
    uint32_t m0, m1;
    pcs_seed_masks(seed, &m0, &m1);
    pcs::PoissonSetup ps = pcs::pcs_poisson_setup(lam);
    if (with_table) {
        ps.logfact = logfact_table();
        ps.logfact_n = pcs::kLogFactEntries;
    }
    for (int j = 0; j < 4; ++j) out[j] = 0;
    for (uint32_t i = 0; i < n; ++i) {
        pcs_u4 r = pcs_draw(i & 4095u, pcs_ctr_tag(PCS_STREAM_POISSON, 1u), i >> 12, pcs_ctr_gen_trial(1u, 0u), m0, m1);
        if ((i & 3u) == 3u) {
            /* near a threshold: us near 0.07, 0.013 or 0.02; V near vr or us */
            const double th[3] = {0.07, 0.013, 0.02};
            const double us = th[r.y % 3u] + ((double)(r.w & 0xffffu) - 32768.0) * 1e-11;
            const double U = (r.y & 8u) ? 0.5 - us : us - 0.5;
            const uint32_t ux = (uint32_t)((U + 0.5) * 4294967296.0);
            r.x = ux;
            if (r.w & 0x10000u) {
                const double V = ((r.w & 0x20000u) ? ps.vr : us) + ((double)(r.z & 0xffffu) - 32768.0) * 1e-11;
                r.z = (uint32_t)(V * 4294967296.0);
            }
        }
        uint32_t ke = 0u, kf = 0u;
        const int de = pcs::pcs_ptrs_exact(ps, r, &ke);
        const int df = pcs::pcs_ptrs_filtered(ps, r, &kf);
        out[2] += de > 0;
        if (df >= 0) {
            out[0] += 1;
            out[3] += df > 0;
            if (df != de || (de > 0 && kf != ke)) out[1] += 1;
        }
    }
}

/* n full draws with the filter and without it: the count of differing draws */
extern "C" uint32_t poisson_filter_diffs(double lam, uint32_t n, uint64_t seed)
{
    uint32_t m0, m1;
    pcs_seed_masks(seed, &m0, &m1);
    pcs::PoissonSetup ps = pcs::pcs_poisson_setup(lam);
    ps.logfact = logfact_table();
    ps.logfact_n = pcs::kLogFactEntries;
    uint32_t diffs = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t gt = pcs_ctr_gen_trial(1u, 0u);
        diffs += pcs::pcs_poisson_draw<true>(ps, i & 4095u, i >> 12, gt, m0, m1) !=
                 pcs::pcs_poisson_draw<false>(ps, i & 4095u, i >> 12, gt, m0, m1);
    }
    return diffs;
}

/* The other pieces of proposal construction shared with k_propose. */
extern "C" double reflect(double bis, double lo, double hi) { return pcs::pcs_reflect(bis, lo, hi); }

extern "C" uint32_t pick(const double* wcum, uint32_t N, double u) { return pcs::pcs_pick(wcum, N, u); }

extern "C" void normals(uint32_t n, uint64_t seed, double* out)
{
    uint32_t m0, m1;
    pcs_seed_masks(seed, &m0, &m1);
    for (uint32_t i = 0; i < n; ++i) {
        const pcs_u4 r = pcs_draw(i, pcs_ctr_tag(PCS_STREAM_PERTURB, 0u), 0u, pcs_ctr_gen_trial(1u, 0u), m0, m1);
        pcs::pcs_normal2(r, out[2 * i], out[2 * i + 1]);
    }
}
