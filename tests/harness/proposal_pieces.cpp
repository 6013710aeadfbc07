/*
 * proposal_pieces.cpp -- test harness: exposes the library's host copy of the
 * proposal's pieces (pcs_proposal.h, shared with k_propose: the Poisson
 * sampler, the Box-Muller normal pair, the reflection into the prior box, the
 * parent pick) to the CPU tests, which check them against the distributions
 * and semantics they implement.  Built by tests/test_proposal_pieces.py into
 * a temporary directory; not part of the library.
 */
#include <stdint.h>

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
