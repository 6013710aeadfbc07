/*
 * poisson_draws.cpp -- test harness: exposes the library's host copy of the
 * proposal's Poisson sampler (pcs_proposal.h, shared with k_propose) to the
 * CPU tests, which check its draws against the Poisson distribution.  Built
 * by tests/test_poisson_sampler.py into a temporary directory; not part of
 * the library.
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
