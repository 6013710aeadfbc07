/*
 * pcs_proposal.h -- construction of one ABC-PMC proposal, shared by the
 * batched device path (k_propose) and the plain per-proposal host path
 * (plain.cpp), so both draw the same parameters from the same streams.
 *
 * Follows the reference's proposal loop (src/gpu/detail/simulation_impl.inl
 * :256-347): weighted parent pick (wrand_idx_ :54-62), reflected Gaussian
 * displacement of every parameter (displace_ :64-79), components sorted by
 * m (:276-303), 10^log10c, Poisson particle counts per video (:307-317),
 * half depths, cumulative component probabilities with the last forced to 2
 * (:319-335), step sd = sqrt(2 m dt) (:337-340).
 */
#ifndef PCS_PROPOSAL_H
#define PCS_PROPOSAL_H

#include <math.h>
#include <stdint.h>

#include "pcs_common.h"
#include "pcs_kernels.h"

namespace pcs {

/* parameter layout: [m | s (lognormal) | log10c | az] */
struct Layout {
    uint32_t m, s, c, az, C, Z;
};

PCS_HD Layout pcs_layout(const JobPmcDev& pm)
{
    Layout L;
    L.C = pm.C;
    L.Z = pm.Z;
    L.m = 0;
    L.s = pm.C;
    L.c = (pm.model == PCS_DEV_MODEL_LOGNORMAL) ? 2 * pm.C : pm.C;
    L.az = L.c + pm.C;
    return L;
}

/* standard normal pair from 4 words (Box-Muller in double) */
PCS_HD void pcs_normal2(pcs_u4 r, double& n0, double& n1)
{
    const double u1 = 1.0 - pcs_u01_53(r.x, r.y); /* (0, 1] */
    const double u2 = pcs_u01_53(r.z, r.w);
    const double rad = sqrt(-2.0 * log(u1));
    double s, c;
#if defined(__CUDA_ARCH__)
    sincospi(2.0 * u2, &s, &c);
#else
    s = sin(2.0 * 3.14159265358979323846 * u2);
    c = cos(2.0 * 3.14159265358979323846 * u2);
#endif
    n0 = rad * s;
    n1 = rad * c;
}

/* displace_ reflection, with a bounded loop and a closed-form fold after it */
PCS_HD double pcs_reflect(double bis, double lo, double hi)
{
    for (int it = 0; it < 64 && (bis < lo || bis > hi); ++it) {
        if (bis < lo) bis += 2.0 * (lo - bis);
        if (bis > hi) bis -= 2.0 * (bis - hi);
    }
    if (bis < lo || bis > hi) {
        const double w = hi - lo;
        const double t = fmod(fabs(bis - lo), 2.0 * w);
        bis = lo + (t <= w ? t : 2.0 * w - t);
    }
    return bis;
}

/* Poisson(lambda): inversion below 12, PTRS transformed rejection above
 * (W. Hoermann, "The transformed rejection method for generating Poisson
 * random variables", Insurance: Mathematics and Economics 12, 1993).  The
 * constants depend on lambda only, so a proposal computes them once for all
 * of its videos.  logfact (nullable): log(k!) for k < logfact_n, built on
 * the host with lgamma, which the device then reads instead of evaluating
 * lgamma in FP64 (on this GPU a long chain of low-rate FP64 operations on
 * the proposal kernel's critical path); past the table, and on the host,
 * lgamma itself. */
struct PoissonSetup {
    double lam, explam, loglam, b, a, invalpha, vr, log_invalpha;
    const double* logfact;
    uint32_t logfact_n;
    float lamf, af, bf, vrf, loglamf, linvf; /* the same constants rounded to float (pcs_ptrs_filtered) */
};

PCS_HD PoissonSetup pcs_poisson_setup(double lam)
{
    PoissonSetup ps;
    ps.lam = lam;
    ps.explam = ps.loglam = ps.b = ps.a = ps.invalpha = ps.vr = ps.log_invalpha = 0.0;
    ps.logfact = nullptr;
    ps.logfact_n = 0u;
    ps.lamf = ps.af = ps.bf = ps.vrf = ps.loglamf = ps.linvf = 0.0f;
    if (!(lam > 0.0)) return ps;
    if (lam < 12.0) {
        ps.explam = exp(-lam);
        return ps;
    }
    const double slam = sqrt(lam);
    ps.loglam = log(lam);
    ps.b = 0.931 + 2.53 * slam;
    ps.a = -0.059 + 0.02483 * ps.b;
    ps.invalpha = 1.1239 + 1.1328 / (ps.b - 3.4);
    ps.vr = 0.9277 - 3.6224 / (ps.b - 2.0);
    ps.log_invalpha = log(ps.invalpha);
    ps.lamf = (float)lam;
    ps.af = (float)ps.a;
    ps.bf = (float)ps.b;
    ps.vrf = (float)ps.vr;
    ps.loglamf = (float)ps.loglam;
    ps.linvf = (float)ps.log_invalpha;
    return ps;
}

/* Scale of the FP32 filter's error margins below: 1 in the library; the
 * CPU tests build a copy with a small scale to show that their comparison
 * with the FP64 iteration detects margins that are too narrow. */
#ifndef PCS_PTRS_MARGIN
#define PCS_PTRS_MARGIN 1.0f
#endif

/* One PTRS iteration in FP64 on the draw r: 1 accept (*k), 0 reject. */
PCS_HD int pcs_ptrs_exact(const PoissonSetup& ps, const pcs_u4& r, uint32_t* k)
{
    const double lam = ps.lam, a = ps.a, b = ps.b;
    const double U = pcs_u01_53(r.x, r.y) - 0.5;
    const double V = pcs_u01_53(r.z, r.w);
    const double us = 0.5 - fabs(U);
    const double kf = floor((2.0 * a / us + b) * U + lam + 0.43);
    if (us >= 0.07 && V <= ps.vr) {
        *k = (uint32_t)kf;
        return 1;
    }
    if (kf < 0.0 || (us < 0.013 && V > us)) return 0;
    const double lf = (ps.logfact && kf < (double)ps.logfact_n) ? ps.logfact[(uint32_t)kf] : lgamma(kf + 1.0);
    if (log(V) + ps.log_invalpha - log(a / (us * us) + b) <= -lam + kf * ps.loglam - lf) {
        *k = (uint32_t)kf;
        return 1;
    }
    return 0;
}

/* The same iteration decided in FP32 where that is certain: every test of
 * pcs_ptrs_exact evaluated on the top 24 bits of its uniforms (U and V then
 * differ from the FP64 ones by less than u = 2^-24) with a bound on the
 * FP32 error, derived term by term below (u per rounding, the inputs'
 * truncation, 1 ulp per logf); a test inside its bound, a small us, a V near
 * 0 or a k past the log-factorial table leaves the iteration to
 * pcs_ptrs_exact (-1).  Where it decides, its decision and k are the FP64
 * iteration's: the counts do not change, most of the FP64 work does.
 * On this GPU FP64 runs at a small fraction of the FP32 rate. */
PCS_HD int pcs_ptrs_filtered(const PoissonSetup& ps, const pcs_u4& r, uint32_t* k)
{
    const float u = 5.9604645e-8f; /* 2^-24 */
    if (!(ps.lamf <= 4.0e6f)) return -1; /* k exact in float with room */
    const float Uf = (float)(r.x >> 8) * u - 0.5f; /* U - Uf in [0, u) */
    const float Vf = (float)(r.z >> 8) * u;        /* V - Vf in [0, u) */
    const float usf = 0.5f - fabsf(Uf);            /* |us - usf| < u */
    const float m = 4.0e-7f; /* input truncation plus the constants' rounding to float */
    /* us >= 0.07 and V <= vr */
    const int A = usf > 0.07f + m ? 1 : (usf < 0.07f - m ? 0 : -1);
    const int Bv = Vf < ps.vrf - m ? 1 : (Vf > ps.vrf + m ? 0 : -1);
    const bool fast_no = A == 0 || Bv == 0;
    if (!fast_no && (A < 0 || Bv < 0)) return -1;
    /* us < 0.013 and V > us */
    const int C1 = usf < 0.013f - m ? 1 : (usf > 0.013f + m ? 0 : -1);
    const int C2 = Vf > usf + m ? 1 : (Vf < usf - m ? 0 : -1);
    if (fast_no && C1 == 1 && C2 == 1) return 0;
    /* k = floor((2a/us + b) U + lam + 0.43).  With ru = 1.01 u / usf above
     * us's relative error, 2a/us is within (2u + ru)|t1|, and x within
     * (u + ru/2)|t1| + u (0.5|b| + 1.5|t2| + 2|t3| + 2 lam + |x| + 0.43);
     * the margin doubles that (and covers the FP64 evaluation's own
     * rounding) */
    if (usf < 0.005f) return -1;
    const float ru = 1.01f * u / usf;
    const float t1 = 2.0f * ps.af / usf;
    const float t2 = t1 + ps.bf;
    const float t3 = t2 * Uf;
    const float xf = (t3 + ps.lamf) + 0.43f;
    const float mx = PCS_PTRS_MARGIN * ((4.0f * u + 1.2f * ru) * fabsf(t1) +
                                        u * (4.0f * (fabsf(ps.bf) + fabsf(t2) + fabsf(t3)) + 4.0f * ps.lamf +
                                             4.0f * fabsf(xf) + 8.0f));
    const float n = floorf(xf);
    if (!(xf - n > mx && (n + 1.0f) - xf > mx)) return -1;
    if (!fast_no) { /* A and Bv both 1 */
        *k = (uint32_t)n;
        return 1;
    }
    if (n < 0.0f) return 0;
    if (C1 < 0 || C2 < 0) {
        if (!(C1 == 0 || C2 == 0)) return -1;
    }
    /* log(V) + log_invalpha - log(a/us^2 + b) <= -lam + k loglam - log(k!) */
    if (!ps.logfact || !(n < (float)ps.logfact_n) || Vf < 1.0e-6f) return -1;
    const float lf = (float)ps.logfact[(uint32_t)n];
    const float lV = logf(Vf);
    const float l2 = logf(ps.af / (usf * usf) + ps.bf);
    const float lhs = (lV + ps.linvf) - l2;
    const float kl = n * ps.loglamf;
    const float rhs = (kl - ps.lamf) - lf;
    const float d = lhs - rhs;
    /* error of lhs below u/V (V's truncation) + 3u|log V| + 2u|log_invalpha|
     * + (4u + 2ru) (a/us^2 + b is positive, to that relative error) + 2u|l2|
     * + u|lhs|; of rhs below 2u lam + 3u|k loglam| + u|log k!| + u|rhs|; of
     * d, u|d| more.  The margin is at least that sum with room for its own
     * rounding. */
    const float ms = PCS_PTRS_MARGIN * 2.4f * ru + PCS_PTRS_MARGIN * u * (1.0f / Vf + 4.0f * fabsf(lV) + 3.0f * fabsf(ps.linvf) + 4.0f * fabsf(l2) +
                                     2.0f * fabsf(lhs) + 16.0f + 4.0f * ps.lamf + 4.0f * fabsf(kl) +
                                     2.0f * fabsf(lf) + 2.0f * fabsf(rhs) + 2.0f * fabsf(d));
    if (d < -ms) {
        *k = (uint32_t)n;
        return 1;
    }
    if (d > ms) return 0;
    return -1;
}

template <bool FILTER = true>
PCS_HD uint32_t pcs_poisson_draw(const PoissonSetup& ps, uint32_t video, uint32_t slot, uint32_t gt, uint32_t k0,
                                 uint32_t k1)
{
    const double lam = ps.lam;
    if (!(lam > 0.0)) return 0u;
    if (lam < 12.0) {
        const pcs_u4 r = pcs_draw(video, pcs_ctr_tag(PCS_STREAM_POISSON, 0u), slot, gt, k0, k1);
        const double u = pcs_u01_53(r.x, r.y);
        double p = ps.explam, F = p;
        uint32_t k = 0;
        while (u > F && k < 1000u) {
            ++k;
            p *= lam / k;
            F += p;
        }
        return k;
    }
    for (uint32_t it = 0; it < 256u; ++it) {
        const pcs_u4 r = pcs_draw(video, pcs_ctr_tag(PCS_STREAM_POISSON, 1u + it), slot, gt, k0, k1);
        uint32_t kk = 0u;
        int dec = FILTER ? pcs_ptrs_filtered(ps, r, &kk) : -1;
        if (dec < 0) dec = pcs_ptrs_exact(ps, r, &kk);
        if (dec > 0) return kk;
    }
    return (uint32_t)floor(lam + 0.5);
}

PCS_HD uint32_t pcs_poisson(double lam, uint32_t video, uint32_t slot, uint32_t gt, uint32_t k0, uint32_t k1)
{
    return pcs_poisson_draw(pcs_poisson_setup(lam), video, slot, gt, k0, k1);
}

/* first cumulative weight >= u (std::lower_bound), clamped to N - 1 */
PCS_HD uint32_t pcs_pick(const double* wcum, uint32_t N, double u)
{
    uint32_t lo = 0, hi = N;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (wcum[mid] < u)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo < N ? lo : N - 1;
}

/* Parameter p of a perturbed proposal: parent value tp[p] displaced by the
 * perturbation factor applied to the normals nrm[0..p] (Cholesky) or nrm[p]
 * (diagonal), reflected into the prior box; fixed parameters stay at lo. */
PCS_HD double pcs_perturb_one(const JobPmcDev& pm, const double* tp, const double* factor, const double* nrm,
                              uint32_t p)
{
    const uint32_t P = pm.P;
    if (pm.fixed[p]) return pm.lo[p];
    double delta;
    if (pm.perturbation == 1u) {
        delta = 0.0;
        for (uint32_t i = 0; i <= p; ++i)
            if (!pm.fixed[i]) delta += factor[p * P + i] * nrm[i];
    } else {
        delta = factor[p * P + p] * nrm[p];
    }
    return pcs_reflect(tp[p] + delta, pm.lo[p], pm.hi[p]);
}

/* Sort the components by the first parameter group (label switching). */
PCS_HD void pcs_sort_components(const JobPmcDev& pm, double* th)
{
    const Layout L = pcs_layout(pm);
    for (uint32_t i = 1; i < L.C; ++i) {
        for (uint32_t x = i; x > 0 && th[L.m + x] < th[L.m + x - 1]; --x) {
            double t;
            t = th[L.m + x];
            th[L.m + x] = th[L.m + x - 1];
            th[L.m + x - 1] = t;
            t = th[L.c + x];
            th[L.c + x] = th[L.c + x - 1];
            th[L.c + x - 1] = t;
            if (pm.model == PCS_DEV_MODEL_LOGNORMAL) {
                t = th[L.s + x];
                th[L.s + x] = th[L.s + x - 1];
                th[L.s + x - 1] = t;
            }
            if (L.Z > 1u) {
                t = th[L.az + x];
                th[L.az + x] = th[L.az + x - 1];
                th[L.az + x - 1] = t;
            }
        }
    }
}

/* Parameters of trial `trial` of population slot `slot` in generation `gen`.
 * Generation 0 (the prior pass) simulates the slot's own parameters. */
PCS_HD void pcs_build_theta(const JobPmcDev& pm, const double* theta_pop, const double* wcum,
                            const double* factor, uint32_t slot, uint32_t trial, uint32_t gen,
                            uint32_t k0, uint32_t k1, double* th)
{
    const uint32_t P = pm.P, N = pm.N;
    const uint32_t gt = pcs_ctr_gen_trial(gen, trial);
    if (gen == 0u) {
        for (uint32_t p = 0; p < P; ++p) th[p] = theta_pop[(uint64_t)slot * P + p];
        return;
    }
    const pcs_u4 r = pcs_draw(0u, pcs_ctr_tag(PCS_STREAM_PICK, 0u), slot, gt, k0, k1);
    const uint32_t parent = pcs_pick(wcum, N, pcs_u01_53(r.x, r.y));
    const double* tp = theta_pop + (uint64_t)parent * P;
    double nrm[PCS_MAX_P];
    for (uint32_t p = 0; p < P; p += 2) {
        const pcs_u4 rr = pcs_draw(p >> 1, pcs_ctr_tag(PCS_STREAM_PERTURB, 0u), slot, gt, k0, k1);
        double n0, n1;
        pcs_normal2(rr, n0, n1);
        nrm[p] = n0;
        if (p + 1 < P) nrm[p + 1] = n1;
    }
    for (uint32_t p = 0; p < P; ++p) th[p] = pcs_perturb_one(pm, tp, factor, nrm, p);
    pcs_sort_components(pm, th);
}

/* Per-component forward-model arguments: 10^log10c and the step sd's scale
 * and shape (lognormal) or the fixed step sd. */
struct CompArgs {
    double powc;
    float sd_scale, sd_shape;
};

PCS_HD CompArgs pcs_comp_args(const JobPmcDev& pm, const double* th, uint32_t i)
{
    const Layout L = pcs_layout(pm);
    CompArgs ca;
    ca.powc = exp10(th[L.c + i]); /* 10^x: one exponential, where pow(10, x) adds a logarithm */
    if (pm.model == PCS_DEV_MODEL_LOGNORMAL) {
        /* lognormal diameter (nm), mean mu and sd s: sigma_ln^2 = ln(1 + s^2 / mu^2) */
        const double mu = th[L.m + i], sdv = th[L.s + i];
        const double sl2 = log1p((sdv * sdv) / (mu * mu));
        const double mul = log(mu) - 0.5 * sl2;
        ca.sd_scale = (float)(pm.sd_const * exp(-0.5 * mul));
        ca.sd_shape = (float)(-0.5 * sqrt(sl2));
    } else {
        ca.sd_scale = (float)sqrt(2.0 * th[L.m + i] * pm.delta_t);
        ca.sd_shape = 0.0f;
    }
    return ca;
}

/* Assembles a proposal's forward-model arguments from its components';
 * returns the Poisson mean per video. */
PCS_HD double pcs_assemble_args(const JobPmcDev& pm, const double* th, const CompArgs* ca, uint32_t gen, PropDev& pd)
{
    const Layout L = pcs_layout(pm);
    double csum = 0.0;
    for (uint32_t i = 0; i < L.C; ++i) csum += ca[i].powc;
    for (uint32_t i = 0; i < PCS_MAX_C; ++i) {
        pd.pre_comp_prob[i] = 2.0f;
        pd.sd_scale[i] = 0.0f;
        pd.sd_shape[i] = 0.0f;
        pd.half_az[i] = 0.0f;
    }
    double acc = 0.0;
    for (uint32_t i = 0; i < L.C; ++i) {
        acc += ca[i].powc / csum;
        pd.pre_comp_prob[i] = (float)acc;
        pd.sd_scale[i] = ca[i].sd_scale;
        pd.sd_shape[i] = ca[i].sd_shape;
    }
    pd.pre_comp_prob[L.C - 1] = 2.0f;
    for (uint32_t z = 0; z < L.Z; ++z) {
        const float azf = (float)th[L.az + z];
        pd.half_az[z] = (gen == 0u && pm.quirk_full_az) ? azf : 0.5f * azf;
    }
    return csum * pm.volume_factor;
}

/* Forward-model arguments of a proposal; returns the Poisson mean per video. */
PCS_HD double pcs_build_args(const JobPmcDev& pm, const double* th, uint32_t gen, PropDev& pd)
{
    CompArgs ca[PCS_MAX_C];
    for (uint32_t i = 0; i < pm.C; ++i) ca[i] = pcs_comp_args(pm, th, i);
    return pcs_assemble_args(pm, th, ca, gen, pd);
}

/* Poisson counts per video and their prefix; returns total particles (and
 * particle-steps through *steps). */
PCS_HD uint64_t pcs_draw_counts(double lambda, uint32_t V, const uint32_t* frames, uint32_t slot,
                                uint32_t trial, uint32_t gen, uint32_t k0, uint32_t k1, uint32_t* cnt,
                                uint32_t* pre, uint64_t* steps)
{
    const uint32_t gt = pcs_ctr_gen_trial(gen, trial);
    const PoissonSetup ps = pcs_poisson_setup(lambda);
    uint64_t total = 0, st = 0;
    pre[0] = 0u;
    for (uint32_t v = 0; v < V; ++v) {
        const uint32_t c = pcs_poisson_draw(ps, v, slot, gt, k0, k1);
        cnt[v] = c;
        total += c;
        st += (uint64_t)c * frames[v];
        pre[v + 1] = (uint32_t)(total < 0xFFFFFFFFull ? total : 0xFFFFFFFFull);
    }
    if (steps) *steps = st;
    return total;
}

} // namespace pcs

#endif
