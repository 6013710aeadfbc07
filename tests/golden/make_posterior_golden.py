"""Generates posterior_cases.npz: the CPU oracle's ABC-PMC posteriors
(oracle/abc_oracle.c, an independent restatement of the reference's
algorithm with its own random numbers) on the problems of posterior_cases.py,
ten seeds each.  Runs on the CPU (minutes on 8 cores):

    python tests/golden/make_posterior_golden.py [--out PATH] [--cases NAME ...]

Stored per case NAME: NAME__hist (the observed R x B histogram),
NAME__summaries [seeds, P, 3] (weighted mean, 5% and 95% quantiles per
parameter), NAME__generations [seeds] (generations committed after the
prior pass), NAME__converged [seeds] (1 if the trial cap ended the run) and
NAME__trials [seeds].
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import posterior_cases as PC  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "posterior_cases.npz"))
    ap.add_argument("--cases", nargs="*", default=list(PC.CASES))
    ap.add_argument("--seeds", type=int, default=PC.SEEDS)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args()
    import oracle as O
    O.build()
    out = {}
    if os.path.exists(args.out):  # keep the cases not regenerated
        out.update(dict(np.load(args.out)))
    for name in args.cases:
        case = PC.CASES[name]
        hist = PC.observed_hist(O, case)
        sat = np.cumsum(np.cumsum(hist.astype(np.uint64), 0), 1).astype(np.uint32)
        fr = np.full(case["V"], case["F"], np.uint32)
        pb = PC.oracle_problem(case)
        summ, gens, conv, trials = [], [], [], []
        for k in range(args.seeds):
            t0 = time.time()
            th, w, tr, g, cv = O.abc_pmc(pb, fr, sat, 1001 + k, args.threads, full=True)
            summ.append(PC.summaries(th, w))
            gens.append(g)
            conv.append(int(cv))
            trials.append(tr)
            print(f"{name} seed {k}: {time.time() - t0:.1f} s, {tr} trials, {g} generations, converged {cv}, "
                  f"means {np.round(summ[-1][:, 0], 4)}", flush=True)
        out[f"{name}__hist"] = hist
        out[f"{name}__summaries"] = np.array(summ)
        out[f"{name}__generations"] = np.array(gens, np.int64)
        out[f"{name}__converged"] = np.array(conv, np.int64)
        out[f"{name}__trials"] = np.array(trials, np.int64)
        s = np.array(summ)
        rng = PC.prior_ranges(case)
        rng[rng == 0] = 1.0
        print(name, "tracks", int(hist.sum()), "\nseed-averaged [mean, q05, q95]:\n", np.round(s.mean(0), 4),
              "\nseed sd / prior range:\n", np.round(s.std(0, ddof=1) / rng[:, None], 4),
              "\ntruth", PC.truth_vector(case), flush=True)
    np.savez_compressed(args.out, **out)
    print("->", args.out)


if __name__ == "__main__":
    main()
