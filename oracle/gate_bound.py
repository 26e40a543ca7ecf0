"""Upper bound of any middle gate on the 100k-spacepoint workload.

TEST / ANALYSIS INFRASTRUCTURE (runs the oracle; not part of the product).

A gate that drops whole middles keeps exactly the plain seeds of the middles
it keeps (the reference selects seeds per middle from that middle's triplets
alone, core/src/seeding/seed_finding.cpp:76-116).  So the work such a gate
can save at a given seed recall is bounded by a perfect gate: drop the
middles with the fewest seeds per unit of work first, until the seeds lost
reach 0.5 %.  For each event this prints, for several per-middle work
measures counted by the oracle (doublets, doublet pairs, triplets), the share
of the work in middles without any seed and the share a perfect gate at
99.5 % seed recall saves.

    python -m oracle.gate_bound [seed ...]
"""
from __future__ import annotations

import sys

import numpy as np


def bound(seed: int, loss: float = 0.005):
    import oracle as O
    from traccc_gb300 import synth
    ev = synth.workload_event("pileup9k", seed)
    seeds, st, dump, trip = O.seeding_ex(ev, dump=True, triplets=True)
    n = len(ev["global"])
    mb = np.bincount(dump["middle"][dump["top"] == 0], minlength=n)
    mt = np.bincount(dump["middle"][dump["top"] == 1], minlength=n)
    nt = np.bincount(trip["middle"], minlength=n)
    ns = np.bincount(seeds["middle"], minlength=n)
    both = (mb > 0) & (mt > 0)
    out = {"seed": seed, "seeds": int(len(seeds)), "middles_both_roles": int(both.sum()),
           "middles_with_seeds": int((ns > 0).sum()),
           "middles_both_roles_no_seed": int((both & (ns == 0)).sum())}
    idx = np.nonzero(both)[0]
    for name, cost in (("doublets", mb + mt), ("doublet_pairs", mb * mt), ("triplets", nt)):
        c = cost[idx].astype(np.float64)
        tot = c.sum()
        order = np.argsort(ns[idx] / np.maximum(c, 1e-9), kind="stable")
        lost = np.cumsum(ns[idx][order])
        saved = np.cumsum(c[order])
        k = np.searchsorted(lost, loss * len(seeds), side="right")
        out[name] = {"no_seed_share": float(c[ns[idx] == 0].sum() / tot),
                     "perfect_gate_saves": float(saved[k - 1] / tot) if k > 0 else 0.0}
    return out


def main(argv):
    seeds = [int(a) for a in argv] or [0]
    for s in seeds:
        print(bound(s), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
