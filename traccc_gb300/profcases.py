"""Small fixed workloads for ncu captures of single kernels.

Each case sets itself up (and, for the learned filter, trains and
calibrates), then runs the launches to be captured inside the NVTX range
"profile", so that

    ncu --nvtx --nvtx-include "profile/" -k regex:<kernel> -c <n> ... \\
        python -m traccc_gb300.profcases <case>

captures exactly those launches however many came before.  Cases:

  plain4    plain seeding of 4 events of the 100k-spacepoint workload
  learned4  the same 4 events with the learned doublet filter (trained on 16
            events, calibrated on 4, top doublets pruned)
  train     one gradient step of the filter's network on the doublets of
            4 events (the tensor-core training kernel)
  batch64   one graph launch of the 64-event uneven batch
"""
from __future__ import annotations

import sys


def _events(n, seed0=0):
    from traccc_gb300 import synth
    return [synth.workload_event("pileup9k", seed0 + s) for s in range(n)]


def _range(torch, fn):
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("profile")
    fn()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()


def case_plain4():
    import torch

    from traccc_gb300 import seeding
    sps = [seeding.SpacepointCollection.from_numpy(e) for e in _events(4)]
    alg = seeding.TripletSeedingAlgorithm()
    outs = [seeding.SeedBuffer(alg.max_seeds(len(s))) for s in sps]
    for _ in range(2):
        alg.run_batch(sps, outs)
    _range(torch, lambda: alg.run_batch(sps, outs))
    assert alg.last_status() == seeding.OK


def _trained_model(alg):
    from traccc_gb300 import learned, synth
    model, rep = learned.build_filter(alg, synth.batch_events(16, 10), synth.batch_events(4, 20),
                                      epochs=3, target=0.995)
    return model, rep


def case_learned4():
    import torch

    from traccc_gb300 import seeding
    alg = seeding.TripletSeedingAlgorithm()
    model, rep = _trained_model(alg)
    sps = [seeding.SpacepointCollection.from_numpy(e) for e in _events(4)]
    outs = [seeding.SeedBuffer(alg.max_seeds(len(s))) for s in sps]
    alg.set_filter(model.struct())
    for _ in range(2):
        alg.run_batch(sps, outs)
    _range(torch, lambda: alg.run_batch(sps, outs))
    assert alg.last_status() == seeding.OK
    per, fb, _ = alg.filter_stats(4)
    print("pruned fraction per event:", ((per[:, 1] + per[:, 3]) / per[:, 2].clip(1)).round(3),
          "fallback:", fb.tolist(), "threshold:", model.threshold)


def case_train():
    import torch

    from traccc_gb300 import learned, seeding
    alg = seeding.TripletSeedingAlgorithm()
    data = learned.collect(alg, _events(4, 100), neg_keep=0.05)
    n = len(data.labels)
    P = torch.from_numpy(learned.init_params(0)).cuda()
    norm = torch.from_numpy(learned.feature_norm(data.features)).cuda()
    G = torch.empty_like(P)
    L = torch.empty(1, dtype=torch.float32, device="cuda")
    pw = float((n - data.labels.sum()) / data.labels.sum())
    for _ in range(2):
        seeding.mlp_grad(P, norm, data.features, data.labels, pw, G, L)
    _range(torch, lambda: seeding.mlp_grad(P, norm, data.features, data.labels, pw, G, L))
    print(f"{n} samples, loss {float(L.item()):.4f}")


def case_batch64():
    import torch

    from traccc_gb300 import seeding, synth
    sps = [seeding.SpacepointCollection.from_numpy(e) for e in synth.batch_events(64, 3)]
    alg = seeding.TripletSeedingAlgorithm()
    outs = [seeding.SeedBuffer(alg.max_seeds(len(s))) for s in sps]
    alg.graph_create(64, sum(len(s) for s in sps))
    for _ in range(2):
        alg.graph_launch(sps, outs)
    _range(torch, lambda: alg.graph_launch(sps, outs))
    assert alg.last_status() == seeding.OK


CASES = {"plain4": case_plain4, "learned4": case_learned4, "train": case_train,
         "batch64": case_batch64}


def main(argv):
    if len(argv) != 1 or argv[0] not in CASES:
        print(__doc__)
        return 2
    CASES[argv[0]]()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
