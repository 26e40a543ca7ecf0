"""The GPU seeds of both full-size workloads -- the 20 events of the
100k-spacepoint bench step through the batched launch, the 64-event uneven
batch through the captured graph -- against the oracle's, through the
committed per-event digests (tests/golden/workload_hashes.json): seed count
and SHA-256 of the seed bytes, 2.9 M seeds in all."""
import json
import os
import sys

import pytest

from traccc_gb300 import seeding

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_workload_hashes as W  # noqa: E402


def test_full_workloads_match_the_oracle_digests():
    import torch
    with open(os.path.join(HERE, "golden", "workload_hashes.json")) as f:
        golden = json.load(f)
    for name, events in W.workloads():
        for ev, g in zip(events, golden[name]):
            assert W.input_digest(ev) == g["input"], "the generator made other events here"
        sps = [seeding.SpacepointCollection.from_numpy(e) for e in events]
        alg = seeding.TripletSeedingAlgorithm()
        if name == "uneven64":
            alg.graph_create(len(sps), sum(len(s) for s in sps))
            outs = alg.graph_launch(sps)
        else:
            outs = alg.run_batch(sps)
        torch.cuda.synchronize()
        assert alg.last_status() == seeding.OK
        for e, (o, g) in enumerate(zip(outs, golden[name])):
            got = o.to_numpy()
            assert len(got) == g["n_seeds"], (name, e)
            assert W.seed_digest(got) == g["seeds"], (name, e)
