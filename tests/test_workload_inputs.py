"""The event generator reproduces the full-size workloads whose oracle seed
digests are committed (tests/golden/workload_hashes.json, made by
tests/golden/make_workload_hashes.py): same spacepoint columns, byte for
byte, for the 20 events of the 100k-spacepoint workload and the 64 events of
the uneven batch."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_workload_hashes as W  # noqa: E402


def test_generator_reproduces_the_golden_workloads():
    with open(os.path.join(HERE, "golden", "workload_hashes.json")) as f:
        golden = json.load(f)
    for name, events in W.workloads():
        assert len(events) == len(golden[name])
        for ev, g in zip(events, golden[name]):
            assert len(ev["global"]) == g["n_sp"]
            assert W.input_digest(ev) == g["input"], name
