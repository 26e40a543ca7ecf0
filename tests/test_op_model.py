"""The algorithmic-work model the bench's FP32 roofline uses
(profiles/op_model.json, generated by `python -m oracle.op_model`): its
counts are the oracle's for the bench events, and the operation counts are
bounded by the per-test constants of the reference's tests."""
import json
import os

import oracle
from oracle import op_model
from traccc_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _model():
    with open(os.path.join(ROOT, "profiles", "op_model.json")) as f:
        return json.load(f)


def test_model_covers_the_bench_events():
    m = _model()
    assert m["events"] == 20
    assert [e["seed"] for e in m["per_event"]] == list(range(20))
    total = 0
    for e in m["per_event"]:
        f = e["ops_doublet_tests"] + e["ops_triplet_tests"] + 27 * (e["n_mb"] + e["n_mt"])
        assert e["flop_seeding"] == f
        total += f
    assert m["flop_seeding_total"] == total


def test_model_matches_the_oracle():
    """Event seed 0 recounted now equals the committed entry."""
    got = op_model.event_counts(0)
    want = _model()["per_event"][0]
    assert got == want


def test_operation_counts_are_bounded_by_the_stage_costs():
    ev = synth.workload_event("trk1000", 2)
    _, st = oracle.seeding(ev, phi_mode=oracle.PHI_CR)
    pairs, win = st["n_pair_tests"], st["n_window_pairs"]
    assert 0 < win <= pairs
    # doublet test: 8 operations, 39 more inside the window
    assert st["ops_doublet_tests"] == 8 * pairs + 39 * win
    # triplet test: at least 11, at most 11 + 5 + 1 + 8 + 15
    t = st["n_triplet_tests"]
    assert 11 * t <= st["ops_triplet_tests"] <= 40 * t
    assert st["n_triplets"] <= t
