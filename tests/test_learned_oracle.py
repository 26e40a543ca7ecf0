"""The CPU restatement of the learned doublet filter (oracle side).

* bf16 rounding: the C oracle and the numpy reference agree bit for bit
  (nearest even, NaN kept quiet).
* The numpy reference's backward pass is plain backpropagation: without
  rounding it matches central finite differences of its own loss.
* The C oracle's network (sequential fp32 sums) agrees with the numpy
  reference (float64 sums) to fp32 rounding.
* Seeding with the filter: keeping everything reproduces plain seeding, the
  dump holds exactly the scored doublets with the documented features, and
  pruning only removes work (recall and the pruned fraction move the right
  way with the threshold).
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from oracle import mlp_reference as R
from traccc_gb300 import synth


def _model(seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, R.N_PARAMS).astype(np.float32)
    norm = np.concatenate([rng.normal(0, 50, 8), rng.uniform(0.01, 0.1, 8)]).astype(np.float32)
    return p, norm


def _model_dict(p, norm, edges=(52.0, 94.0, 144.0, 216.0)):
    w1, b1, w2, b2, w3, b3 = R.unpack(p)
    return dict(mu=norm[:8], isd=norm[8:], w1=w1, b1=b1, w2=w2, b2=b2, w3=w3, b3=b3,
                edges=np.asarray(edges, np.float32))


def test_bf16_rounding_matches():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(0, 1, 2000), rng.normal(0, 1e-30, 50), rng.normal(0, 1e30, 50),
                        [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, np.inf, -np.inf]]).astype(np.float32)
    ref = R.bf16(x)
    L = O.lib()
    got = np.array([L.or_bf16_round(float(v)) for v in x], np.float32)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    # ties go to even
    assert R.bf16(np.float32(1.0 + 2 ** -8)) == np.float32(1.0)
    assert R.bf16(np.float32(1.0 + 3 * 2 ** -8)) == np.float32(1.0 + 2 ** -6)
    assert np.isnan(R.bf16(np.float32(np.nan)))


def test_reference_backward_is_backpropagation():
    rng = np.random.default_rng(2)
    p = rng.normal(0, 0.3, R.N_PARAMS)
    norm = np.concatenate([rng.normal(0, 1, 8), rng.uniform(0.5, 2, 8)])
    x = rng.normal(0, 1, (48, 8))
    y = (rng.random(48) < 0.3).astype(float)
    _, g = R.loss_and_grad(p, norm, x, y, 3.0, exact=True)
    eps = 1e-6
    idx = rng.choice(R.N_PARAMS, 120, replace=False)
    for i in idx:
        q = p.copy()
        q[i] += eps
        a, _ = R.loss_and_grad(q, norm, x, y, 3.0, exact=True)
        q[i] -= 2 * eps
        b, _ = R.loss_and_grad(q, norm, x, y, 3.0, exact=True)
        assert abs((a - b) / (2 * eps) - g[i]) < 1e-7 * max(1.0, abs(g[i]))
    # with the GPU's bf16 operands the gradient stays close to the exact one
    _, gr = R.loss_and_grad(p, norm, x, y, 3.0)
    assert np.linalg.norm(gr - g) < 0.05 * np.linalg.norm(g)


def test_c_network_matches_numpy_reference():
    p, norm = _model(3)
    f = O.doublet_filter(_model_dict(p, norm), 0.0)
    rng = np.random.default_rng(4)
    feat = np.stack([rng.uniform(30, 200, 500), rng.uniform(-1000, 1000, 500),
                     rng.uniform(-150, 150, 500), rng.uniform(-300, 300, 500),
                     rng.normal(0, 2, 500), rng.normal(0, 0.05, 500),
                     rng.normal(0, 100, 500), rng.integers(0, 25, 500)], 1).astype(np.float32)
    ref, _ = R.forward(p, norm, feat)
    L = O.lib()
    got = np.array([L.or_mlp_logit(C.byref(f), row.ctypes.data_as(C.POINTER(C.c_float)))
                    for row in feat], np.float32)
    # the two differ only in the fp32 rounding of the sums; a hidden value
    # that lands on the other side of a bf16 rounding boundary moves the
    # logit by one bf16 step of that value
    d = np.abs(got - ref)
    assert np.median(d) <= 1e-5 * (1 + np.median(np.abs(ref)))
    assert d.max() <= 0.05 * (1 + np.abs(ref).max())


@pytest.fixture(scope="module")
def trk1000_event():
    return synth.workload_event("trk1000", 3)


def test_keep_all_is_plain_seeding(trk1000_event):
    p, norm = _model(5)
    f = O.doublet_filter(_model_dict(p, norm), (-np.inf, -np.inf))
    seeds, st, d = O.seeding_ex(trk1000_event, filt=f, dump=True)
    plain, st0 = O.seeding(trk1000_event)
    assert np.array_equal(seeds, plain)
    assert st["n_pruned_mb"] == 0 and st["n_pruned_mt"] == 0
    assert len(d) == st["n_scored_mb"] + st["n_scored_mt"] > 0
    # only middles with both roles are scored
    assert 0 < st["n_scored_mb"] <= st0["n_mb"] and 0 < st["n_scored_mt"] <= st0["n_mt"]
    # nothing kept: no seeds
    f2 = O.doublet_filter(_model_dict(p, norm), (np.inf, np.inf))
    none, st2, _ = O.seeding_ex(trk1000_event, filt=f2)
    assert len(none) == 0 and st2["n_pruned_mb"] == st2["n_scored_mb"]


def test_dump_features(trk1000_event):
    p, norm = _model(6)
    edges = (52.0, 94.0, 144.0, 216.0)
    f = O.doublet_filter(_model_dict(p, norm, edges), (-np.inf, -np.inf))
    _, _, d = O.seeding_ex(trk1000_event, filt=f, dump=True)
    g = trk1000_event["global"].astype(np.float32)
    r = np.sqrt(g[:, 0] * g[:, 0] + g[:, 1] * g[:, 1]).astype(np.float32)
    m, o = d["middle"], d["other"]
    F = d["feat"]
    assert np.array_equal(F[:, 0], r[m])
    assert np.array_equal(F[:, 1], g[m, 2])
    assert np.array_equal(F[:, 2], (r[o] - r[m]).astype(np.float32))
    assert np.array_equal(F[:, 3], (g[o, 2] - g[m, 2]).astype(np.float32))
    f32 = np.float32
    cphi, sphi = (g[m, 0] / r[m]).astype(f32), (g[m, 1] / r[m]).astype(f32)
    dx, dy = (g[o, 0] - g[m, 0]).astype(f32), (g[o, 1] - g[m, 1]).astype(f32)
    y = ((dy * cphi).astype(f32) - (dx * sphi).astype(f32)).astype(f32)
    idr2 = (f32(1) / ((dx * dx).astype(f32) + (dy * dy).astype(f32)).astype(f32)).astype(f32)
    assert np.array_equal(F[:, 5], (y * np.sqrt(idr2).astype(f32)).astype(f32))
    assert np.all(np.abs(F[:, 5]) <= 1.0)
    top = d["top"] == 1
    assert np.all(F[top, 2] > 0) and np.all(F[~top, 2] < 0)
    # cot(theta) points from bottom to top: the sign of dz / dr
    assert np.all((np.sign(F[:, 4]) == np.sign(F[:, 3] * np.sign(F[:, 2]))) | (F[:, 3] == 0))
    band = lambda v: np.searchsorted(np.asarray(edges, np.float32), v, side="right")
    assert np.array_equal(F[:, 7], (band(r[m]) * 5 + band(r[o])).astype(np.float32))
    # the logits are the network's
    ref, _ = R.forward(p, norm, F)
    assert np.median(np.abs(ref - d["logit"])) <= 1e-5 * (1 + np.median(np.abs(ref)))


def test_pruning_is_monotone(trk1000_event):
    p, norm = _model(7)
    _, _, d = O.seeding_ex(trk1000_event, filt=O.doublet_filter(_model_dict(p, norm), -np.inf),
                           dump=True)
    plain, _ = O.seeding(trk1000_event)
    pk = set(zip(plain["bottom"], plain["middle"], plain["top"]))
    fracs, recalls = [], []
    for q in (0.1, 0.3, 0.5):
        th = np.quantile(d["logit"], q)
        s, st, _ = O.seeding_ex(trk1000_event, filt=O.doublet_filter(_model_dict(p, norm), th))
        fracs.append((st["n_pruned_mb"] + st["n_pruned_mt"]) /
                     (st["n_scored_mb"] + st["n_scored_mt"]))
        recalls.append(len(pk & set(zip(s["bottom"], s["middle"], s["top"]))) / len(pk))
    assert fracs[0] < fracs[1] < fracs[2]
    assert recalls[0] >= recalls[1] >= recalls[2]


def test_middle_gate_keeps_exactly_the_plain_seeds_of_kept_middles(trk1000_event):
    """Gating whole middles (prune_top = FILTER_GATE_MIDDLE): a middle is
    seeded, unpruned, iff one of its middle-top doublets reaches the
    threshold; the reference selects seeds per middle from that middle's
    triplets alone (core/src/seeding/seed_finding.cpp:76-116), so the output
    is the plain seeds of the kept middles -- a subset by construction --
    for any network and threshold."""
    p, norm = _model(8)
    _, _, d = O.seeding_ex(trk1000_event, filt=O.doublet_filter(_model_dict(p, norm), -np.inf),
                           dump=True)
    plain, _ = O.seeding(trk1000_event)
    tops = d[d["top"] == 1]
    for q in (0.2, 0.5, 0.8):
        th = float(np.quantile(tops["logit"], q))
        f = O.doublet_filter(_model_dict(p, norm), (-np.inf, th), prune_bottom=O.FILTER_KEEP,
                             prune_top=O.FILTER_GATE_MIDDLE)
        s, st, _ = O.seeding_ex(trk1000_event, filt=f)
        best = {}
        for m, lg in zip(tops["middle"].tolist(), tops["logit"].tolist()):
            best[m] = max(best.get(m, -np.inf), lg)
        kept = np.array([best.get(m, -np.inf) >= th for m in plain["middle"].tolist()])
        assert np.array_equal(s, plain[kept])
        assert 0 < len(s) < len(plain)
        gated = [m for m, b in best.items() if b < th]
        n_gated_tops = int(np.isin(tops["middle"], gated).sum())
        assert st["n_pruned_mt"] == n_gated_tops and st["n_pruned_mb"] == 0


def test_middle_gate_size_limit_keeps_large_middles(trk1000_event):
    """With gate_max_tops = K the gate scores only middles with at most K
    middle-top doublets; larger middles keep all their plain seeds even when
    no doublet reaches the threshold (here: a threshold nothing reaches)."""
    p, norm = _model(9)
    _, _, d = O.seeding_ex(trk1000_event, filt=O.doublet_filter(_model_dict(p, norm), -np.inf),
                           dump=True)
    plain, _ = O.seeding(trk1000_event)
    tops = d[d["top"] == 1]
    n_mt = np.bincount(tops["middle"], minlength=len(trk1000_event["global"]))
    K = 8
    f = O.doublet_filter(_model_dict(p, norm), (-np.inf, np.inf), prune_bottom=O.FILTER_KEEP,
                         prune_top=O.FILTER_GATE_MIDDLE, gate_max_tops=K)
    s, st, _ = O.seeding_ex(trk1000_event, filt=f)
    kept = n_mt[plain["middle"]] > K
    assert np.array_equal(s, plain[kept])
    assert 0 < len(s) < len(plain)
    assert st["n_pruned_mt"] == int(n_mt[(n_mt > 0) & (n_mt <= K)][
        np.isin(np.nonzero((n_mt > 0) & (n_mt <= K))[0], np.unique(tops["middle"]))].sum())
