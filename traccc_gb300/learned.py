"""Learned doublet filter: data, training and calibration on the GPU.

The filter (seedgb_doublet_filter, include/seedgb.h) scores every doublet of
a middle spacepoint that has both roles with an MLP 8 -> 32 -> 32 -> 1.  By
default it gates whole middles: a middle none of whose middle-top doublets
reaches the threshold yields no seed, every other middle is seeded with all
its doublets and the plain cuts.  The reference selects seeds per middle
from that middle's triplets alone, so the output is a subset of the plain
seeds by construction.  (The older mode, dropping single doublets below a
per-role threshold, changes the surviving middles' seed weights and ranks
and so can emit seeds outside the plain set.)  Everything here runs through
the seeding library's own kernels:

* ``collect``   -- plain seeding of training events with the doublet dump on;
                   label = the doublet appears in an accepted seed (middle and
                   bottom of a seed for middle-bottom doublets, middle and top
                   for middle-top ones); all positives and a random share of
                   the negatives are kept on the device.
* ``train``     -- mini-batch Adam on the weighted logistic loss with the
                   library's forward/backward kernels (bf16 operands, fp32
                   accumulate on the tensor cores, fp32 master weights).
* ``calibrate`` -- middle gate: the highest threshold on a middle's best
                   middle-top logit whose seed recall against plain seeding
                   is >= the target over the held-out events and >= a floor on
                   every one of them, read off exactly from one scored plain
                   run (the gated seeds are the plain seeds of the kept
                   middles), then confirmed by a gated run; doublet pruning:
                   per-role thresholds at a common quantile of the positive
                   doublets' logits, checked by seeding runs.  The
                   pruned-fraction band is the range seen on those events,
                   widened by a margin.

Torch tensors serve as device buffers and for bookkeeping (keys, sorting,
sampling); the network's arithmetic is in the library.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import seeding, synth

N_IN, N_H = 8, 32
LAYER_RADII = synth.LAYER_RADII


def band_edges(layer_radii=LAYER_RADII):
    """Radial band edges halfway between consecutive layers."""
    r = np.asarray(layer_radii, np.float32)
    return ((r[1:] + r[:-1]) * np.float32(0.5)).astype(np.float32)


@dataclasses.dataclass
class FilterModel:
    params: np.ndarray            # fp32 [1377]: w1[8][32], b1, w2[32][32], b2, w3, b3
    norm: np.ndarray              # fp32 [16]: mu[8], isd[8]
    edges: np.ndarray             # fp32 radial band edges
    threshold: tuple = (-np.inf, -np.inf)
    band: tuple = (0.0, 1.0)
    # seeding.FILTER_* modes per role.  Default: gate middles on their
    # middle-top doublets (whose features come with the lin_circles the
    # seeder computes anyway); middle-bottom doublets are not scored
    prune_bottom: int = seeding.FILTER_KEEP
    prune_top: int = seeding.FILTER_GATE_MIDDLE
    # per-event-size classes: [(max spacepoints, (thr bottom, thr top),
    # (band lo, band hi)), ...] ascending, or None
    classes: list = None
    # middle gate: middles with more middle-top doublets are kept unscored
    # (0: no limit); nearly every middle without a seed is small
    gate_max_tops: int = 32

    def struct(self, threshold=None, band=None, prune=None) -> seeding.DoubletFilter:
        """The C struct, optionally with other thresholds / band / pruning
        (an explicit threshold or band replaces the size classes)."""
        p = np.asarray(self.params, np.float32)
        f = seeding.DoubletFilter()
        f.mu[:] = self.norm[:8].tolist()
        f.isd[:] = self.norm[8:].tolist()
        f.w1[:] = p[0:256].tolist()
        f.b1[:] = p[256:288].tolist()
        f.w2[:] = p[288:1312].tolist()
        f.b2[:] = p[1312:1344].tolist()
        f.w3[:] = p[1344:1376].tolist()
        f.b3 = float(p[1376])
        th = self.threshold if threshold is None else threshold
        f.threshold[0] = float(np.float32(th[0]))
        f.threshold[1] = float(np.float32(th[1]))
        e = np.asarray(self.edges, np.float32)
        f.n_edges = len(e)
        f.edges[: len(e)] = e.tolist()
        pb, pt = (self.prune_bottom, self.prune_top) if prune is None else prune
        f.prune_bottom = int(pb)
        f.prune_top = int(pt)
        b = self.band if band is None else band
        f.band[0] = float(b[0])
        f.band[1] = float(b[1])
        f.gate_max_tops = int(self.gate_max_tops)
        if self.classes and threshold is None and band is None:
            f.n_size_classes = len(self.classes)
            for k, (mx, th_k, band_k) in enumerate(self.classes):
                f.size_class_max[k] = int(min(mx, 0xFFFFFFFF))
                f.size_class_threshold[k][0] = float(np.float32(th_k[0]))
                f.size_class_threshold[k][1] = float(np.float32(th_k[1]))
                f.size_class_band[k][0] = float(band_k[0])
                f.size_class_band[k][1] = float(band_k[1])
        return f

    def save(self, path):
        cl = np.asarray([[mx, t[0], t[1], b[0], b[1]] for mx, t, b in (self.classes or [])],
                        np.float64).reshape(-1, 5)
        np.savez(path, params=self.params, norm=self.norm, edges=self.edges,
                 threshold=np.asarray(self.threshold, np.float32),
                 band=np.asarray(self.band, np.float32),
                 prune=np.asarray([int(self.prune_bottom), int(self.prune_top)], np.uint8),
                 classes=cl, gate_max_tops=np.asarray(int(self.gate_max_tops), np.uint32))

    @classmethod
    def from_struct(cls, f: seeding.DoubletFilter) -> "FilterModel":
        """The model of a seedgb_doublet_filter (as the library's training and
        calibration drivers return it)."""
        params = np.concatenate([np.asarray(f.w1, np.float32), np.asarray(f.b1, np.float32),
                                 np.asarray(f.w2, np.float32), np.asarray(f.b2, np.float32),
                                 np.asarray(f.w3, np.float32),
                                 np.asarray([f.b3], np.float32)])
        norm = np.concatenate([np.asarray(f.mu, np.float32), np.asarray(f.isd, np.float32)])
        edges = np.asarray(f.edges[: f.n_edges], np.float32)
        classes = [(int(f.size_class_max[k]),
                    (float(f.size_class_threshold[k][0]), float(f.size_class_threshold[k][1])),
                    (float(f.size_class_band[k][0]), float(f.size_class_band[k][1])))
                   for k in range(f.n_size_classes)]
        return cls(params, norm, edges, (float(f.threshold[0]), float(f.threshold[1])),
                   (float(f.band[0]), float(f.band[1])), int(f.prune_bottom), int(f.prune_top),
                   classes or None, int(f.gate_max_tops))

    @classmethod
    def load(cls, path):
        with np.load(path) as z:
            cl = [(int(r[0]), (float(r[1]), float(r[2])), (float(r[3]), float(r[4])))
                  for r in z["classes"]] if "classes" in z.files else []
            return cls(z["params"].astype(np.float32), z["norm"].astype(np.float32),
                       z["edges"].astype(np.float32), tuple(float(v) for v in z["threshold"]),
                       tuple(float(v) for v in z["band"]), int(z["prune"][0]),
                       int(z["prune"][1]), cl or None,
                       int(z["gate_max_tops"]) if "gate_max_tops" in z.files else 0)


def init_params(seed=0) -> np.ndarray:
    """He-uniform weights, zero biases."""
    rng = np.random.default_rng(seed)
    p = np.zeros(seeding.mlp_num_params(), np.float32)
    lim1, lim2, lim3 = np.sqrt(6 / 8), np.sqrt(6 / 32), np.sqrt(3 / 32)
    p[0:256] = rng.uniform(-lim1, lim1, 256)
    p[288:1312] = rng.uniform(-lim2, lim2, 1024)
    p[1344:1376] = rng.uniform(-lim3, lim3, 32)
    return p


def scoring_model(edges=None) -> FilterModel:
    """A filter that scores (for the dump) but prunes nothing."""
    return FilterModel(init_params(), np.concatenate([np.zeros(8), np.ones(8)]).astype(np.float32),
                       band_edges() if edges is None else np.asarray(edges, np.float32),
                       prune_bottom=seeding.FILTER_KEEP, prune_top=seeding.FILTER_KEEP)


def _key(torch, ev, mid, other):
    return (ev.to(torch.int64) << 42) | (mid.to(torch.int64) << 21) | other.to(torch.int64)


def _device_events(torch, events, device):
    return [seeding.SpacepointCollection.from_numpy(e, device=device) for e in events]


def run_dump(alg, sps, model: FilterModel, stream=None, records=None, triplets=False):
    """Plain seeding of a batch with every scored doublet recorded (and every
    triplet of the scored middles when `triplets`).  Returns (seed buffers,
    doublet records as a torch uint8 tensor [n, 48][, triplet records as a
    torch int32 tensor [m, 4]])."""
    import torch
    dev = sps[0].global_.device
    n_sp = sum(len(s) for s in sps)
    guess, tguess = 80 * n_sp + 1024, 8 * n_sp + 1024
    trec = None
    for _ in range(3):
        if records is None or records.shape[0] < guess:
            records = torch.empty((guess, 48), dtype=torch.uint8, device=dev)
        if triplets and (trec is None or trec.shape[0] < tguess):
            trec = torch.empty((tguess, 4), dtype=torch.int32, device=dev)
        alg.set_filter(model.struct(prune=(False, False), band=(0.0, 1.0)))
        alg.set_doublet_dump(records)
        if triplets:
            alg.set_triplet_dump(trec.view(torch.uint8))
        outs = alg.run_batch(sps, stream=stream)
        _, _, nrec, ntrip = alg.filter_stats(len(sps), stream, triplets=True)
        if nrec <= records.shape[0] and (not triplets or ntrip <= trec.shape[0]):
            break
        guess = max(guess, int(nrec * 1.1) + 1024)
        tguess = max(tguess, int(ntrip * 1.1) + 1024)
        records = None
        trec = None
    alg.set_doublet_dump(None)
    alg.set_triplet_dump(None)
    alg.set_filter(None)
    if triplets:
        return outs, records[:nrec], trec[:ntrip]
    return outs, records[:nrec]


def _ordered(torch, rec):
    """Doublet records in a fixed order (event, role, middle, other): the dump
    appends them in the order the GPU finds them, which varies between runs."""
    if len(rec) < 2:
        return rec
    words = rec.view(torch.int32).to(torch.int64) & 0xffffffff
    minor = (words[:, 0] << 32) | words[:, 1]
    order = torch.sort(minor, stable=True).indices
    order = order[torch.sort(words[order, 2], stable=True).indices]
    return rec[order]


def _labels(torch, rec, outs, trec=None):
    """Per-record label: the doublet belongs to an accepted seed, or, with
    triplet records `trec`, to any triplet (a doublet in no triplet can
    change no seed)."""
    words = rec.view(torch.int32)
    mid = words[:, 0].to(torch.int64) & 0xffffffff
    oth = words[:, 1].to(torch.int64) & 0xffffffff
    role = words[:, 2].to(torch.int64) & 0xffffffff
    ev = role >> 1
    top = (role & 1).bool()
    kb, kt = [], []
    if trec is not None:
        t64 = trec.to(torch.int64) & 0xffffffff
        kb.append(_key(torch, t64[:, 3], t64[:, 0], t64[:, 1]))
        kt.append(_key(torch, t64[:, 3], t64[:, 0], t64[:, 2]))
    else:
        for e, o in enumerate(outs):
            n = int(o.size.item())
            if n == 0:
                continue
            ee = torch.full((n,), e, dtype=torch.int64, device=rec.device)
            b = o.bottom_index[:n].to(torch.int64) & 0xffffffff
            m = o.middle_index[:n].to(torch.int64) & 0xffffffff
            t = o.top_index[:n].to(torch.int64) & 0xffffffff
            kb.append(_key(torch, ee, m, b))
            kt.append(_key(torch, ee, m, t))
    key = _key(torch, ev, mid, oth)
    if not kb:
        return torch.zeros(len(rec), dtype=torch.float32, device=rec.device), top
    kb = torch.unique(torch.cat(kb))
    kt = torch.unique(torch.cat(kt))
    lab = torch.where(top, torch.isin(key, kt), torch.isin(key, kb))
    return lab.to(torch.float32), top


@dataclasses.dataclass
class Dataset:
    features: "object"   # torch fp32 [n, 8] on the device
    labels: "object"     # torch fp32 [n]
    n_doublets: int      # doublets before negative subsampling
    n_positive: int
    neg_keep: float


def collect(alg, events, neg_keep=0.05, batch=8, seed=0, model=None, roles=(1,),
            label="seed") -> Dataset:
    """Training doublets of `events` (numpy event dicts), labelled by the
    plain seeder (label "seed": in an accepted seed; "triplet": in any
    triplet), negatives subsampled with probability neg_keep; roles: 0
    middle-bottom, 1 middle-top."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    model = model or scoring_model()
    feats, labs = [], []
    n_all = n_pos = 0
    records = None
    for i in range(0, len(events), batch):
        sps = _device_events(torch, events[i:i + batch], dev)
        if label == "triplet":
            outs, rec, trec = run_dump(alg, sps, model, records=records, triplets=True)
        else:
            outs, rec = run_dump(alg, sps, model, records=records)
            trec = None
        rec = _ordered(torch, rec)
        lab, top = _labels(torch, rec, outs, trec)
        want = torch.zeros_like(top)
        for r in roles:
            want |= top if r == 1 else ~top
        lab = torch.where(want, lab, torch.full_like(lab, -1.0))
        keep = want & ((lab > 0) | (torch.rand(len(lab), generator=gen, device=dev) < neg_keep))
        f = rec[keep].view(torch.float32)[:, 3:11].contiguous()
        feats.append(f)
        labs.append(lab[keep])
        n_all += int(want.sum().item())
        n_pos += int((lab > 0).sum().item())
        records = None
    return Dataset(torch.cat(feats), torch.cat(labs), n_all, n_pos, neg_keep)


def feature_norm(features) -> np.ndarray:
    """mu and 1/sigma of the training features (fp32 [16])."""
    f = features.double()
    mu = f.mean(0)
    sd = f.std(0).clamp_min(1e-6)
    return np.concatenate([mu.cpu().numpy(), (1.0 / sd).cpu().numpy()]).astype(np.float32)


def train(data: Dataset, epochs=3, batch=16384, lr=3e-3, pos_weight=None, seed=0,
          params=None, log=None):
    """Adam on the library's forward/backward kernels.  Returns
    (params fp32 numpy, norm, per-epoch mean loss)."""
    import torch
    dev = data.features.device
    n = len(data.labels)
    norm = feature_norm(data.features)
    if pos_weight is None:
        # the negatives were subsampled: weight positives by the kept ratio
        pos = float(data.labels.sum().item())
        pos_weight = max(1.0, (n - pos) / max(pos, 1.0))
    P = torch.from_numpy(init_params(seed) if params is None else params.copy()).to(dev)
    normd = torch.from_numpy(norm).to(dev)
    G = torch.zeros_like(P)
    M = torch.zeros_like(P)
    V = torch.zeros_like(P)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    step = 0
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen, device=dev)
        X = data.features[perm]
        Y = data.labels[perm]
        acc = torch.zeros(1, dtype=torch.float64, device=dev)
        nb = 0
        for i in range(0, n, batch):
            x = X[i:i + batch]
            y = Y[i:i + batch]
            seeding.mlp_grad(P, normd, x, y, pos_weight, G, loss)
            step += 1
            seeding.mlp_adam(P, G, M, V, step, lr)
            acc += loss
            nb += 1
        hist.append(float(acc.item()) / max(nb, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4f}")
    return P.cpu().numpy(), norm, hist


def pruned_fraction(per_event):
    """Per event, the pruned share of the scored doublets (filter_stats rows:
    scored / pruned middle-bottom, scored / pruned middle-top)."""
    per = np.asarray(per_event, np.float64)
    return (per[:, 1] + per[:, 3]) / np.maximum(per[:, 0] + per[:, 2], 1)


def seed_keys(outs):
    """Per event, the set of (bottom, middle, top) of a batch's seed buffers."""
    res = []
    for o in outs:
        s = o.to_numpy()
        res.append(set(zip(s["bottom"].tolist(), s["middle"].tolist(), s["top"].tolist())))
    return res


def compare(plain, learned):
    """Per-event recall of the plain seeds and seeds outside the plain set."""
    rec, out = [], []
    for p, l in zip(plain, learned):
        rec.append(len(p & l) / len(p) if p else 1.0)
        out.append(len(l - p))
    return np.asarray(rec), np.asarray(out)


def middle_scores(torch, rec, outs):
    """Per middle with both roles, from a scored plain run's doublet records
    and seeds: (event, best middle-top logit, plain seed count, middle-top
    doublet count), numpy arrays."""
    words = rec.view(torch.int32)
    role = words[:, 2].to(torch.int64) & 0xffffffff
    top = (role & 1).bool()
    ev = (role >> 1)[top]
    mid = (words[:, 0].to(torch.int64) & 0xffffffff)[top]
    logit = rec.view(torch.float32)[:, 11][top]
    key = (ev << 32) | mid
    ukey, inv = torch.unique(key, return_inverse=True)
    best = torch.full((len(ukey),), -float("inf"), dtype=torch.float32, device=rec.device)
    best = best.scatter_reduce(0, inv, logit, reduce="amax", include_self=True)
    n_mt = torch.bincount(inv, minlength=len(ukey))
    seeds = torch.zeros(len(ukey), dtype=torch.int64, device=rec.device)
    for e, o in enumerate(outs):
        n = int(o.size.item())
        if n == 0:
            continue
        sk = (torch.full((n,), e, dtype=torch.int64, device=rec.device) << 32) | (
            o.middle_index[:n].to(torch.int64) & 0xffffffff)
        pos = torch.searchsorted(ukey, sk)
        hit = (pos < len(ukey)) & (ukey[pos.clamp_max(len(ukey) - 1)] == sk)
        seeds.index_add_(0, pos[hit], torch.ones(int(hit.sum().item()), dtype=torch.int64,
                                                   device=rec.device))
    return ((ukey >> 32).cpu().numpy(), best.cpu().numpy(), seeds.cpu().numpy(),
            n_mt.cpu().numpy())


def gate_recall(ev, best, seeds, n_mt, n_events, thr, max_tops=0):
    """Exact per-event seed recall and pruned fraction of the middle gate at
    threshold `thr` (the kept middles keep exactly their plain seeds; middles
    above max_tops middle-top doublets are kept unscored)."""
    kept = (best >= thr) | ((n_mt > max_tops) if max_tops else False)
    tot = np.bincount(ev, weights=seeds, minlength=n_events)
    keep = np.bincount(ev, weights=seeds * kept, minlength=n_events)
    mt = np.bincount(ev, weights=n_mt, minlength=n_events)
    gated = np.bincount(ev, weights=n_mt * ~kept, minlength=n_events)
    rec = np.where(tot > 0, keep / np.maximum(tot, 1), 1.0)
    return rec, keep.sum() / max(tot.sum(), 1), gated / np.maximum(mt, 1)


def calibrate_gate(alg, model: FilterModel, events, target=0.995, margin=0.05, log=None,
                   min_event=0.0, **_):
    """Middle-gate threshold and pruned-fraction band on held-out events: the
    highest threshold on a middle's best middle-top logit whose exact seed
    recall (read off one scored plain run) is >= `target` over all held-out
    seeds and >= `min_event` on every event; then one gated run confirms the
    recall and that no seed lies outside the plain set."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    sps = _device_events(torch, events, dev)
    outs, rec = run_dump(alg, sps, model)
    plain = seed_keys(outs)
    ev, best, seeds, n_mt = middle_scores(torch, rec, outs)
    mx = int(model.gate_max_tops)
    cand = np.unique(best[(seeds > 0) & ((n_mt <= mx) if mx else True)])
    lo, hi = 0, len(cand) - 1          # recall is non-increasing in the threshold
    chosen = -np.inf
    while lo <= hi:
        mid = (lo + hi) // 2
        r, agg, _ = gate_recall(ev, best, seeds, n_mt, len(events), cand[mid], mx)
        if agg >= target and r.min() >= min_event:
            chosen = float(cand[mid])
            lo = mid + 1
        else:
            hi = mid - 1
    r, agg, frac = gate_recall(ev, best, seeds, n_mt, len(events), chosen, mx)
    thr = (-np.inf, chosen)
    alg.set_filter(model.struct(threshold=thr, band=(0.0, 1.0)))
    louts = alg.run_batch(sps)
    per, _, _ = alg.filter_stats(len(sps))
    alg.set_filter(None)
    rr, oo = compare(plain, seed_keys(louts))
    frac_run = pruned_fraction(per)
    c = {"threshold": thr, "recall": float(agg), "min_recall": float(r.min()),
         "mean_recall": float(r.mean()), "pruned_fraction": [float(frac.min()), float(frac.max())],
         "mean_pruned_fraction": float(frac.mean()),
         "gated_run": {"min_recall": float(rr.min()), "outside": int(oo.sum()),
                       "mean_pruned_fraction": float(frac_run.mean())},
         "middles": int(len(best)), "middles_gated": int((best < chosen).sum())}
    if log:
        log(f"gate threshold {chosen:.4f}: recall {agg:.5f} (event min {r.min():.5f}), "
            f"gated run min {rr.min():.5f} outside {oo.sum()}, pruned {frac.mean():.4f}")
    b = (max(0.0, float(frac.min()) - margin), min(1.0, float(frac.max()) + margin))
    return dataclasses.replace(model, threshold=thr, band=b), {"chosen": c, "band": b}


def calibrate(alg, model: FilterModel, events, target=0.995, margin=0.05,
              quantiles=(0.02, 0.015, 0.01, 0.007, 0.005, 0.003, 0.002, 0.001, 0.0005),
              log=None, criterion="total", min_event=0.0):
    """Thresholds and pruned-fraction band on held-out events (numpy dicts).
    Middle gate: calibrate_gate.  Doublet pruning: the most aggressive
    quantile whose seed recall against plain seeding reaches `target` over
    all held-out seeds (criterion "total") or on every event ("event"), and
    `min_event` on every event.  Returns (model with threshold/band set,
    report)."""
    if model.prune_top == seeding.FILTER_GATE_MIDDLE:
        if criterion == "event":
            min_event = max(min_event, target)
        return calibrate_gate(alg, model, events, target=target, margin=margin, log=log,
                              min_event=min_event)
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    sps = _device_events(torch, events, dev)
    # logits of the held-out doublets under the trained network, and labels
    outs, rec = run_dump(alg, sps, model)
    plain = seed_keys(outs)
    lab, top = _labels(torch, rec, outs)
    logit = rec.view(torch.float32)[:, 11]
    pos_b = logit[(lab > 0) & ~top].float()
    pos_t = logit[(lab > 0) & top].float()
    report = {"candidates": []}
    chosen = None
    def qt(pos, q, on):
        if not on or q <= 0.0 or not len(pos):
            return -np.inf  # keep every doublet of the role
        return float(torch.quantile(pos.cpu(), q))

    for q in quantiles:
        tb = qt(pos_b, q, model.prune_bottom)
        tt = qt(pos_t, q, model.prune_top)
        alg.set_filter(model.struct(threshold=(tb, tt), band=(0.0, 1.0)))
        louts = alg.run_batch(sps)
        per, _, _ = alg.filter_stats(len(sps))
        alg.set_filter(None)
        lkeys = seed_keys(louts)
        r, o = compare(plain, lkeys)
        total = sum(len(p) for p in plain)
        agg = sum(len(p & l) for p, l in zip(plain, lkeys)) / max(total, 1)
        frac = pruned_fraction(per)
        c = {"quantile": q, "threshold": (tb, tt), "recall": float(agg),
             "min_recall": float(r.min()), "mean_recall": float(r.mean()),
             "outside": int(o.sum()), "pruned_fraction": [float(frac.min()), float(frac.max())],
             "mean_pruned_fraction": float(frac.mean())}
        report["candidates"].append(c)
        if log:
            log(f"q={q}: thresholds ({tb:.3f}, {tt:.3f}) recall {agg:.4f} (event min "
                f"{r.min():.4f}) outside {o.sum()} pruned {frac.mean():.3f}")
        if (agg if criterion == "total" else r.min()) >= target and r.min() >= min_event:
            chosen = c
            break
    if chosen is None:
        raise RuntimeError("no threshold reaches the target recall")
    lo, hi = chosen["pruned_fraction"]
    band = (max(0.0, lo - margin), min(1.0, hi + margin))
    model = dataclasses.replace(model, threshold=chosen["threshold"], band=band)
    report["chosen"] = chosen
    report["band"] = band
    return model, report


def calibrate_classes(alg, model: FilterModel, events, class_max, target=0.995, margin=0.05,
                      log=None, **kw):
    """calibrate() separately for the held-out events of each size class
    (class k: events with <= class_max[k] spacepoints, the last class takes
    the rest).  Returns (model with size classes, report)."""
    sizes = np.asarray([len(e["global"]) for e in events])
    bounds = list(class_max)
    classes, reports = [], []
    lo = -1
    for k, mx in enumerate(bounds):
        last = k == len(bounds) - 1
        sel = [e for e, n in zip(events, sizes) if n > lo and (last or n <= mx)]
        if not sel:
            raise RuntimeError(f"no calibration event in size class {k}")
        m, rep = calibrate(alg, model, sel, target=target, margin=margin, log=log, **kw)
        classes.append((int(mx), tuple(m.threshold), tuple(m.band)))
        rep["events"] = len(sel)
        rep.pop("candidates", None)
        reports.append(rep)
        lo = mx
    out = dataclasses.replace(model, classes=classes, threshold=classes[-1][1],
                              band=classes[-1][2])
    return out, {"classes": reports}


def build_filter(alg, train_events, calib_events, epochs=3, neg_keep=0.05, target=0.995,
                 seed=0, log=None, quantiles=None, label="seed", criterion="total",
                 class_max=None, min_event=0.0, impl="library"):
    """collect -> train -> calibrate (per size class when class_max is
    given).  Returns (model, report).  impl "library": the library's C++
    drivers (seedgb_filter_train, seedgb_filter_calibrate_gate; middle gate,
    seed labels); impl "torch": the orchestration below (torch tensors as
    device buffers around the same kernels), which also serves the doublet-
    pruning mode and the triplet label."""
    if impl == "library":
        return _build_filter_library(alg, train_events, calib_events, epochs, neg_keep, target,
                                     seed, class_max, min_event)
    import torch
    t0 = time.perf_counter()
    data = collect(alg, train_events, neg_keep=neg_keep, seed=seed, label=label)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    params, norm, hist = train(data, epochs=epochs, seed=seed, log=log)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    model = FilterModel(params, norm, band_edges())
    kw = {"min_event": min_event}
    if quantiles is not None:
        kw["quantiles"] = quantiles
    if class_max:
        model, rep = calibrate_classes(alg, model, calib_events, class_max, target=target,
                                       log=log, criterion=criterion, **kw)
    else:
        model, rep = calibrate(alg, model, calib_events, target=target, log=log,
                               criterion=criterion, **kw)
    t3 = time.perf_counter()
    rep.update({"label": label, "criterion": criterion,
                "train_events": len(train_events), "calib_events": len(calib_events),
                "doublets_seen": data.n_doublets, "positives": data.n_positive,
                "samples": int(len(data.labels)), "epochs": epochs, "loss": hist,
                "collect_s": t1 - t0, "train_s": t2 - t1, "calibrate_s": t3 - t2})
    return model, rep


def _build_filter_library(alg, train_events, calib_events, epochs, neg_keep, target, seed,
                          class_max, min_event):
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.perf_counter()
    tr = _device_events(torch, train_events, dev)
    f, loss = alg.train_filter(tr, band_edges(), epochs=epochs, neg_keep=neg_keep, seed=seed)
    del tr
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ca = _device_events(torch, calib_events, dev)
    f, rec, frac = alg.calibrate_gate(f, ca, class_max=tuple(class_max or ()), target=target,
                                      min_event=min_event)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    model = FilterModel.from_struct(f)
    rep = {"impl": "library (seedgb_filter_train, seedgb_filter_calibrate_gate)",
           "label": "seed", "mode": "middle gate", "train_events": len(train_events),
           "calib_events": len(calib_events), "epochs": epochs, "loss": loss,
           "calib_recall": {"min": float(rec.min()), "mean": float(rec.mean())},
           "calib_gated_fraction": {"min": float(frac.min()), "mean": float(frac.mean()),
                                    "max": float(frac.max())},
           "train_s": t1 - t0, "calibrate_s": t2 - t1}
    return model, rep
