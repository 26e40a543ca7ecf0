"""Host-side bookkeeping of the learned filter's training data (CPU).

The doublet dump appends records in the order the GPU finds them, which
varies between runs; collect() puts them in a fixed order before labelling
and negative subsampling, so that a training run is reproducible.
"""
import numpy as np
import torch

from traccc_gb300 import learned


def _records(n, seed):
    rng = np.random.default_rng(seed)
    words = np.zeros((n, 12), np.uint32)
    words[:, 0] = rng.integers(0, 5000, n)                # middle
    words[:, 1] = rng.integers(0, 5000, n)                # other
    words[:, 2] = (rng.integers(0, 4, n) << 1) | rng.integers(0, 2, n)  # event << 1 | role
    words[:, 3:11] = rng.normal(0, 1, (n, 8)).astype(np.float32).view(np.uint32)
    words[:, 11] = rng.normal(0, 1, n).astype(np.float32).view(np.uint32)
    # unique (event, role, middle, other): the dump holds each doublet once
    _, idx = np.unique(words[:, [2, 0, 1]], axis=0, return_index=True)
    return torch.from_numpy(words[np.sort(idx)].view(np.uint8).reshape(-1, 48).copy())


def test_order_does_not_depend_on_dump_order():
    rec = _records(5000, 1)
    a = learned._ordered(torch, rec)
    perm = torch.from_numpy(np.random.default_rng(2).permutation(len(rec)))
    b = learned._ordered(torch, rec[perm])
    assert torch.equal(a, b)


def test_order_is_event_role_middle_other():
    rec = learned._ordered(torch, _records(3000, 3))
    w = rec.view(torch.int32).numpy().view(np.uint32).astype(np.int64)
    key = (w[:, 2] << 40) | (w[:, 0] << 20) | w[:, 1]
    assert np.all(np.diff(key) > 0)


def test_order_of_tiny_dumps():
    for n in (0, 1):
        rec = _records(4, 4)[:n]
        assert torch.equal(learned._ordered(torch, rec), rec)
