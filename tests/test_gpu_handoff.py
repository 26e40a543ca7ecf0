"""Hand-off of the estimated parameters to the combinatorial Kalman filter
(seedgb_params_to_ckf): the records the reference's track finding takes as
seeds (full_chain_algorithm.cpp:241-247), written on the device from the
library's parameter buffer.  Every field round-trips bit for bit: the
parameter vector, the barcode (= the bottom spacepoint's measurement surface
link) and the covariance as an array of columns (the transpose of the
row-major input); the count is written on the device, clipped to the output
capacity.  The input parameters themselves are checked against the oracle
in test_gpu_parity.py."""
import numpy as np
import pytest

from traccc_gb300 import seeding, synth

pytestmark = pytest.mark.gpu


def _params(name, seed):
    import torch
    ev = synth.workload_event(name, seed)
    f, g, fl, tp = seeding.default_configs()
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    est = seeding.SeedParameterEstimationAlgorithm(tp)
    sps = seeding.SpacepointCollection.from_numpy(ev)
    seeds = alg(sps)
    par = est((0.0, 0.0, float(f.bFieldInZ)), seeding.MeasurementCollection.from_numpy(ev),
              sps, seeds)
    torch.cuda.synchronize()
    return ev, seeds, par


def test_params_to_ckf_round_trip():
    import torch
    ev, seeds, par = _params("trk1000", 7)
    out, n = seeding.params_to_ckf(par)
    torch.cuda.synchronize()
    src = par.to_numpy()
    k = int(n.item())
    assert k == len(src) > 0
    got = out[: k * 176].cpu().numpy().view(seeding.CKF_PARAMS_DTYPE)
    assert np.array_equal(got["vector"].view(np.uint32), src["params"].view(np.uint32))
    assert np.array_equal(got["barcode"], src["surface_link"])
    cov_in = src["cov"].reshape(-1, 6, 6)
    cov_out = got["covariance"].reshape(-1, 6, 6)  # [col][row]
    assert np.array_equal(cov_out.transpose(0, 2, 1).view(np.uint32), cov_in.view(np.uint32))
    # the barcode is the bottom spacepoint's measurement surface
    s = seeds.to_numpy()
    mi = np.asarray(ev["measurement_index_1"])[s["bottom"]]
    assert np.array_equal(got["barcode"], np.asarray(ev["surface_link"], np.uint64)[mi])


def test_params_to_ckf_clips_to_capacity_and_writes_nothing_beyond():
    import torch
    _, _, par = _params("trk100", 3)
    m = len(par)
    assert m > 4
    out = torch.full((6 * 176,), 0xAB, dtype=torch.uint8, device="cuda")
    out_view = out[: 4 * 176]
    n = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    seeding.params_to_ckf(par, out_view, n)
    torch.cuda.synchronize()
    assert int(n.item()) == 4
    got = out[: 4 * 176].cpu().numpy().view(seeding.CKF_PARAMS_DTYPE)
    assert np.array_equal(got["vector"], par.to_numpy()["params"][:4])
    assert np.all(out[4 * 176:].cpu().numpy() == 0xAB)
