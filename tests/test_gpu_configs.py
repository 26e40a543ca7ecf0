"""GPU seeding vs the oracle across configurations other than the default:
several z bins, a wider neighbourhood (with several z bins: up to 25 grid
bins around a middle, more than the fast kernel stages, so most middles go
through the large-capacity kernel), one and eight seeds per middle, an offset beam spot,
a higher pT threshold (fewer phi bins) and tighter impact / pT cuts, and
nonzero spacepoint variances on both seeding kernels.  Grids and seed sets
bit-exact, parameters to 1e-5."""
import numpy as np
import pytest

import oracle as O
from traccc_gb300 import seeding, synth

pytestmark = pytest.mark.gpu


def _zbins(f):
    f.cotThetaMax = 7.4


def _scope2(f):
    f.neighbor_scope[0] = 2
    f.neighbor_scope[1] = 2


def _zbins_scope2(f):
    _zbins(f)
    _scope2(f)


def _seeds(n):
    def mod(f):
        f.maxSeedsPerSpM = n
    return mod


def _beam(f):
    f.beamPos[0] = 0.5
    f.beamPos[1] = -0.3


def _minpt(f):
    f.minPt = 0.9


def _tight(f):
    f.impactMax = 5.0
    f.maxPtScattering = 5.0


VARIANTS = {"zbins": _zbins, "scope2": _scope2, "zbins_scope2": _zbins_scope2,
            "seeds1": _seeds(1), "seeds8": _seeds(8), "beam": _beam, "minpt": _minpt,
            "tight": _tight}


def _configs(mod, module):
    f, g, fl, tp = module.default_configs()
    mod(f)
    if module is O:
        O.lib().or_finder_config_setup(__import__("ctypes").byref(f))
        g = O.GridConfig()
        O.lib().or_grid_config_from_finder(__import__("ctypes").byref(g),
                                           __import__("ctypes").byref(f))
    else:
        f.setup()
        g = seeding.grid_config_from_finder(f)
    return f, g, fl, tp


@pytest.mark.parametrize("variant", list(VARIANTS))
def test_config_variant_matches_oracle(variant):
    import torch
    ev = synth.workload_event("trk1000", 9)
    mod = VARIANTS[variant]
    f, g, fl, tp = _configs(mod, seeding)
    of, og, ofl, otp = _configs(mod, O)
    ax = seeding.get_axes(g)
    if variant.startswith("zbins"):
        assert ax.z_bins > 1
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    sps = seeding.SpacepointCollection.from_numpy(ev)
    out = alg(sps)
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.OK
    off, bsp = alg.grid(0, len(ev["global"]))
    roff, rsp, _, _ = O.binning(ev, of, og, phi_mode=O.PHI_CR)
    assert np.array_equal(off, roff)
    assert np.array_equal(bsp, rsp)
    got = out.to_numpy()
    ref, _ = O.seeding(ev, of, og, ofl, phi_mode=O.PHI_CR)
    assert len(ref) > 0
    assert np.array_equal(got, ref)
    if variant == "beam":
        est = seeding.SeedParameterEstimationAlgorithm(tp)
        params = est((0.0, 0.0, float(f.bFieldInZ)), seeding.MeasurementCollection.from_numpy(ev),
                     sps, out).to_numpy()
        refp = O.track_params(ev, ref, (0.0, 0.0, float(of.bFieldInZ)), otp)
        assert np.array_equal(params["surface_link"], refp["surface_link"])
        assert np.allclose(params["params"], refp["params"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("variant", ["default", "zbins_scope2"])
def test_variance_event_matches_oracle(variant):
    """Nonzero spacepoint variances (the kernels' variance bodies): the
    default config through the fast kernel, several z bins with scope 2
    mostly through the large-capacity kernel."""
    import torch
    ev = synth.workload_event("trk1000", 9)
    rng = np.random.default_rng(9)
    ev["z_variance"] = rng.uniform(0.0, 0.05, len(ev["layer"])).astype(np.float32)
    ev["radius_variance"] = rng.uniform(0.0, 0.01, len(ev["layer"])).astype(np.float32)
    mod = VARIANTS.get(variant, lambda f: None)
    f, g, fl, _ = _configs(mod, seeding)
    of, og, ofl, _ = _configs(mod, O)
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    out = alg(seeding.SpacepointCollection.from_numpy(ev))
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.OK
    assert (alg.counters()["n_overflow_middles"] > 0) == (variant == "zbins_scope2")
    got = out.to_numpy()
    ref, _ = O.seeding(ev, of, og, ofl, phi_mode=O.PHI_CR)
    assert len(ref) > 0
    assert np.array_equal(got, ref)


def test_general_path_tiers_match_oracle():
    """A staging capacity too small for any neighbourhood sends every middle
    to the general path; its middle tier seeds them (lists above the fast
    capacities included), and with SEEDGB_OPTION_LAST_TIER_ONLY the last,
    large-capacity tier seeds all of them.  Seeds equal the oracle's on a
    100k-spacepoint event and on the densest event of an uneven batch."""
    import torch
    dense = max(synth.batch_events(64, 3), key=lambda e: len(e["global"]))
    assert len(dense["global"]) > 110000
    for ev in (synth.workload_event("pileup9k", 6), dense):
        ref, _ = O.seeding(ev, phi_mode=O.PHI_CR)
        for last_only in (False, True):
            alg = seeding.TripletSeedingAlgorithm()
            alg.set_tune(16, 256, 256, 1)
            alg.set_option(seeding.OPTION_LAST_TIER_ONLY, int(last_only))
            out = alg(seeding.SpacepointCollection.from_numpy(ev))
            torch.cuda.synchronize()
            assert alg.last_status() == seeding.OK
            c = alg.counters()
            assert c["n_overflow_middles"] >= 0.9 * c["n_valid"] > 0
            if last_only:
                assert c["n_last_tier_middles"] == c["n_overflow_middles"], c
            else:
                assert c["n_last_tier_middles"] == 0, c
            assert np.array_equal(out.to_numpy(), ref)


@pytest.mark.parametrize("variant", ["seeds8", "beam", "tight"])
def test_config_variant_dense_event(variant):
    """Config variants on a 100k-spacepoint event: eight seeds per middle
    (the most the seed slots hold), an offset beam spot, tighter cuts."""
    import torch
    ev = synth.workload_event("pileup9k", 8)
    mod = VARIANTS[variant]
    f, g, fl, _ = _configs(mod, seeding)
    of, og, ofl, _ = _configs(mod, O)
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    out = alg(seeding.SpacepointCollection.from_numpy(ev))
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.OK
    ref, _ = O.seeding(ev, of, og, ofl, phi_mode=O.PHI_CR)
    assert len(ref) > 0
    assert np.array_equal(out.to_numpy(), ref)


def test_zbins_dense_event():
    """Several z bins on a 100k-spacepoint event (fast path with z segments)."""
    import torch
    ev = synth.workload_event("pileup9k", 5)
    f, g, fl, _ = _configs(_zbins, seeding)
    of, og, ofl, _ = _configs(_zbins, O)
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    out = alg(seeding.SpacepointCollection.from_numpy(ev))
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.OK
    ref, _ = O.seeding(ev, of, og, ofl, phi_mode=O.PHI_CR)
    assert np.array_equal(out.to_numpy(), ref)
