"""Python host mirror of traccc's seeding call surface over the C ABI.

Names and call shapes follow the reference:

* ``TripletSeedingAlgorithm(finder, grid, filter)(spacepoints) -> SeedBuffer``
  mirrors ``traccc::cuda::triplet_seeding_algorithm``
  (device/cuda/include/traccc/cuda/seeding/triplet_seeding_algorithm.hpp:35-40,
  ``operator()`` at device/common/include/traccc/seeding/device/
  triplet_seeding_algorithm.hpp:68-69).
* ``SeedParameterEstimationAlgorithm(config)(bfield, measurements, spacepoints,
  seeds) -> ParamsBuffer`` mirrors ``traccc::cuda::
  seed_parameter_estimation_algorithm`` (device/common/include/traccc/seeding/
  device/seed_parameter_estimation_algorithm.hpp:48-67).
* Config objects mirror ``seedfinder_config``, ``spacepoint_grid_config``,
  ``seedfilter_config`` and ``track_params_estimation_config``; invalid grids
  raise ``ValueError`` where the reference throws ``std::domain_error``.

Device memory is held in torch CUDA tensors; the work runs in the native
library ``_lib/libseedgb.so``.  There is no CPU fallback: without the library
or without a GPU, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

# ---------------------------------------------------------------------------
# C structures (include/seedgb.h)
# ---------------------------------------------------------------------------


class SeedfinderConfig(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "zMin", "zMax", "rMax", "rMin", "collisionRegionMin",
        "collisionRegionMax", "phiMin", "phiMax", "minPt", "cotThetaMax",
        "deltaRMin", "deltaRMax", "deltaZMax", "impactMax", "sigmaScattering",
        "maxPtScattering")] + [
        ("maxSeedsPerSpM", C.c_uint32), ("bFieldInZ", C.c_float),
        ("beamPos", C.c_float * 2)] + [(n, C.c_float) for n in (
            "radLengthPerSeed", "zAlign", "rAlign", "sigmaError", "highland",
            "maxScatteringAngle2", "pTPerHelixRadius", "minHelixDiameter2",
            "minHelixRadius", "pT2perRadius")] + [
        ("phiBinDeflectionCoverage", C.c_int32),
        ("neighbor_scope", C.c_uint32 * 2)]

    def setup(self):
        """seedfinder_config::setup(): recompute the derived members."""
        lib().seedgb_seedfinder_config_setup(C.byref(self))
        return self


class SpacepointGridConfig(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "bFieldInZ", "minPt", "rMax", "zMax", "zMin", "deltaRMax",
        "cotThetaMax", "impactMax", "phiMin", "phiMax")] + [
        ("phiBinDeflectionCoverage", C.c_int32)]


class SeedfilterConfig(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "deltaInvHelixDiameter", "impactWeightFactor", "compatSeedWeight",
        "deltaRMin")] + [("compatSeedLimit", C.c_uint64)] + [
        (n, C.c_float) for n in (
            "good_spB_min_radius", "good_spB_weight_increase",
            "good_spT_max_radius", "good_spT_weight_increase",
            "good_spB_min_weight", "seed_min_weight", "spB_min_radius")]


class TrackParamsEstimationConfig(C.Structure):
    _fields_ = [("initial_sigma", C.c_float * 6),
                ("initial_sigma_qopt", C.c_float),
                ("initial_sigma_pt_rel", C.c_float),
                ("initial_inflation", C.c_float * 6)]


class GridAxes(C.Structure):
    _fields_ = [("phi_bins", C.c_uint32), ("phi_min", C.c_float),
                ("phi_max", C.c_float), ("z_bins", C.c_uint32),
                ("z_min", C.c_float), ("z_max", C.c_float)]


class _SpacepointView(C.Structure):
    _fields_ = [("measurement_index_1", C.c_void_p),
                ("measurement_index_2", C.c_void_p), ("glob", C.c_void_p),
                ("z_variance", C.c_void_p), ("radius_variance", C.c_void_p),
                ("size", C.c_uint32)]


class _SeedBuffer(C.Structure):
    _fields_ = [("bottom_index", C.c_void_p), ("middle_index", C.c_void_p),
                ("top_index", C.c_void_p), ("quality", C.c_void_p),
                ("capacity", C.c_uint32), ("size", C.c_void_p)]


class _MeasurementView(C.Structure):
    _fields_ = [("local_position", C.c_void_p), ("surface_link", C.c_void_p),
                ("size", C.c_uint32)]


class Tune(C.Structure):
    """seedgb_tune: launch shape of the seeding kernel."""
    _fields_ = [("warps_per_cta", C.c_int32), ("middles_per_item", C.c_int32),
                ("neighbourhood_capacity", C.c_int32), ("ctas_per_sm", C.c_int32)]

    def astuple(self):
        return (self.warps_per_cta, self.middles_per_item, self.neighbourhood_capacity,
                self.ctas_per_sm)


class FilterTrainConfig(C.Structure):
    """seedgb_filter_train_config."""
    _fields_ = [("epochs", C.c_uint32), ("batch", C.c_uint32), ("learning_rate", C.c_float),
                ("neg_keep", C.c_float), ("seed", C.c_uint64), ("events_per_pass", C.c_uint32)]


# seedgb_doublet_filter.prune_bottom / prune_top modes
FILTER_KEEP, FILTER_PRUNE_DOUBLETS, FILTER_GATE_MIDDLE = 0, 1, 2


class DoubletFilter(C.Structure):
    """seedgb_doublet_filter: the learned doublet filter's network, input
    standardisation, per-role thresholds, radial band edges and the
    pruned-fraction band outside which an event is re-seeded plain."""
    _fields_ = [("mu", C.c_float * 8), ("isd", C.c_float * 8),
                ("w1", C.c_float * 256), ("b1", C.c_float * 32),
                ("w2", C.c_float * 1024), ("b2", C.c_float * 32),
                ("w3", C.c_float * 32), ("b3", C.c_float),
                ("threshold", C.c_float * 2), ("n_edges", C.c_uint32),
                ("edges", C.c_float * 15), ("prune_bottom", C.c_uint32),
                ("prune_top", C.c_uint32), ("band", C.c_float * 2),
                ("n_size_classes", C.c_uint32), ("size_class_max", C.c_uint32 * 8),
                ("size_class_threshold", (C.c_float * 2) * 8),
                ("size_class_band", (C.c_float * 2) * 8), ("gate_max_tops", C.c_uint32)]


class _SpacepointBuffer(C.Structure):
    _fields_ = [("measurement_index_1", C.c_void_p), ("measurement_index_2", C.c_void_p),
                ("global_", C.c_void_p), ("z_variance", C.c_void_p),
                ("radius_variance", C.c_void_p), ("capacity", C.c_uint32),
                ("size", C.c_void_p)]


class _ParamsBuffer(C.Structure):
    _fields_ = [("data", C.c_void_p), ("capacity", C.c_uint32),
                ("size", C.c_void_p)]


STATUS = {0: "ok", 1: "empty input", 2: "bad configuration", 3: "CUDA error",
          4: "device buffer capacity exceeded", 5: "device wait timed out",
          6: "invalid argument", 7: "unsupported configuration",
          8: "input larger than the fixed capacity of this entry point"}
OK, EMPTY, BAD_CONFIG, CUDA_ERROR, CAPACITY_OVERFLOW, TIMEOUT = 0, 1, 2, 3, 4, 5
INVALID_ARGUMENT, UNSUPPORTED, SIZE_LIMIT = 6, 7, 8
NOALLOC_MAX_SPACEPOINTS = 65536
OPTION_EXHAUSTIVE_TRIPLETS = 1
OPTION_KERNEL_TIMING = 2
OPTION_LAST_TIER_ONLY = 3
KERNEL_NAMES = ("bin_count", "bin_scan", "item_order", "bin_scatter", "bin_rsort",
                "seed_fast", "seed_mid", "seed_slow", "seed_count", "seed_compact")

PARAMS_DTYPE = np.dtype([("surface_link", "<u8"), ("params", "<f4", (6,)),
                         ("cov", "<f4", (36,))])
SEED_DTYPE = np.dtype([("bottom", "<u4"), ("middle", "<u4"), ("top", "<u4"),
                       ("quality", "<f4")])
# seedgb_ckf_bound_track_parameters: the CKF's record (parameter vector,
# surface barcode, covariance as an array of columns)
CKF_PARAMS_DTYPE = np.dtype([("vector", "<f4", (6,)), ("barcode", "<u8"),
                             ("covariance", "<f4", (36,))])


class SeedingError(RuntimeError):
    def __init__(self, status, what=""):
        super().__init__(f"{what}: {STATUS.get(status, status)} (status {status})")
        self.status = status


_lib = None


def library_path() -> str:
    return os.path.join(_build.LIBDIR, "libseedgb.so")


def lib():
    """Load the native library.  It must have been built (``build()``)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"native seeding library missing ({path}); run "
                "traccc_gb300._build.build_all() first -- there is no CPU fallback")
        L = C.CDLL(path)
        P = C.POINTER
        vp = C.c_void_p
        L.seedgb_seedfinder_config_default.argtypes = [P(SeedfinderConfig)]
        L.seedgb_seedfinder_config_setup.argtypes = [P(SeedfinderConfig)]
        L.seedgb_spacepoint_grid_config_from_finder.argtypes = [
            P(SpacepointGridConfig), P(SeedfinderConfig)]
        L.seedgb_seedfilter_config_default.argtypes = [P(SeedfilterConfig)]
        L.seedgb_track_params_estimation_config_default.argtypes = [
            P(TrackParamsEstimationConfig)]
        L.seedgb_get_axes.argtypes = [P(SpacepointGridConfig), P(GridAxes)]
        L.seedgb_get_axes.restype = C.c_int
        L.seedgb_seeding_create.argtypes = [P(SeedfinderConfig), P(SpacepointGridConfig),
                                            P(SeedfilterConfig), P(vp)]
        L.seedgb_seeding_create.restype = C.c_int
        L.seedgb_seeding_destroy.argtypes = [vp]
        L.seedgb_seeding_destroy.restype = C.c_int
        L.seedgb_seeding_reserve.argtypes = [vp, C.c_uint32, C.c_uint64]
        L.seedgb_seeding_reserve.restype = C.c_int
        L.seedgb_seeding_run.argtypes = [vp, P(_SpacepointView), P(_SeedBuffer), vp]
        L.seedgb_seeding_run.restype = C.c_int
        L.seedgb_seeding_run_batch.argtypes = [vp, P(_SpacepointView), C.c_uint32,
                                               P(_SeedBuffer), vp]
        L.seedgb_seeding_run_batch.restype = C.c_int
        L.seedgb_seeding_last_status.argtypes = [vp, vp]
        L.seedgb_seeding_last_status.restype = C.c_int
        L.seedgb_seeding_counters.argtypes = [vp, P(C.c_uint64)]
        L.seedgb_seeding_counters.restype = C.c_int
        L.seedgb_seeding_copy_grid.argtypes = [vp, C.c_uint32, P(C.c_uint32),
                                               P(C.c_uint32), C.c_uint32,
                                               P(C.c_uint32), vp]
        L.seedgb_seeding_copy_grid.restype = C.c_int
        L.seedgb_seeding_set_option.argtypes = [vp, C.c_int, C.c_int64]
        L.seedgb_seeding_set_option.restype = C.c_int
        L.seedgb_seeding_kernel_times.argtypes = [vp, P(C.c_float)]
        L.seedgb_seeding_kernel_times.restype = C.c_int
        L.seedgb_seeding_graph_create.argtypes = [vp, C.c_uint32, C.c_uint64]
        L.seedgb_seeding_graph_create.restype = C.c_int
        L.seedgb_seeding_graph_launch.argtypes = [vp, P(_SpacepointView), C.c_uint32,
                                                  P(_SeedBuffer), vp]
        L.seedgb_seeding_graph_launch.restype = C.c_int
        L.seedgb_seeding_set_tune.argtypes = [vp, P(Tune)]
        L.seedgb_seeding_set_tune.restype = C.c_int
        L.seedgb_seeding_get_tune.argtypes = [vp, P(Tune)]
        L.seedgb_seeding_get_tune.restype = C.c_int
        L.seedgb_seeding_set_filter.argtypes = [vp, P(DoubletFilter)]
        L.seedgb_seeding_set_filter.restype = C.c_int
        L.seedgb_seeding_set_doublet_dump.argtypes = [vp, vp, C.c_uint64]
        L.seedgb_seeding_set_doublet_dump.restype = C.c_int
        L.seedgb_seeding_set_triplet_dump.argtypes = [vp, vp, C.c_uint64]
        L.seedgb_seeding_set_triplet_dump.restype = C.c_int
        L.seedgb_seeding_filter_stats.argtypes = [vp, C.c_uint32, P(C.c_uint32),
                                                  P(C.c_uint8), P(C.c_uint64), P(C.c_uint64), vp]
        L.seedgb_seeding_filter_stats.restype = C.c_int
        L.seedgb_form_spacepoints.argtypes = [vp, C.c_uint32, P(_MeasurementView), vp, vp, vp,
                                              vp, vp, vp, vp, vp]
        L.seedgb_form_spacepoints.restype = C.c_int
        L.seedgb_formation_create.argtypes = [vp, C.c_uint32, P(vp)]
        L.seedgb_formation_create.restype = C.c_int
        L.seedgb_formation_destroy.argtypes = [vp]
        L.seedgb_formation_destroy.restype = C.c_int
        L.seedgb_formation_run_batch.argtypes = [vp, P(_MeasurementView), vp,
                                                 P(_SpacepointBuffer), C.c_uint32, vp]
        L.seedgb_formation_run_batch.restype = C.c_int
        L.seedgb_csv_rows.argtypes = [C.c_char_p]
        L.seedgb_csv_rows.restype = C.c_int64
        L.seedgb_csv_read_spacepoints.argtypes = [C.c_char_p, C.c_char_p, C.c_uint64, vp, vp,
                                                  vp, vp, vp, P(C.c_uint64)]
        L.seedgb_csv_read_spacepoints.restype = C.c_int
        L.seedgb_csv_read_measurements.argtypes = [C.c_char_p, C.c_uint64, vp, vp, vp,
                                                   P(C.c_uint64)]
        L.seedgb_csv_read_measurements.restype = C.c_int
        L.seedgb_mlp_num_params.restype = C.c_uint32
        L.seedgb_mlp_forward.argtypes = [vp, vp, vp, C.c_uint32, vp, vp]
        L.seedgb_mlp_forward.restype = C.c_int
        L.seedgb_mlp_grad.argtypes = [vp, vp, vp, vp, C.c_uint32, C.c_float, vp, vp, vp]
        L.seedgb_mlp_grad.restype = C.c_int
        L.seedgb_mlp_adam.argtypes = [vp, vp, vp, vp, C.c_uint32, C.c_uint32, C.c_float,
                                      C.c_float, C.c_float, C.c_float, vp]
        L.seedgb_mlp_adam.restype = C.c_int
        L.seedgb_seeding_autotune.argtypes = [vp, P(_SpacepointView), C.c_uint32, P(_SeedBuffer),
                                              P(Tune), C.c_uint32, C.c_uint32, P(Tune),
                                              P(C.c_float), vp]
        L.seedgb_seeding_autotune.restype = C.c_int
        L.seedgb_filter_train.argtypes = [vp, P(_SpacepointView), C.c_uint32, P(C.c_float),
                                          C.c_uint32, P(FilterTrainConfig), P(DoubletFilter),
                                          P(C.c_float), vp]
        L.seedgb_filter_train.restype = C.c_int
        L.seedgb_filter_calibrate_gate.argtypes = [vp, P(_SpacepointView), C.c_uint32,
                                                   P(C.c_uint32), C.c_uint32, C.c_float,
                                                   C.c_float, C.c_float, P(DoubletFilter),
                                                   P(C.c_float), P(C.c_float), vp]
        L.seedgb_filter_calibrate_gate.restype = C.c_int
        L.seedgb_params_create.argtypes = [P(TrackParamsEstimationConfig), P(vp)]
        L.seedgb_params_create.restype = C.c_int
        L.seedgb_params_destroy.argtypes = [vp]
        L.seedgb_params_destroy.restype = C.c_int
        L.seedgb_params_run.argtypes = [vp, P(C.c_float), P(_MeasurementView),
                                        P(_SpacepointView), P(_SeedBuffer),
                                        P(_ParamsBuffer), vp]
        L.seedgb_params_run.restype = C.c_int
        L.seedgb_params_run_batch.argtypes = [vp, P(C.c_float), P(_MeasurementView),
                                              P(_SpacepointView), P(_SeedBuffer),
                                              P(_ParamsBuffer), C.c_uint32, vp]
        L.seedgb_params_run_batch.restype = C.c_int
        L.seedgb_params_to_ckf.argtypes = [P(_ParamsBuffer), vp, C.c_uint32, vp, vp]
        L.seedgb_params_to_ckf.restype = C.c_int
        L.seedgb_spacepoint_binning_noalloc.argtypes = [
            P(SeedfinderConfig), P(SpacepointGridConfig), P(_SpacepointView), vp, vp, vp]
        L.seedgb_spacepoint_binning_noalloc.restype = C.c_int
        L.seedgb_status_string.argtypes = [C.c_int]
        L.seedgb_status_string.restype = C.c_char_p
        L.seedgb_abi_version.restype = C.c_uint32
        _lib = L
    return _lib


def _check(status, what):
    if status != OK:
        raise SeedingError(status, what)


def default_configs():
    """Reference defaults: (seedfinder, spacepoint_grid, seedfilter,
    track_params_estimation) configs."""
    L = lib()
    f, g, fl, tp = (SeedfinderConfig(), SpacepointGridConfig(), SeedfilterConfig(),
                    TrackParamsEstimationConfig())
    L.seedgb_seedfinder_config_default(C.byref(f))
    L.seedgb_spacepoint_grid_config_from_finder(C.byref(g), C.byref(f))
    L.seedgb_seedfilter_config_default(C.byref(fl))
    L.seedgb_track_params_estimation_config_default(C.byref(tp))
    return f, g, fl, tp


def grid_config_from_finder(f: SeedfinderConfig) -> SpacepointGridConfig:
    g = SpacepointGridConfig()
    lib().seedgb_spacepoint_grid_config_from_finder(C.byref(g), C.byref(f))
    return g


def get_axes(g: SpacepointGridConfig) -> GridAxes:
    a = GridAxes()
    st = lib().seedgb_get_axes(C.byref(g), C.byref(a))
    if st == BAD_CONFIG:
        raise ValueError("invalid spacepoint grid configuration")
    _check(st, "get_axes")
    return a


# ---------------------------------------------------------------------------
# Device collections (torch tensors)
# ---------------------------------------------------------------------------


def _torch():
    import torch
    return torch


def _stream_ptr(stream):
    """A torch.cuda.Stream, a raw cudaStream_t (int) or None (current stream)."""
    if isinstance(stream, int):
        return C.c_void_p(stream)
    if stream is None:
        stream = _torch().cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


class SpacepointCollection:
    """Device SoA of edm::spacepoint_collection (spacepoint_collection.hpp:
    222-234): measurement_index_1/2 (u32, stored as int32), global (N, 3 f32,
    xyz interleaved), z_variance, radius_variance (f32)."""

    def __init__(self, measurement_index_1, measurement_index_2, global_,
                 z_variance, radius_variance):
        self.measurement_index_1 = measurement_index_1
        self.measurement_index_2 = measurement_index_2
        self.global_ = global_
        self.z_variance = z_variance
        self.radius_variance = radius_variance

    @classmethod
    def from_numpy(cls, ev, device="cuda"):
        torch = _torch()
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).view(dt)).to(device)
        return cls(t(ev["measurement_index_1"].astype(np.uint32), np.int32),
                   t(ev["measurement_index_2"].astype(np.uint32), np.int32),
                   t(np.asarray(ev["global"], np.float32).reshape(-1, 3), np.float32),
                   t(np.asarray(ev["z_variance"], np.float32), np.float32),
                   t(np.asarray(ev["radius_variance"], np.float32), np.float32))

    def __len__(self):
        return int(self.global_.shape[0])

    def view(self) -> _SpacepointView:
        n = len(self)
        return _SpacepointView(self.measurement_index_1.data_ptr(),
                               self.measurement_index_2.data_ptr(),
                               self.global_.data_ptr(), self.z_variance.data_ptr(),
                               self.radius_variance.data_ptr(), n)


class MeasurementCollection:
    """The measurement columns the path reads: local_position (M, 2 f32),
    surface_link (u64, stored as int64) and, for GBTS seeding, the cluster
    diameter (M f32, optional)."""

    def __init__(self, local_position, surface_link, diameter=None):
        self.local_position = local_position
        self.surface_link = surface_link
        self.diameter = diameter

    @classmethod
    def from_numpy(cls, ev, device="cuda"):
        torch = _torch()
        sl = torch.from_numpy(np.ascontiguousarray(ev["surface_link"], np.uint64)
                              .view(np.int64)).to(device)
        if "local_position" in ev:
            lp = torch.from_numpy(np.ascontiguousarray(ev["local_position"], np.float32)
                                  .reshape(-1, 2)).to(device)
        else:
            lp = torch.zeros((sl.shape[0], 2), dtype=torch.float32, device=device)
        dia = None
        if "diameter" in ev:
            dia = torch.from_numpy(np.ascontiguousarray(ev["diameter"], np.float32)).to(device)
        return cls(lp, sl, dia)

    def view(self) -> _MeasurementView:
        return _MeasurementView(self.local_position.data_ptr(),
                                self.surface_link.data_ptr(),
                                int(self.surface_link.shape[0]))


class SeedBuffer:
    """Device edm::seed_collection buffer: four columns of `capacity` and a
    device-resident size (seed_collection.hpp:142-146)."""

    def __init__(self, capacity, device="cuda"):
        torch = _torch()
        cap = max(1, int(capacity))
        self.capacity = int(capacity)
        self.bottom_index = torch.empty(cap, dtype=torch.int32, device=device)
        self.middle_index = torch.empty(cap, dtype=torch.int32, device=device)
        self.top_index = torch.empty(cap, dtype=torch.int32, device=device)
        self.quality = torch.empty(cap, dtype=torch.float32, device=device)
        self.size = torch.zeros(1, dtype=torch.int32, device=device)

    def buf(self) -> _SeedBuffer:
        return _SeedBuffer(self.bottom_index.data_ptr(), self.middle_index.data_ptr(),
                           self.top_index.data_ptr(), self.quality.data_ptr(),
                           self.capacity, self.size.data_ptr())

    def __len__(self):
        return int(self.size.item())

    def to_numpy(self):
        n = len(self)
        out = np.zeros(n, SEED_DTYPE)
        out["bottom"] = self.bottom_index[:n].cpu().numpy().view(np.uint32)
        out["middle"] = self.middle_index[:n].cpu().numpy().view(np.uint32)
        out["top"] = self.top_index[:n].cpu().numpy().view(np.uint32)
        out["quality"] = self.quality[:n].cpu().numpy()
        return out


class ParamsBuffer:
    """Device bound_track_parameters collection (176-byte records)."""

    def __init__(self, capacity, device="cuda"):
        torch = _torch()
        self.capacity = int(capacity)
        self.data = torch.empty(max(1, self.capacity) * PARAMS_DTYPE.itemsize,
                                dtype=torch.uint8, device=device)
        self.size = torch.zeros(1, dtype=torch.int32, device=device)

    def buf(self) -> _ParamsBuffer:
        return _ParamsBuffer(self.data.data_ptr(), self.capacity, self.size.data_ptr())

    def __len__(self):
        return int(self.size.item())

    def to_numpy(self):
        n = len(self)
        raw = self.data[: n * PARAMS_DTYPE.itemsize].cpu().numpy()
        return raw.view(PARAMS_DTYPE).copy()


# ---------------------------------------------------------------------------
# Algorithms
# ---------------------------------------------------------------------------


def params_to_ckf(params: "ParamsBuffer", out=None, out_size=None, stream=None):
    """The parameters of `params` in the combinatorial Kalman filter's record
    layout (seedgb_params_to_ckf), device-resident: returns (out, out_size),
    a uint8 CUDA tensor of capacity x 176 bytes (CKF_PARAMS_DTYPE records)
    and an int32 device count."""
    torch = _torch()
    dev = params.data.device
    cap = params.capacity
    if out is None:
        out = torch.empty(max(1, cap) * CKF_PARAMS_DTYPE.itemsize, dtype=torch.uint8,
                          device=dev)
    if out_size is None:
        out_size = torch.zeros(1, dtype=torch.int32, device=dev)
    cap_out = out.numel() // CKF_PARAMS_DTYPE.itemsize
    b = params.buf()
    _check(lib().seedgb_params_to_ckf(C.byref(b), C.c_void_p(out.data_ptr()), cap_out,
                                      C.c_void_p(out_size.data_ptr()), _stream_ptr(stream)),
           "seedgb_params_to_ckf")
    return out, out_size


def spacepoint_binning_noalloc(finder_config, grid_config, spacepoints, bin_offsets,
                               bin_sps, stream=None) -> int:
    """Bin one event into the phi-z grid without any device allocation by the
    library (seedgb_spacepoint_binning_noalloc): for callers that must not
    allocate on their event path.  bin_offsets (nbins + 1) and bin_sps (>= the
    spacepoint count) are caller-owned int32 CUDA tensors.  Returns the status
    code (SIZE_LIMIT above NOALLOC_MAX_SPACEPOINTS spacepoints)."""
    v = spacepoints.view()
    return int(lib().seedgb_spacepoint_binning_noalloc(
        C.byref(finder_config), C.byref(grid_config), C.byref(v),
        C.c_void_p(bin_offsets.data_ptr()),
        C.c_void_p(bin_sps.data_ptr() if bin_sps is not None else 0),
        _stream_ptr(stream)))


class TripletSeedingAlgorithm:
    """traccc::cuda::triplet_seeding_algorithm on one GB300."""

    def __init__(self, finder_config=None, grid_config=None, filter_config=None):
        if finder_config is None:
            finder_config, g0, f0, _ = default_configs()
            grid_config = grid_config or g0
            filter_config = filter_config or f0
        if grid_config is None:
            grid_config = grid_config_from_finder(finder_config)
        if filter_config is None:
            filter_config = default_configs()[2]
        self.finder_config = finder_config
        self.grid_config = grid_config
        self.filter_config = filter_config
        self._h = C.c_void_p()
        st = lib().seedgb_seeding_create(C.byref(finder_config), C.byref(grid_config),
                                         C.byref(filter_config), C.byref(self._h))
        if st == BAD_CONFIG:
            raise ValueError("invalid seeding configuration (get_axes domain error)")
        _check(st, "seedgb_seeding_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.seedgb_seeding_destroy(h)
            self._h = C.c_void_p()

    def max_seeds(self, n_sp: int) -> int:
        return max(1, int(self.finder_config.maxSeedsPerSpM) * int(n_sp))

    def reserve(self, max_events: int, max_total_spacepoints: int):
        _check(lib().seedgb_seeding_reserve(self._h, max_events, max_total_spacepoints),
               "seedgb_seeding_reserve")

    def set_option(self, option: int, value: int):
        _check(lib().seedgb_seeding_set_option(self._h, option, value),
               "seedgb_seeding_set_option")

    def __call__(self, spacepoints: SpacepointCollection, out: SeedBuffer | None = None,
                 stream=None) -> SeedBuffer:
        if out is None:
            out = SeedBuffer(self.max_seeds(len(spacepoints)),
                             device=spacepoints.global_.device)
        v = spacepoints.view()
        b = out.buf()
        _check(lib().seedgb_seeding_run(self._h, C.byref(v), C.byref(b),
                                        _stream_ptr(stream)), "seedgb_seeding_run")
        return out

    def run_batch(self, events, outs=None, stream=None):
        n = len(events)
        if outs is None:
            outs = [SeedBuffer(self.max_seeds(len(e)), device=e.global_.device)
                    for e in events]
        views = (_SpacepointView * n)(*[e.view() for e in events])
        bufs = (_SeedBuffer * n)(*[o.buf() for o in outs])
        _check(lib().seedgb_seeding_run_batch(self._h, views, n, bufs,
                                              _stream_ptr(stream)),
               "seedgb_seeding_run_batch")
        return outs

    def graph_create(self, max_events: int, max_total_spacepoints: int):
        """Capture the batched launch sequence for batches up to this size."""
        _check(lib().seedgb_seeding_graph_create(self._h, max_events, max_total_spacepoints),
               "seedgb_seeding_graph_create")

    def graph_launch(self, events, outs=None, stream=None):
        """run_batch through the captured graph (graph_create first)."""
        n = len(events)
        if outs is None:
            outs = [SeedBuffer(self.max_seeds(len(e)), device=e.global_.device)
                    for e in events]
        views = (_SpacepointView * n)(*[e.view() for e in events])
        bufs = (_SeedBuffer * n)(*[o.buf() for o in outs])
        _check(lib().seedgb_seeding_graph_launch(self._h, views, n, bufs,
                                                 _stream_ptr(stream)),
               "seedgb_seeding_graph_launch")
        return outs

    def set_tune(self, warps_per_cta, middles_per_item, neighbourhood_capacity, ctas_per_sm):
        t = Tune(warps_per_cta, middles_per_item, neighbourhood_capacity, ctas_per_sm)
        _check(lib().seedgb_seeding_set_tune(self._h, C.byref(t)), "seedgb_seeding_set_tune")
        return self.get_tune()

    def get_tune(self) -> tuple:
        t = Tune()
        _check(lib().seedgb_seeding_get_tune(self._h, C.byref(t)), "seedgb_seeding_get_tune")
        return t.astuple()

    def autotune(self, events, outs, candidates=None, reps=3, stream=None):
        """The library's autotuner (seedgb_seeding_autotune) on this batch:
        returns (best shape, [(shape, ms or None if skipped), ...]) and leaves
        the best shape set with the graph captured."""
        n = len(events)
        ev = (_SpacepointView * n)(*[e.view() for e in events])
        bufs = (_SeedBuffer * n)(*[o.buf() for o in outs])
        shapes = list(candidates) if candidates is not None else None
        nc = len(shapes) if shapes is not None else 3 * 5 * 4 * 2  # the library's default grid
        cand = (Tune * nc)(*[Tune(*sh) for sh in shapes]) if shapes is not None else None
        times = (C.c_float * nc)()
        best = Tune()
        _check(lib().seedgb_seeding_autotune(self._h, ev, n, bufs, cand, len(shapes or []),
                                             reps, C.byref(best), times, _stream_ptr(stream)),
               "seedgb_seeding_autotune")
        if shapes is None:
            shapes = [(w, m, nb, c) for w in (8, 12, 16) for m in (64, 256, 384, 512, 1024)
                      for nb in (1536, 2048, 2560, 3072) for c in (1, 2)]
        return best.astuple(), [(tuple(sh), (float(t) if t >= 0 else None))
                                for sh, t in zip(shapes, times)]

    def train_filter(self, events, band_edges, epochs=4, batch=16384, lr=3e-3, neg_keep=0.05,
                     seed=0, events_per_pass=8, stream=None):
        """The library's filter training (seedgb_filter_train) on device
        events: returns (DoubletFilter with prune_top = FILTER_GATE_MIDDLE,
        mean loss per epoch)."""
        n = len(events)
        ev = (_SpacepointView * n)(*[e.view() for e in events])
        edges = np.ascontiguousarray(band_edges, np.float32)
        cfg = FilterTrainConfig(epochs, batch, lr, neg_keep, seed, events_per_pass)
        out = DoubletFilter()
        loss = (C.c_float * epochs)()
        _check(lib().seedgb_filter_train(self._h, ev, n,
                                         edges.ctypes.data_as(C.POINTER(C.c_float)), len(edges),
                                         C.byref(cfg), C.byref(out), loss, _stream_ptr(stream)),
               "seedgb_filter_train")
        return out, [float(v) for v in loss]

    def calibrate_gate(self, filt: "DoubletFilter", events, class_max=(), target=0.997,
                       min_event=0.995, margin=0.05, stream=None):
        """The library's gate calibration (seedgb_filter_calibrate_gate):
        returns (calibrated DoubletFilter, per-event recall, per-event gated
        fraction)."""
        n = len(events)
        ev = (_SpacepointView * n)(*[e.view() for e in events])
        cm = (C.c_uint32 * max(1, len(class_max)))(*[min(int(c), 0xFFFFFFFF)
                                                      for c in class_max])
        f = DoubletFilter()
        C.memmove(C.byref(f), C.byref(filt), C.sizeof(DoubletFilter))
        rec = (C.c_float * n)()
        frac = (C.c_float * n)()
        _check(lib().seedgb_filter_calibrate_gate(self._h, ev, n, cm, len(class_max), target,
                                                  min_event, margin, C.byref(f), rec, frac,
                                                  _stream_ptr(stream)),
               "seedgb_filter_calibrate_gate")
        return f, np.asarray(rec, np.float64), np.asarray(frac, np.float64)

    def set_filter(self, filt: "DoubletFilter | None"):
        """Install the learned doublet filter (None: plain seeding)."""
        _check(lib().seedgb_seeding_set_filter(self._h, C.byref(filt) if filt is not None
                                               else None), "seedgb_seeding_set_filter")

    def set_doublet_dump(self, records, capacity: int = 0):
        """Record scored doublets into `records` (a device uint8 tensor of
        48-byte records, or None to stop)."""
        ptr = records.data_ptr() if records is not None else None
        cap = capacity or (records.numel() * records.element_size() // 48 if records is not None
                           else 0)
        _check(lib().seedgb_seeding_set_doublet_dump(self._h, ptr, cap),
               "seedgb_seeding_set_doublet_dump")

    def set_triplet_dump(self, records, capacity: int = 0):
        """Record the triplets of scored middles into `records` (a device
        uint8 tensor of 16-byte records, or None to stop)."""
        ptr = records.data_ptr() if records is not None else None
        cap = capacity or (records.numel() * records.element_size() // 16 if records is not None
                           else 0)
        _check(lib().seedgb_seeding_set_triplet_dump(self._h, ptr, cap),
               "seedgb_seeding_set_triplet_dump")

    def filter_stats(self, n_events: int, stream=None, triplets=False):
        """(per-event [n, 4] scored/pruned MB, scored/pruned MT counts,
        fell_back [n] bools, number of doublet records[, number of triplet
        records]) of the last run."""
        per = np.zeros((max(1, n_events), 4), np.uint32)
        fb = np.zeros(max(1, n_events), np.uint8)
        nrec = C.c_uint64(0)
        ntrip = C.c_uint64(0)
        _check(lib().seedgb_seeding_filter_stats(
            self._h, n_events, per.ctypes.data_as(C.POINTER(C.c_uint32)),
            fb.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(nrec), C.byref(ntrip),
            _stream_ptr(stream)), "seedgb_seeding_filter_stats")
        res = (per[:n_events], fb[:n_events].astype(bool), int(nrec.value))
        return res + (int(ntrip.value),) if triplets else res

    def last_status(self, stream=None) -> int:
        return int(lib().seedgb_seeding_last_status(self._h, _stream_ptr(stream)))

    def counters(self) -> dict:
        arr = (C.c_uint64 * 9)()
        _check(lib().seedgb_seeding_counters(self._h, arr), "seedgb_seeding_counters")
        keys = ("n_valid", "n_overflow_middles", "n_mb", "n_mt", "n_triplets",
                "n_seeds", "phi_undecided", "n_items", "n_last_tier_middles")
        return {k: int(v) for k, v in zip(keys, arr)}

    def kernel_times(self) -> dict:
        """Per-kernel device ms of the last run (OPTION_KERNEL_TIMING on)."""
        arr = (C.c_float * len(KERNEL_NAMES))()
        _check(lib().seedgb_seeding_kernel_times(self._h, arr), "seedgb_seeding_kernel_times")
        return {k: float(v) for k, v in zip(KERNEL_NAMES, arr)}

    def grid(self, event: int = 0, n_sp: int = 0, stream=None):
        """(bin_offsets, bin_sps) of the last run's event (host copy)."""
        ax = get_axes(self.grid_config)
        nb = ax.phi_bins * ax.z_bins
        off = np.zeros(nb + 1, np.uint32)
        sps = np.zeros(max(1, n_sp), np.uint32)
        nv = C.c_uint32(0)
        _check(lib().seedgb_seeding_copy_grid(
            self._h, event, off.ctypes.data_as(C.POINTER(C.c_uint32)),
            sps.ctypes.data_as(C.POINTER(C.c_uint32)), len(sps), C.byref(nv),
            _stream_ptr(stream)), "seedgb_seeding_copy_grid")
        return off, sps[: nv.value].copy()


SURFACE_DTYPE = np.dtype([("type", "<u4"), ("radius", "<f4"), ("rotation", "<f4", (9,)),
                          ("translation", "<f4", (3,))])
SURFACE_PLANE, SURFACE_CYLINDER = 0, 1


def form_spacepoints(surfaces, measurements: MeasurementCollection, dimensions=None,
                     stream=None):
    """silicon_pixel_spacepoint_formation on the GPU: a SpacepointCollection
    (device, capacity = number of measurements) and the number of
    spacepoints formed.  surfaces: numpy array of SURFACE_DTYPE indexed by
    surface_link; dimensions: optional device uint8 tensor (2 = pixel)."""
    torch = _torch()
    surfaces = np.ascontiguousarray(surfaces, SURFACE_DTYPE)
    dev = measurements.local_position.device
    n = len(measurements.surface_link)
    cols = SpacepointCollection(torch.empty(n, dtype=torch.int32, device=dev),
                                torch.empty(n, dtype=torch.int32, device=dev),
                                torch.empty((n, 3), dtype=torch.float32, device=dev),
                                torch.empty(n, dtype=torch.float32, device=dev),
                                torch.empty(n, dtype=torch.float32, device=dev))
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    mv = measurements.view()
    _check(lib().seedgb_form_spacepoints(
        surfaces.ctypes.data if len(surfaces) else None, len(surfaces), C.byref(mv),
        dimensions.data_ptr() if dimensions is not None else None,
        cols.measurement_index_1.data_ptr(), cols.measurement_index_2.data_ptr(),
        cols.global_.data_ptr(), cols.z_variance.data_ptr(), cols.radius_variance.data_ptr(),
        count.data_ptr(), _stream_ptr(stream)), "seedgb_form_spacepoints")
    k = int(count.item())
    return SpacepointCollection(cols.measurement_index_1[:k], cols.measurement_index_2[:k],
                                cols.global_[:k], cols.z_variance[:k],
                                cols.radius_variance[:k]), k


class SpacepointFormationAlgorithm:
    """Spacepoint formation of many events per call on a device-resident
    surface table (seedgb_formation_*): the same spacepoints as
    form_spacepoints per event, one launch sequence per batch, no host
    synchronisation."""

    def __init__(self, surfaces):
        self.surfaces = np.ascontiguousarray(surfaces, SURFACE_DTYPE)
        self._h = C.c_void_p()
        _check(lib().seedgb_formation_create(
            self.surfaces.ctypes.data if len(self.surfaces) else None, len(self.surfaces),
            C.byref(self._h)), "seedgb_formation_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.seedgb_formation_destroy(h)
            self._h = C.c_void_p()

    def run_batch(self, measurements, dimensions=None, outs=None, stream=None):
        """Returns (list of SpacepointCollection with room for every
        measurement, int32 device tensor of the per-event counts).  Slice
        each collection by its count before seeding it."""
        torch = _torch()
        n = len(measurements)
        if n == 0:
            return [], None
        dev = measurements[0].local_position.device
        if outs is None:
            outs = []
            for m in measurements:
                k = len(m.surface_link)
                outs.append(SpacepointCollection(
                    torch.empty(k, dtype=torch.int32, device=dev),
                    torch.empty(k, dtype=torch.int32, device=dev),
                    torch.empty((k, 3), dtype=torch.float32, device=dev),
                    torch.empty(k, dtype=torch.float32, device=dev),
                    torch.empty(k, dtype=torch.float32, device=dev)))
        counts = torch.zeros(n, dtype=torch.int32, device=dev)
        mv = (_MeasurementView * n)(*[m.view() for m in measurements])
        ob = (_SpacepointBuffer * n)(*[_SpacepointBuffer(
            o.measurement_index_1.data_ptr(), o.measurement_index_2.data_ptr(),
            o.global_.data_ptr(), o.z_variance.data_ptr(), o.radius_variance.data_ptr(),
            len(o.measurement_index_1), counts.data_ptr() + 4 * e) for e, o in enumerate(outs)])
        dims = None
        if dimensions is not None:
            dims = (C.c_void_p * n)(*[d.data_ptr() if d is not None else None
                                      for d in dimensions])
        _check(lib().seedgb_formation_run_batch(self._h, mv, dims, ob, n, _stream_ptr(stream)),
               "seedgb_formation_run_batch")
        return outs, counts


def read_spacepoints_csv(hits_path, meas_hit_map_path=None) -> dict:
    """traccc's CSV spacepoints (hits + measurement-hit-id map) as numpy columns."""
    n = int(lib().seedgb_csv_rows(str(hits_path).encode()))
    if n < 0:
        raise SeedingError(INVALID_ARGUMENT, f"cannot read {hits_path}")
    out = {"measurement_index_1": np.zeros(n, np.uint32),
           "measurement_index_2": np.zeros(n, np.uint32),
           "global": np.zeros((n, 3), np.float32),
           "z_variance": np.zeros(n, np.float32),
           "radius_variance": np.zeros(n, np.float32)}
    got = C.c_uint64(0)
    _check(lib().seedgb_csv_read_spacepoints(
        str(hits_path).encode(),
        str(meas_hit_map_path).encode() if meas_hit_map_path is not None else None, n,
        out["measurement_index_1"].ctypes.data, out["measurement_index_2"].ctypes.data,
        out["global"].ctypes.data, out["z_variance"].ctypes.data,
        out["radius_variance"].ctypes.data, C.byref(got)), "seedgb_csv_read_spacepoints")
    return {k: v[: got.value] for k, v in out.items()}


def read_measurements_csv(meas_path) -> dict:
    """local_position, surface_link (the file's geometry_id) and dimensions."""
    n = int(lib().seedgb_csv_rows(str(meas_path).encode()))
    if n < 0:
        raise SeedingError(INVALID_ARGUMENT, f"cannot read {meas_path}")
    out = {"local_position": np.zeros((n, 2), np.float32),
           "surface_link": np.zeros(n, np.uint64), "dimensions": np.zeros(n, np.uint8)}
    got = C.c_uint64(0)
    _check(lib().seedgb_csv_read_measurements(
        str(meas_path).encode(), n, out["local_position"].ctypes.data,
        out["surface_link"].ctypes.data, out["dimensions"].ctypes.data, C.byref(got)),
        "seedgb_csv_read_measurements")
    return {k: v[: got.value] for k, v in out.items()}


DOUBLET_DTYPE = np.dtype([("middle", "<u4"), ("other", "<u4"), ("role", "<u4"),
                          ("feat", "<f4", (8,)), ("logit", "<f4")])


def mlp_num_params() -> int:
    return int(lib().seedgb_mlp_num_params())


def mlp_forward(params, norm, features, logits=None, stream=None):
    """Logits of n doublets (device tensors: params fp32 [num_params], norm
    fp32 [16], features fp32 [n, 8]) on the tensor cores."""
    torch = _torch()
    n = int(features.shape[0])
    if logits is None:
        logits = torch.empty(n, dtype=torch.float32, device=features.device)
    _check(lib().seedgb_mlp_forward(params.data_ptr(), norm.data_ptr(), features.data_ptr(), n,
                                    logits.data_ptr(), _stream_ptr(stream)), "seedgb_mlp_forward")
    return logits


def mlp_grad(params, norm, features, labels, pos_weight, grad, loss, stream=None):
    """Gradient and value of the mean weighted logistic loss (overwrites grad, loss)."""
    _check(lib().seedgb_mlp_grad(params.data_ptr(), norm.data_ptr(), features.data_ptr(),
                                 labels.data_ptr(), int(features.shape[0]), float(pos_weight),
                                 grad.data_ptr(), loss.data_ptr(), _stream_ptr(stream)),
           "seedgb_mlp_grad")


def mlp_adam(params, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
    _check(lib().seedgb_mlp_adam(params.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(),
                                 int(params.numel()), int(step), float(lr), float(beta1),
                                 float(beta2), float(eps), _stream_ptr(stream)),
           "seedgb_mlp_adam")


class SeedParameterEstimationAlgorithm:
    """traccc::cuda::seed_parameter_estimation_algorithm (constant field)."""

    def __init__(self, config: TrackParamsEstimationConfig | None = None):
        if config is None:
            config = default_configs()[3]
        self.config = config
        self._h = C.c_void_p()
        _check(lib().seedgb_params_create(C.byref(config), C.byref(self._h)),
               "seedgb_params_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.seedgb_params_destroy(h)
            self._h = C.c_void_p()

    def __call__(self, bfield, measurements: MeasurementCollection,
                 spacepoints: SpacepointCollection, seeds: SeedBuffer,
                 out: ParamsBuffer | None = None, stream=None) -> ParamsBuffer:
        if out is None:
            out = ParamsBuffer(seeds.capacity, device=spacepoints.global_.device)
        bf = (C.c_float * 3)(*[float(x) for x in bfield])
        mv, sv, sb, pb = measurements.view(), spacepoints.view(), seeds.buf(), out.buf()
        _check(lib().seedgb_params_run(self._h, bf, C.byref(mv), C.byref(sv),
                                       C.byref(sb), C.byref(pb), _stream_ptr(stream)),
               "seedgb_params_run")
        return out

    def run_batch(self, bfield, measurements, spacepoints, seeds, outs=None, stream=None):
        """Parameters of many events in one launch (seedgb_params_run_batch):
        element e of each list belongs to event e."""
        n = len(seeds)
        if not (len(measurements) == len(spacepoints) == n):
            raise ValueError("one measurement and spacepoint collection per seed buffer")
        if outs is None:
            outs = [ParamsBuffer(s.capacity, device=sp.global_.device)
                    for s, sp in zip(seeds, spacepoints)]
        bf = (C.c_float * 3)(*[float(x) for x in bfield])
        mv = (_MeasurementView * n)(*[m.view() for m in measurements])
        sv = (_SpacepointView * n)(*[sp.view() for sp in spacepoints])
        sb = (_SeedBuffer * n)(*[s.buf() for s in seeds])
        pb = (_ParamsBuffer * n)(*[o.buf() for o in outs])
        _check(lib().seedgb_params_run_batch(self._h, bf, mv, sv, sb, pb, n,
                                             _stream_ptr(stream)),
               "seedgb_params_run_batch")
        return outs
