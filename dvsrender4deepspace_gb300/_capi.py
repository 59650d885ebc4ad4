"""ctypes binding of libdvs_gb300.so (the C-ABI in include/dvs_gb300.h).

The library is built in-tree (dvsrender4deepspace_gb300/build.py).  Loading
fails loudly when it is missing or has no CUDA device behind it: there is no
CPU fallback for the hot path.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libdvs_gb300.so")

DVS_OK = 0
DVS_ERR_CAPACITY = 1
DVS_ERR_OPTICAL = 2
DVS_ERR_INVALID = 3
DVS_ERR_CUDA = 4
DVS_ERR_STALLED = 5
DVS_ERR_OUTPUT_SMALL = 6

# Layout-identical to OpticalState / OpticalInterval / Event of the reference
# (include/dvs/optical_sensor.hpp:148-153, include/dvs/dvs_base.hpp:9-18).
STATE_DTYPE = np.dtype({"names": ["position", "velocity", "light", "light_rate", "rotation", "intensity",
                                  "intensity_rate"],
                        "formats": [("<f4", 3), ("<f4", 3), ("<f4", 3), ("<f4", 3), ("<f4", 4), "<f4", "<f4"],
                        "offsets": [0, 12, 24, 36, 48, 64, 68], "itemsize": 80})
INTERVAL_DTYPE = np.dtype({"names": ["start", "end", "t0", "t1"], "formats": [STATE_DTYPE, STATE_DTYPE, "<f8", "<f8"],
                           "offsets": [0, 80, 160, 168], "itemsize": 176})
EVENT_DTYPE = np.dtype([("timestamp", "<f8"), ("x", "<i2"), ("y", "<i2"), ("polarity", "i1"), ("depth", "<f4")])
assert EVENT_DTYPE.itemsize == 17


class Camera(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float)]


HAPKE_KEYS = ("b", "c", "hS", "hC", "thetap", "w", "B_S0", "B_C0", "phi")


class Hapke(C.Structure):
    _fields_ = [(k, C.c_float) for k in HAPKE_KEYS]


PHYSIC_FLOAT_FIELDS = ("threshold_pos", "threshold_neg", "refractory_time", "readout_bandwidth",
                       "readout_latency", "threshold_std", "threshold_min", "wavelength_nm",
                       "quantum_efficiency", "pixel_pitch_um", "fill_factor", "f_number",
                       "lens_transmission", "radiance_scale", "temperature_k", "subthreshold_kappa",
                       "receptor_capacitance_f", "reset_capacitance_f", "dark_current_a",
                       "reset_leakage_a", "circuit_step")
PHYSIC_INT_FIELDS = ("photon_shot_noise", "reset_thermal_noise", "random_seed", "max_events_per_step",
                     "readout_queue_capacity")


class Physic(C.Structure):
    _fields_ = [(k, C.c_float) for k in PHYSIC_FLOAT_FIELDS] + [(k, C.c_int32) for k in PHYSIC_INT_FIELDS]


class SensorOptions(C.Structure):
    _fields_ = [("physic_effects", C.c_int32), ("aer_delay", C.c_int32), ("cells_per_chunk", C.c_int32),
                ("cells_per_warp", C.c_int32), ("timing", C.c_int32), ("row_begin", C.c_int32),
                ("row_end", C.c_int32), ("circuit_precision", C.c_int32), ("host_readout", C.c_int32)]


class BvhParams(C.Structure):
    _fields_ = [("leaf_size", C.c_int32), ("precision", C.c_int32), ("builder", C.c_int32), ("reserved", C.c_int32)]


class SceneInfo(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("vertices", C.c_uint64), ("nodes", C.c_uint64), ("depth", C.c_int32),
                ("root", C.c_int32), ("device_bytes", C.c_uint64), ("build_seconds", C.c_double),
                ("leaf_size", C.c_int32), ("precision", C.c_int32), ("builder", C.c_int32),
                ("reserved", C.c_int32), ("sah_node_visits", C.c_double), ("sah_triangle_tests", C.c_double)]


class BatchStats(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("graph_launches", C.c_uint64), ("graph_captures", C.c_uint64),
                ("persistent_launches", C.c_uint64), ("trace_items", C.c_uint64), ("step_ms", C.c_double),
                ("host_ms", C.c_double), ("capture_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SensorStats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("events_generated", C.c_uint64),
                ("events_delivered", C.c_uint64), ("dropped", C.c_uint64), ("peak_queue", C.c_uint64),
                ("circuit_cells", C.c_uint64), ("launches", C.c_uint64), ("optics_ms", C.c_double),
                ("circuit_ms", C.c_double), ("events_ms", C.c_double), ("readout_ms", C.c_double),
                ("optics_launches", C.c_uint64), ("circuit_launches", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# every symbol include/dvs_gb300.h declares
EXPORTS = ("dvs_last_error", "dvs_version", "dvs_sensor_options_default", "dvs_derive_parameters",
           "dvs_scene_create", "dvs_scene_destroy", "dvs_scene_info_get", "dvs_cam_render", "dvs_sensor_create",
           "dvs_sensor_destroy", "dvs_sensor_initialize", "dvs_sensor_process", "dvs_sensor_read",
           "dvs_sensor_process_events", "dvs_sensor_enqueue", "dvs_sensor_collect", "dvs_sensor_drain", "dvs_sensor_stats_get", "dvs_sensor_stats_reset",
           "dvs_sensor_stream", "dvs_sensor_read_state", "dvs_cam_render_noalloc", "dvs_sensor_process_adaptive",
           "dvs_sensor_refinement_stats", "dvs_sensor_last_convergence", "dvs_sensor_adaptive_capacity",
           "dvs_readout_create", "dvs_readout_destroy", "dvs_readout_submit", "dvs_readout_drain", "dvs_readout_read",
           "dvs_readout_counters", "dvs_config_load", "dvs_frames_load", "dvs_trajectory_create",
           "dvs_trajectory_destroy", "dvs_trajectory_range", "dvs_trajectory_evaluate", "dvs_cam_render_blur",
           "dvs_scene_view_create", "dvs_sensor_device_bytes", "dvs_sensor_set_tuning", "dvs_sensor_autotune",
           "dvs_batch_create", "dvs_batch_destroy", "dvs_batch_process", "dvs_batch_stats_get", "dvs_noise_poisson",
           "dvs_device_readout_create", "dvs_device_readout_destroy", "dvs_device_readout_submit",
           "dvs_device_readout_drain", "dvs_device_readout_read", "dvs_device_readout_counters",
           "dvs_device_readout_last_ms")


class Tuning(C.Structure):
    _fields_ = [("cells_per_warp", C.c_int32), ("rays_per_lane", C.c_int32), ("candidates", C.c_int32),
                ("cells_timed", C.c_int32), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("cells_per_chunk", C.c_int32), ("chunk_candidates", C.c_int32), ("chunk_cells", C.c_int32),
                ("chunk_best_ms", C.c_double), ("chunk_default_ms", C.c_double)]


class SceneConfig(C.Structure):
    _fields_ = [("frame_count", C.c_int32), ("fps", C.c_float), ("imu_fps", C.c_float), ("cam_fps", C.c_float),
                ("time_resolution", C.c_float), ("blur_resolution", C.c_float), ("supersample_factor", C.c_int32),
                ("translation", C.c_float * 3), ("rotation", C.c_float * 3)]


# dvs_frame (include/dvs_gb300.h): one trajectory key of frames.bin.
FRAME_DTYPE = np.dtype({"names": ["frame_index", "timestamp_seconds", "camera_origin", "camera_world", "light_dir",
                                  "light_intensity"],
                        "formats": ["<i4", "<f8", ("<f4", 3), ("<f4", 9), ("<f4", 3), "<f4"],
                        "offsets": [0, 8, 16, 28, 64, 76], "itemsize": 80})


class RefinementStats(C.Structure):
    _fields_ = [("traced_pixel_samples", C.c_uint64), ("fallback_pixels", C.c_int32), ("maximum_knots", C.c_int32),
                ("exact_segments", C.c_int32), ("native_cell_queries", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ReceptorProbe(C.Structure):
    _fields_ = [("maximum_log_voltage_error", C.c_double), ("p99_log_voltage_error", C.c_double),
                ("mean_log_voltage_error", C.c_double), ("pixels", C.c_int32), ("circuit_cells", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

_LIB = None


def _declare(lib):
    vp, sz, f_p = C.c_void_p, C.c_size_t, C.POINTER(C.c_float)
    lib.dvs_last_error.restype = C.c_char_p
    lib.dvs_version.restype = C.c_char_p
    lib.dvs_sensor_options_default.argtypes = [C.POINTER(SensorOptions)]
    lib.dvs_sensor_options_default.restype = None
    lib.dvs_derive_parameters.argtypes = [C.POINTER(Physic), C.c_int32, C.POINTER(C.c_double)]
    lib.dvs_noise_poisson.argtypes = [C.c_int32, C.c_double, C.c_uint32, sz, C.POINTER(C.c_double)]
    lib.dvs_scene_create.argtypes = [f_p, f_p, C.POINTER(C.c_uint32), f_p, sz, sz, C.POINTER(Camera), C.c_int32,
                                     C.POINTER(Hapke), C.POINTER(BvhParams), C.POINTER(vp)]
    lib.dvs_scene_destroy.argtypes = [vp]
    lib.dvs_scene_info_get.argtypes = [vp, C.POINTER(SceneInfo)]
    lib.dvs_cam_render.argtypes = [vp, vp, f_p, f_p]
    lib.dvs_sensor_create.argtypes = [vp, C.POINTER(Physic), C.POINTER(SensorOptions), C.POINTER(vp)]
    lib.dvs_sensor_destroy.argtypes = [vp]
    lib.dvs_sensor_initialize.argtypes = [vp, vp, C.c_double]
    lib.dvs_sensor_process.argtypes = [vp, vp, sz, C.POINTER(sz)]
    lib.dvs_sensor_read.argtypes = [vp, vp, sz, C.POINTER(sz)]
    lib.dvs_sensor_process_events.argtypes = [vp, vp, sz, vp, sz, C.POINTER(sz)]
    lib.dvs_sensor_drain.argtypes = [vp, vp, sz, C.POINTER(sz)]
    lib.dvs_sensor_enqueue.argtypes = [vp, vp, sz]
    lib.dvs_sensor_collect.argtypes = [vp, C.POINTER(sz)]
    lib.dvs_sensor_stats_get.argtypes = [vp, C.POINTER(SensorStats)]
    lib.dvs_sensor_stats_reset.argtypes = [vp]
    lib.dvs_sensor_stream.argtypes = [vp]
    lib.dvs_sensor_stream.restype = vp
    lib.dvs_sensor_read_state.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    lib.dvs_cam_render_noalloc.argtypes = [vp, vp, vp, vp, vp]
    lib.dvs_cam_render_blur.argtypes = [vp, vp, f_p, sz, f_p]
    lib.dvs_scene_view_create.argtypes = [vp, C.POINTER(Camera), C.c_int32, C.POINTER(Hapke), C.POINTER(vp)]
    lib.dvs_sensor_device_bytes.argtypes = [vp, C.POINTER(C.c_uint64)]
    lib.dvs_sensor_set_tuning.argtypes = [vp, C.c_int32, C.c_int32]
    lib.dvs_sensor_autotune.argtypes = [vp, vp, sz, C.POINTER(Tuning)]
    lib.dvs_sensor_process_adaptive.argtypes = [vp, vp, sz, C.c_double, C.c_int32, C.POINTER(C.c_int32),
                                                C.POINTER(sz)]
    lib.dvs_sensor_refinement_stats.argtypes = [vp, C.POINTER(RefinementStats)]
    lib.dvs_sensor_last_convergence.argtypes = [vp, C.POINTER(ReceptorProbe)]
    lib.dvs_sensor_adaptive_capacity.argtypes = [vp, C.POINTER(C.c_int32)]
    lib.dvs_readout_create.argtypes = [C.c_double, C.c_double, sz, C.POINTER(vp)]
    lib.dvs_readout_destroy.argtypes = [vp]
    lib.dvs_readout_submit.argtypes = [vp, vp, sz, C.c_double, C.POINTER(sz)]
    lib.dvs_readout_drain.argtypes = [vp, C.POINTER(sz)]
    lib.dvs_readout_read.argtypes = [vp, vp, sz, C.POINTER(sz)]
    lib.dvs_readout_counters.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.dvs_device_readout_create.argtypes = [C.c_double, C.c_double, sz, sz, C.POINTER(vp)]
    lib.dvs_device_readout_destroy.argtypes = [vp]
    lib.dvs_device_readout_submit.argtypes = [vp, vp, sz, C.c_double, C.POINTER(sz)]
    lib.dvs_device_readout_drain.argtypes = [vp, C.POINTER(sz)]
    lib.dvs_device_readout_read.argtypes = [vp, vp, sz, C.POINTER(sz)]
    lib.dvs_device_readout_counters.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.dvs_device_readout_last_ms.argtypes = [vp, C.POINTER(C.c_double)]
    lib.dvs_config_load.argtypes = [C.c_char_p, C.POINTER(Camera), C.POINTER(Physic), C.POINTER(Hapke),
                                    C.POINTER(SceneConfig)]
    lib.dvs_frames_load.argtypes = [C.c_char_p, vp, sz, C.POINTER(sz)]
    lib.dvs_trajectory_create.argtypes = [vp, sz, C.POINTER(SceneConfig), C.POINTER(vp)]
    lib.dvs_trajectory_destroy.argtypes = [vp]
    lib.dvs_trajectory_range.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    lib.dvs_trajectory_evaluate.argtypes = [vp, C.c_float, vp, f_p]
    lib.dvs_batch_create.argtypes = [vp, sz, C.POINTER(vp)]
    lib.dvs_batch_destroy.argtypes = [vp]
    lib.dvs_batch_process.argtypes = [vp, vp, vp, vp]
    lib.dvs_batch_stats_get.argtypes = [vp, C.POINTER(BatchStats)]
    return lib


def library_path():
    return LIB_PATH


def load(build_if_missing=True):
    """Open the C-ABI library, building it first if it is absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise OSError("libdvs_gb300.so is not built; run dvsrender4deepspace_gb300.build")
            from . import build
            build.build()
        _LIB = _declare(C.CDLL(LIB_PATH))
    return _LIB


class DvsError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


class CapacityError(DvsError):
    pass


class OpticalError(DvsError):
    pass


def check(status):
    if status == DVS_OK:
        return
    msg = load().dvs_last_error().decode(errors="replace")
    if status == DVS_ERR_CAPACITY:
        raise CapacityError(status, msg)
    if status == DVS_ERR_OPTICAL:
        raise OpticalError(status, msg)
    if status == DVS_ERR_INVALID:
        err = DvsError(status, msg)
        raise ValueError(msg) from err
    raise DvsError(status, msg)
