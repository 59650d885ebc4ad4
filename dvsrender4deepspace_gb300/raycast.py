"""Host-side mirror of the reference's renderer facade over the C-ABI.

Class and method names follow include/dvs/raycast.hpp:23-86,
include/dvs/event_sensor.hpp:40-79 and include/dvs/device_scene.hpp:5-15 so
code written against the reference reads the same; arguments are numpy
arrays and plain dicts instead of Eigen/CUDA vector types.  Errors raise the
reference's exception kinds: ValueError for std::invalid_argument, and
CapacityError / OpticalError (RuntimeError) for device status 1 / 2.

An optical state is a dict with keys position, velocity, light, light_rate
(3 floats each), rotation (quaternion x, y, z, w), intensity,
intensity_rate -- the fields of OpticalState (optical_sensor.hpp:148-152).
"""
import ctypes as C

import numpy as np

from . import _capi
from ._capi import EVENT_DTYPE, INTERVAL_DTYPE, STATE_DTYPE, check

HAPKE_DEFAULT = dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=26.0 * float(np.float32(3.14159265358979323846)) / 180.0,
                     w=0.324, B_S0=2.42, B_C0=0.0, phi=0.3)  # HapkeConfig defaults, scene_types.hpp:204-214


def state_array(states):
    """Packs one or more optical-state dicts (or OpticalState records) into the OpticalState layout."""
    if isinstance(states, (np.void, np.ndarray)) and states.dtype.names == STATE_DTYPE.names:
        # same fields, possibly without the padding (np.concatenate drops it)
        return np.atleast_1d(np.asarray(states).astype(STATE_DTYPE))
    if isinstance(states, dict):
        states = [states]
    out = np.zeros(len(states), STATE_DTYPE)
    for i, st in enumerate(states):
        for k in ("position", "velocity", "light", "light_rate"):
            out[i][k] = st.get(k, (0.0, 0.0, 0.0))
        out[i]["rotation"] = st.get("rotation", (0.0, 0.0, 0.0, 1.0))
        out[i]["intensity"] = st.get("intensity", 0.0)
        out[i]["intensity_rate"] = st.get("intensity_rate", 0.0)
    return out


def interval_array(intervals):
    """[(start_state, end_state, t0, t1), ...] -> OpticalInterval layout."""
    if isinstance(intervals, np.ndarray) and intervals.dtype.names == INTERVAL_DTYPE.names:
        # same fields, possibly without the padding (np.concatenate drops it)
        return np.ascontiguousarray(intervals.astype(INTERVAL_DTYPE))
    out = np.zeros(len(intervals), INTERVAL_DTYPE)
    for i, (a, b, t0, t1) in enumerate(intervals):
        out[i]["start"] = state_array(a)[0]
        out[i]["end"] = state_array(b)[0]
        out[i]["t0"] = t0
        out[i]["t1"] = t1
    return out


def camera_struct(camera):
    return _capi.Camera(int(camera["width"]), int(camera["height"]), float(camera["fx"]), float(camera["fy"]),
                        float(camera["cx"]), float(camera["cy"]))


def hapke_struct(h):
    return _capi.Hapke(*[float(h[k]) for k in _capi.HAPKE_KEYS])


def physic_struct(p):
    s = _capi.Physic()
    for k in _capi.PHYSIC_FLOAT_FIELDS:
        setattr(s, k, float(p[k]))
    for k in _capi.PHYSIC_INT_FIELDS:
        setattr(s, k, int(p[k]))
    return s


def derive_parameters(physic, physic_effects=True):
    """parameters()/photo_parameters() (event_sensor.cu:151-176) as a dict."""
    out = (C.c_double * 9)()
    check(_capi.load().dvs_derive_parameters(C.byref(physic_struct(physic)), int(physic_effects), out))
    keys = ("threshold_pos", "threshold_neg", "charge_scale", "refractory_time", "reference_leak",
            "reset_noise_std", "electrons_per_radiance", "dark_electrons", "integration_step")
    return dict(zip(keys, list(out)))


HALF_BOUNDS = 1   # DVS_BVH_HALF_BOUNDS
WATERTIGHT = 2    # DVS_BVH_WATERTIGHT


class DeviceScene:
    """Owner of the device-resident wide BVH, triangle and shading records
    (replaces BVHBuilder::build + DeviceScene)."""

    def __init__(self, vertices, normals, indices, camera, supersample, hapke=None, albedos=None, leaf_size=0,
                 geometry=0, builder=0):
        """geometry: dvs_bvh_params.precision flags -- 0 the reference's (FP32
        child bounds, Moller-Trumbore), HALF_BOUNDS (FP16 child bounds
        quantised outward), WATERTIGHT (watertight triangle test), or both.
        builder: dvs_bvh_params.builder -- 0 binned SAH splits with the
        reference's criterion (the default), 1 Morton radix splits."""
        lib = _capi.load()
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        a = None if albedos is None else np.ascontiguousarray(albedos, np.float32).reshape(-1)
        if n.shape != v.shape or (a is not None and a.size != v.shape[0]):
            raise ValueError("invalid indexed mesh/BVH/material dimensions")
        self.camera = dict(camera)
        self.samples = int(supersample)
        self.hapke = dict(hapke or HAPKE_DEFAULT)
        h = C.c_void_p()
        fp = C.POINTER(C.c_float)
        check(lib.dvs_scene_create(v.ctypes.data_as(fp), n.ctypes.data_as(fp), i.ctypes.data_as(C.POINTER(C.c_uint32)),
                                   a.ctypes.data_as(fp) if a is not None else None, v.shape[0], i.shape[0],
                                   C.byref(camera_struct(camera)), self.samples, C.byref(hapke_struct(self.hapke)),
                                   C.byref(_capi.BvhParams(int(leaf_size), int(geometry), int(builder))),
                                   C.byref(h)))
        self.handle = h
        self.width = int(camera["width"])
        self.height = int(camera["height"])

    def view(self, camera, supersample, hapke=None):
        """A scene with its own camera over this scene's device geometry
        (dvs_scene_view_create): no BVH rebuild, no second copy."""
        v = DeviceScene.__new__(DeviceScene)
        v.camera = dict(camera)
        v.samples = int(supersample)
        v.hapke = dict(hapke or self.hapke)
        h = C.c_void_p()
        check(_capi.load().dvs_scene_view_create(self.handle, C.byref(camera_struct(camera)), v.samples,
                                                 C.byref(hapke_struct(v.hapke)), C.byref(h)))
        v.handle = h
        v.width = int(camera["width"])
        v.height = int(camera["height"])
        return v

    @property
    def pixels(self):
        return self.width * self.height

    def info(self):
        out = _capi.SceneInfo()
        check(_capi.load().dvs_scene_info_get(self.handle, C.byref(out)))
        return {k: getattr(out, k) for k, _ in out._fields_}

    def close(self):
        if getattr(self, "handle", None):
            _capi.load().dvs_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class EventSensor:
    """EventSensor (include/dvs/event_sensor.hpp:40-79) on the GB300 path."""

    def __init__(self, scene, physic, physic_effects=True, aer_delay=True, cells_per_chunk=0, cells_per_warp=0,
                 timing=False, row_begin=0, row_end=0, circuit_precision="fp64", host_readout=False):
        lib = _capi.load()
        self.scene = scene
        self.physic = dict(physic)
        opt = _capi.SensorOptions()
        lib.dvs_sensor_options_default(C.byref(opt))
        opt.physic_effects = int(physic_effects)
        opt.aer_delay = int(aer_delay)
        opt.cells_per_chunk = int(cells_per_chunk)
        opt.cells_per_warp = int(cells_per_warp)
        opt.timing = int(timing)
        opt.row_begin = int(row_begin)
        opt.row_end = int(row_end)
        modes = {"fp64": 0, "fp32": 1, "fp32-philox": 2}
        if circuit_precision not in modes:
            raise ValueError("circuit_precision must be fp64, fp32 or fp32-philox")
        opt.circuit_precision = modes[circuit_precision]
        opt.host_readout = int(host_readout)
        h = C.c_void_p()
        check(lib.dvs_sensor_create(scene.handle, C.byref(physic_struct(physic)), C.byref(opt), C.byref(h)))
        self.handle = h
        self.max_events = int(physic["max_events_per_step"])
        self.rows = (int(row_begin), int(row_end)) if row_end > row_begin else None

    def initialize(self, pose, timestamp):
        st = state_array(pose)
        check(_capi.load().dvs_sensor_initialize(self.handle, st.ctypes.data, float(timestamp)))

    def process(self, interval):
        return self.process_many([interval])

    def process_many(self, intervals):
        ivs = interval_array(intervals)
        n = C.c_size_t()
        check(_capi.load().dvs_sensor_process(self.handle, ivs.ctypes.data, len(ivs), C.byref(n)))
        return self._read(n.value)

    def process_adaptive(self, intervals, log_tolerance=1e-2, check_convergence=False):
        """EventSensor::process_adaptive: returns the ready events, or None
        when the convergence gate rejected the window (nothing changed)."""
        ivs = interval_array(intervals)
        n = C.c_size_t()
        accepted = C.c_int32()
        check(_capi.load().dvs_sensor_process_adaptive(self.handle, ivs.ctypes.data, len(ivs), float(log_tolerance),
                                                       int(check_convergence), C.byref(accepted), C.byref(n)))
        if not accepted.value:
            return None
        return self._read(n.value)

    def refinement_statistics(self):
        out = _capi.RefinementStats()
        check(_capi.load().dvs_sensor_refinement_stats(self.handle, C.byref(out)))
        return out.as_dict()

    def last_convergence(self):
        out = _capi.ReceptorProbe()
        check(_capi.load().dvs_sensor_last_convergence(self.handle, C.byref(out)))
        return out.as_dict()

    def adaptive_cache_capacity(self):
        out = C.c_int32()
        check(_capi.load().dvs_sensor_adaptive_capacity(self.handle, C.byref(out)))
        return out.value

    def enqueue(self, intervals):
        """Launches a batch without waiting; events stay on the device."""
        ivs = interval_array(intervals)
        check(_capi.load().dvs_sensor_enqueue(self.handle, ivs.ctypes.data, len(ivs)))

    def collect(self):
        n = C.c_size_t()
        check(_capi.load().dvs_sensor_collect(self.handle, C.byref(n)))
        return self._read(n.value)

    def _read(self, count):
        out = np.zeros(max(count, 1), EVENT_DTYPE)
        got = C.c_size_t()
        check(_capi.load().dvs_sensor_read(self.handle, out.ctypes.data, len(out), C.byref(got)))
        return out[: got.value].copy()

    def drain(self):
        cap = 1 << 20
        chunks = []
        while True:
            out = np.zeros(cap, EVENT_DTYPE)
            got = C.c_size_t()
            check(_capi.load().dvs_sensor_drain(self.handle, out.ctypes.data, cap, C.byref(got)))
            chunks.append(out[: got.value].copy())
            if got.value < cap:
                break
        return np.concatenate(chunks)

    def stats(self):
        out = _capi.SensorStats()
        check(_capi.load().dvs_sensor_stats_get(self.handle, C.byref(out)))
        return out.as_dict()

    def reset_stats(self):
        check(_capi.load().dvs_sensor_stats_reset(self.handle))

    def set_tuning(self, cells_per_warp=0, rays_per_lane=2):
        check(_capi.load().dvs_sensor_set_tuning(self.handle, int(cells_per_warp), int(rays_per_lane)))

    def autotune(self, intervals):
        """Times the trace of the next batch for each packet shape and keeps
        the fastest (dvs_sensor_autotune); the batch is then processed as usual."""
        ivs = interval_array(intervals)
        out = _capi.Tuning()
        check(_capi.load().dvs_sensor_autotune(self.handle, ivs.ctypes.data, len(ivs), C.byref(out)))
        return {k: getattr(out, k) for k, _ in out._fields_}

    def device_bytes(self):
        out = C.c_uint64()
        check(_capi.load().dvs_sensor_device_bytes(self.handle, C.byref(out)))
        return out.value

    def dropped(self):
        return self.stats()["dropped"]

    def peak_queue(self):
        return self.stats()["peak_queue"]

    def stream(self):
        return _capi.load().dvs_sensor_stream(self.handle)

    def read_state(self):
        n = self.scene.pixels if not self.rows else (self.rows[1] - self.rows[0]) * self.scene.width
        st = np.zeros((n, 5), np.float64)
        rp = np.zeros(n, np.int32)
        check(_capi.load().dvs_sensor_read_state(self.handle, st.ctypes.data_as(C.POINTER(C.c_double)),
                                                 rp.ctypes.data_as(C.POINTER(C.c_int32))))
        return st, rp

    def close(self):
        if getattr(self, "handle", None):
            _capi.load().dvs_sensor_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class EventReadout:
    """EventReadout (include/dvs/event_sensor.hpp:24-37): the finite FIFO bus
    for event runs merged from several sensors -- on the host (serial, the
    reference's structure) or, with device=True, on the GPU (dvs_device_readout_*:
    radix sort, max-plus scan, device ring buffer; up to max_batch events per submit)."""

    def __init__(self, bandwidth, latency, capacity, device=False, max_batch=1 << 20):
        h = C.c_void_p()
        self.fn = "dvs_device_readout_" if device else "dvs_readout_"
        lib = _capi.load()
        if device:
            check(lib.dvs_device_readout_create(float(bandwidth), float(latency), int(capacity), int(max_batch),
                                                C.byref(h)))
        else:
            check(lib.dvs_readout_create(float(bandwidth), float(latency), int(capacity), C.byref(h)))
        self.handle = h

    def _call(self, name, *args):
        return getattr(_capi.load(), self.fn + name)(self.handle, *args)

    def _read(self, n):
        out = np.zeros(max(n, 1), EVENT_DTYPE)
        got = C.c_size_t()
        check(self._call("read", out.ctypes.data, len(out), C.byref(got)))
        return out if got.value == len(out) else out[: got.value].copy()

    def submit(self, events, now):
        ev = np.ascontiguousarray(events, EVENT_DTYPE) if len(events) else np.zeros(0, EVENT_DTYPE)
        n = C.c_size_t()
        check(self._call("submit", ev.ctypes.data if len(ev) else None, len(ev), float(now), C.byref(n)))
        return self._read(n.value)

    def drain(self):
        n = C.c_size_t()
        check(self._call("drain", C.byref(n)))
        return self._read(n.value)

    def dropped(self):
        d, p = C.c_uint64(), C.c_uint64()
        check(self._call("counters", C.byref(d), C.byref(p)))
        return d.value

    def peak_queue(self):
        d, p = C.c_uint64(), C.c_uint64()
        check(self._call("counters", C.byref(d), C.byref(p)))
        return p.value

    def last_ms(self):
        """Device time of the last submit's kernels (device readout only)."""
        ms = C.c_double()
        check(_capi.load().dvs_device_readout_last_ms(self.handle, C.byref(ms)))
        return ms.value

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self._call("destroy")
                self.handle = None
        except Exception:
            pass


class DvsRayCaster:
    """DvsRayCaster (include/dvs/raycast.hpp:23-62)."""

    def __init__(self, scene, physic, **options):
        self.scene = scene
        self.sensor = EventSensor(scene, physic, **options)

    def initialize(self, state, timestamp):
        self.sensor.initialize(state, timestamp)

    def advance(self, start, end, t0, t1):
        return self.sensor.process((start, end, t0, t1))

    def advance_many(self, intervals):
        return self.sensor.process_many(intervals)

    def drain(self):
        return self.sensor.drain()

    def dropped_events(self):
        return self.sensor.dropped()

    def peak_queue(self):
        return self.sensor.peak_queue()


def quaternion_from_matrix(m):
    """Unit quaternion (x, y, z, w) of a 3x3 rotation matrix (Shepperd's method)."""
    m = np.asarray(m, np.float64).reshape(3, 3)
    tr = m[0, 0] + m[1, 1] + m[2, 2]
    if tr > 0:
        s = np.sqrt(tr + 1.0) * 2
        w, x, y, z = 0.25 * s, (m[2, 1] - m[1, 2]) / s, (m[0, 2] - m[2, 0]) / s, (m[1, 0] - m[0, 1]) / s
    elif m[0, 0] > m[1, 1] and m[0, 0] > m[2, 2]:
        s = np.sqrt(1.0 + m[0, 0] - m[1, 1] - m[2, 2]) * 2
        w, x, y, z = (m[2, 1] - m[1, 2]) / s, 0.25 * s, (m[0, 1] + m[1, 0]) / s, (m[0, 2] + m[2, 0]) / s
    elif m[1, 1] > m[2, 2]:
        s = np.sqrt(1.0 + m[1, 1] - m[0, 0] - m[2, 2]) * 2
        w, x, y, z = (m[0, 2] - m[2, 0]) / s, (m[0, 1] + m[1, 0]) / s, 0.25 * s, (m[1, 2] + m[2, 1]) / s
    else:
        s = np.sqrt(1.0 + m[2, 2] - m[0, 0] - m[1, 1]) * 2
        w, x, y, z = (m[1, 0] - m[0, 1]) / s, (m[0, 2] + m[2, 0]) / s, (m[1, 2] + m[2, 1]) / s, 0.25 * s
    q = np.array([x, y, z, w])
    return tuple(float(v) for v in (q / np.linalg.norm(q)).astype(np.float32))


class CamRayCaster:
    """CamRayCaster (include/dvs/raycast.hpp:64-86): image and depth frames."""

    def __init__(self, scene):
        self.scene = scene

    def render_state(self, state):
        st = state_array(state)
        n = self.scene.pixels
        img = np.zeros(n, np.float32)
        dep = np.zeros(n, np.float32)
        fp = C.POINTER(C.c_float)
        check(_capi.load().dvs_cam_render(self.scene.handle, st.ctypes.data, img.ctypes.data_as(fp),
                                          dep.ctypes.data_as(fp)))
        return img, dep

    def render_blur(self, states, weights):
        """Motion-blur exposure: sum_j weights[j] * image(states[j]) in float, pose order."""
        # an explicit 80-byte record array: np.concatenate would drop the
        # trailing padding of STATE_DTYPE and the C side would misread records
        st = np.zeros(len(states), STATE_DTYPE)
        for i, s in enumerate(states):
            st[i] = state_array(s)[0]
        w = np.ascontiguousarray(weights, np.float32)
        assert len(w) == len(st)
        img = np.zeros(self.scene.pixels, np.float32)
        fp = C.POINTER(C.c_float)
        check(_capi.load().dvs_cam_render_blur(self.scene.handle, st.ctypes.data, w.ctypes.data_as(fp), len(st),
                                               img.ctypes.data_as(fp)))
        return img

    def render_main(self, camera_origin, camera_world, light_dir, light_intensity):
        """camera_world: 3x3 rotation (row-major here); light_dir: world light direction."""
        q = quaternion_from_matrix(camera_world)
        return self.render_state(dict(position=camera_origin, rotation=q, light=light_dir,
                                      intensity=light_intensity))


class SensorBatch:
    """Many EventSensors over one scene geometry advanced together
    (dvs_batch_*): each step traces every member in one persistent launch and
    integrates every member's circuits in one launch, the step captured into a
    CUDA graph and replayed while the members' shapes stay the same."""

    def __init__(self, sensors):
        self.sensors = list(sensors)
        arr = (C.c_void_p * len(self.sensors))(*[s.handle for s in self.sensors])
        h = C.c_void_p()
        check(_capi.load().dvs_batch_create(arr, len(self.sensors), C.byref(h)))
        self.handle = h

    def process(self, intervals_per_sensor):
        """intervals_per_sensor[m]: member m's next intervals (empty: idle).
        Returns the ready events of every member."""
        n = len(self.sensors)
        if len(intervals_per_sensor) != n:
            raise ValueError("one interval list per batch sensor")
        arrays = [interval_array(ivs) if len(ivs) else None for ivs in intervals_per_sensor]
        ptrs = (C.c_void_p * n)(*[a.ctypes.data if a is not None else None for a in arrays])
        counts = (C.c_size_t * n)(*[len(a) if a is not None else 0 for a in arrays])
        ready = (C.c_size_t * n)()
        check(_capi.load().dvs_batch_process(self.handle, ptrs, counts, ready))
        return [s._read(ready[m]) if counts[m] else np.zeros(0, EVENT_DTYPE) for m, s in enumerate(self.sensors)]

    def stats(self):
        out = _capi.BatchStats()
        check(_capi.load().dvs_batch_stats_get(self.handle, C.byref(out)))
        return out.as_dict()

    def close(self):
        if getattr(self, "handle", None):
            _capi.load().dvs_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
