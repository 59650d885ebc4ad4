"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py``.  The oracle (``dvs_oracle.c``) restates the reference
algorithm of BugBubbles/DvsRender4DeepSpace; ``liboracle_f32.so`` keeps the
reference's FP32 ray arithmetic and evaluates Hapke in the identity form the
CUDA kernels use (``oracle_set_hapke_form(0)`` selects the reference's own
operation order), ``liboracle_f64.so`` is the FP64 oracle (reference order).  ``load_reference()`` opens ``_ref/libdvsref.so``, the reference's own
host-compilable code built here by ``make ref`` (absent on machines without
the reference checkout).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

c_f_p = C.POINTER(C.c_float)
c_d_p = C.POINTER(C.c_double)
c_i_p = C.POINTER(C.c_int)


class of3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class obvh_node(C.Structure):
    _fields_ = [("bmin", of3), ("bmax", of3), ("left", C.c_int32), ("right", C.c_int32),
                ("start", C.c_int32), ("count", C.c_int32)]


class ohapke(C.Structure):
    _fields_ = [(k, C.c_float) for k in ("b", "c", "hS", "hC", "thetap", "w", "B_S0", "B_C0", "phi")]


class ostate(C.Structure):
    _fields_ = [("position", of3), ("velocity", of3), ("light", of3), ("light_rate", of3),
                ("rotation", C.c_float * 4), ("intensity", C.c_float), ("intensity_rate", C.c_float)]


class ointerval(C.Structure):
    _fields_ = [("start", ostate), ("end", ostate), ("t0", C.c_double), ("t1", C.c_double)]


class oscene(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("vertices", C.c_void_p), ("normals", C.c_void_p),
                ("indices", C.c_void_p), ("albedos", C.c_void_p),
                ("root", C.c_int), ("width", C.c_int), ("height", C.c_int), ("samples", C.c_int),
                ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("hapke", ohapke), ("watertight", C.c_int32)]


class opixel_params(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("threshold_pos", "threshold_neg", "charge_scale",
                                          "refractory_time", "reference_leak", "reset_noise_std")]


class opixel_state(C.Structure):
    _fields_ = [("receptor_log", C.c_double), ("reference_log", C.c_double),
                ("refractory_until", C.c_double), ("threshold_pos", C.c_double),
                ("threshold_neg", C.c_double), ("reset_pending", C.c_int32)]


class ophoto(C.Structure):
    _fields_ = [("electrons_per_radiance", C.c_double), ("dark_electrons", C.c_double),
                ("integration_step", C.c_double), ("shot_noise", C.c_int32)]


PHYSIC_FLOAT_FIELDS = ("threshold_pos", "threshold_neg", "refractory_time", "readout_bandwidth",
                       "readout_latency", "threshold_std", "threshold_min", "wavelength_nm",
                       "quantum_efficiency", "pixel_pitch_um", "fill_factor", "f_number",
                       "lens_transmission", "radiance_scale", "temperature_k", "subthreshold_kappa",
                       "receptor_capacitance_f", "reset_capacitance_f", "dark_current_a",
                       "reset_leakage_a", "circuit_step")
PHYSIC_INT_FIELDS = ("photon_shot_noise", "reset_thermal_noise", "random_seed",
                     "max_events_per_step", "readout_queue_capacity")


class ophysic(C.Structure):
    _fields_ = [(k, C.c_float) for k in PHYSIC_FLOAT_FIELDS] + [(k, C.c_int32) for k in PHYSIC_INT_FIELDS]


class oevent(C.Structure):
    _fields_ = [("timestamp", C.c_double), ("x", C.c_int16), ("y", C.c_int16), ("polarity", C.c_int8),
                ("depth", C.c_float)]


EVENT_DTYPE = np.dtype({"names": ["timestamp", "x", "y", "polarity", "depth"],
                        "formats": ["<f8", "<i2", "<i2", "i1", "<f4"],
                        "offsets": [0, 8, 10, 12, 16], "itemsize": C.sizeof(oevent)})
PACKED_EVENT_DTYPE = np.dtype([("timestamp", "<f8"), ("x", "<i2"), ("y", "<i2"), ("polarity", "i1"),
                               ("depth", "<f4")])  # 17 bytes, include/dvs/dvs_base.hpp:9-18
NODE_DTYPE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left", "<i4"), ("right", "<i4"),
                       ("start", "<i4"), ("count", "<i4")])
STATE_DTYPE = np.dtype({"names": ["receptor_log", "reference_log", "refractory_until", "threshold_pos",
                                  "threshold_neg", "reset_pending"],
                        "formats": ["<f8"] * 5 + ["<i4"], "offsets": [0, 8, 16, 24, 32, 40],
                        "itemsize": C.sizeof(opixel_state)})


def build():
    """Compile the two oracle libraries (and the reference harness when the
    reference checkout is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    # the reference checkout: DVS_REFERENCE_DIR, else the development
    # container's read-only checkout (absent on the GPU machines)
    ref = os.environ.get("DVS_REFERENCE_DIR") or "/root/reference"
    if os.path.isdir(os.path.join(ref, "include", "dvs")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref], check=True)


_LIBS = {}


def _declare(lib):
    lib.oracle_hapke_reflectance.restype = C.c_float
    lib.oracle_hapke_reflectance.argtypes = [C.c_float] * 4 + [C.POINTER(ohapke)]
    lib.oracle_hapke_directional.restype = C.c_float
    lib.oracle_hapke_directional.argtypes = [c_f_p, c_f_p, c_f_p, C.c_float, C.POINTER(ohapke)]
    lib.oracle_set_hapke_form.argtypes = [C.c_int]
    lib.oracle_hapke_form.restype = C.c_int
    lib.oracle_hapke_reflectance_form.restype = C.c_double
    lib.oracle_hapke_reflectance_form.argtypes = [C.c_int] + [C.c_double] * 4 + [C.POINTER(ohapke)]
    lib.oracle_receptor_log_at.restype = C.c_double
    lib.oracle_receptor_log_at.argtypes = [C.c_double] * 4
    lib.oracle_advance_pixel.restype = C.c_int
    lib.oracle_advance_pixel.argtypes = [C.POINTER(opixel_state), C.POINTER(opixel_params), C.c_double,
                                         C.c_double, C.c_double, c_d_p, C.POINTER(C.c_int32), C.c_int]
    lib.oracle_derive_parameters.argtypes = [C.POINTER(ophysic), C.c_int, C.POINTER(opixel_params),
                                             C.POINTER(ophoto)]
    lib.oracle_optical_state_at.argtypes = [C.POINTER(ointerval), C.c_double, C.POINTER(ostate)]
    lib.oracle_sample_pixel.argtypes = [C.POINTER(oscene), C.c_int, C.POINTER(ostate), c_d_p, c_f_p, c_i_p]
    lib.oracle_render.argtypes = [C.POINTER(oscene), C.POINTER(ostate), c_d_p, c_f_p, c_i_p, C.c_int]
    lib.oracle_render_pixels.argtypes = [C.POINTER(oscene), C.POINTER(ostate), C.POINTER(C.c_int32), C.c_int,
                                         c_d_p, c_f_p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.oracle_trace_nearest.restype = C.c_int
    lib.oracle_trace_nearest.argtypes = [C.POINTER(oscene), c_f_p, c_f_p, c_i_p, c_f_p, c_f_p, c_f_p]
    lib.oracle_trace_shadow.restype = C.c_int
    lib.oracle_trace_shadow.argtypes = [C.POINTER(oscene), c_f_p, c_f_p, C.c_int]
    lib.oracle_shadow_origin.argtypes = [C.POINTER(oscene), C.c_int, C.c_float, C.c_float, c_f_p, c_f_p]
    lib.oracle_bvh_build.restype = C.c_int
    lib.oracle_bvh_build.argtypes = [C.c_int, c_f_p, C.c_int, C.POINTER(C.c_uint32), C.c_int, C.c_void_p,
                                     c_i_p]
    lib.oracle_bvh_validate.restype = C.c_int
    lib.oracle_bvh_validate.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.oracle_readout_create.restype = C.c_void_p
    lib.oracle_readout_create.argtypes = [C.c_double, C.c_double, C.c_size_t]
    lib.oracle_readout_destroy.argtypes = [C.c_void_p]
    lib.oracle_readout_submit.restype = C.c_int
    lib.oracle_readout_submit.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_double, C.c_void_p,
                                          C.c_size_t, C.POINTER(C.c_size_t)]
    lib.oracle_readout_drain.restype = C.c_int
    lib.oracle_readout_drain.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]
    lib.oracle_readout_dropped.restype = C.c_size_t
    lib.oracle_readout_dropped.argtypes = [C.c_void_p]
    lib.oracle_readout_peak.restype = C.c_size_t
    lib.oracle_readout_peak.argtypes = [C.c_void_p]
    lib.oracle_sensor_create.restype = C.c_void_p
    lib.oracle_sensor_create.argtypes = [C.POINTER(oscene), C.POINTER(ophysic), C.c_int, C.c_int]
    lib.oracle_sensor_destroy.argtypes = [C.c_void_p]
    lib.oracle_sensor_initialize.restype = C.c_int
    lib.oracle_sensor_initialize.argtypes = [C.c_void_p, C.POINTER(ostate), C.c_double, C.c_int]
    lib.oracle_sensor_process.restype = C.c_int
    lib.oracle_sensor_process.argtypes = [C.c_void_p, C.POINTER(ointerval), C.c_int, C.c_void_p, C.c_size_t,
                                          C.POINTER(C.c_size_t), C.c_int]
    lib.oracle_sensor_drain.restype = C.c_int
    lib.oracle_sensor_drain.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]
    lib.oracle_sensor_states.argtypes = [C.c_void_p, C.c_void_p]
    lib.oracle_sensor_dropped.restype = C.c_size_t
    lib.oracle_sensor_dropped.argtypes = [C.c_void_p]
    lib.oracle_sensor_rays.restype = C.c_uint64
    lib.oracle_sensor_rays.argtypes = [C.c_void_p, C.c_int]
    lib.oracle_set_margin_eta.argtypes = [C.c_double]
    lib.oracle_set_conditioning.argtypes = [C.c_double, C.c_double]
    lib.oracle_render_pixels_margin.argtypes = [C.POINTER(oscene), C.POINTER(ostate), C.POINTER(C.c_int32),
                                                C.c_int, c_d_p, c_f_p, C.POINTER(C.c_uint8), C.c_int]
    lib.oracle_sensor_set_margin.restype = C.c_int
    lib.oracle_sensor_set_margin.argtypes = [C.c_void_p, C.c_double]
    lib.oracle_sensor_margins.argtypes = [C.c_void_p, C.POINTER(C.c_uint8)]
    return lib


# Margin classification defaults (the accuracy statement's exception classes).
# MARGIN_ETA: image-plane displacement of a sub-ray's direction, about ten
# times the FP32 rounding error of a normalized ray direction (a few ulps of
# 6e-8); MARGIN_SHIFT: the log-intensity margin to a threshold, 1e-4.
MARGIN_ETA = 2e-6
MARGIN_SHIFT = 1e-4
MARGIN_OPTICAL, MARGIN_CIRCUIT, MARGIN_DEPTH, MARGIN_CONDITIONING, MARGIN_CRACK = 1, 2, 4, 8, 16


def load(fp64=False):
    """Open liboracle_f32.so (reference arithmetic) or liboracle_f64.so."""
    name = "liboracle_f64.so" if fp64 else "liboracle_f32.so"
    if name not in _LIBS:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            subprocess.run(["make", "-s", "-C", HERE, name], check=True)
        _LIBS[name] = _declare(C.CDLL(path))
    return _LIBS[name]


def reference_path():
    return os.path.join(HERE, "_ref", "libdvsref.so")


def load_reference():
    """The reference's own compiled host code, or None where it was not built."""
    path = reference_path()
    if not os.path.exists(path):
        return None
    if "ref" not in _LIBS:
        lib = C.CDLL(path)
        lib.ref_receptor_log_at.restype = C.c_double
        lib.ref_receptor_log_at.argtypes = [C.c_double] * 4
        lib.ref_advance_pixel.restype = C.c_int
        lib.ref_advance_pixel.argtypes = [c_d_p, c_i_p, c_d_p, C.c_double, C.c_double, C.c_double, c_d_p, c_i_p,
                                          C.c_int]
        lib.ref_hapke_reflectance.restype = C.c_float
        lib.ref_hapke_reflectance.argtypes = [C.c_float] * 4 + [c_f_p]
        lib.ref_hapke_directional.restype = C.c_float
        lib.ref_hapke_directional.argtypes = [c_f_p, c_f_p, c_f_p, C.c_float, c_f_p]
        lib.ref_invert_hapke_if.restype = C.c_float
        lib.ref_invert_hapke_if.argtypes = [C.c_float] * 4 + [c_f_p]
        lib.ref_bvh_build.restype = C.c_int
        lib.ref_bvh_build.argtypes = [C.c_int, c_f_p, C.c_int, C.POINTER(C.c_uint32), C.c_int, C.c_void_p, c_i_p]
        lib.ref_readout_create.restype = C.c_void_p
        lib.ref_readout_create.argtypes = [C.c_double, C.c_double, C.c_size_t]
        lib.ref_readout_destroy.argtypes = [C.c_void_p]
        lib.ref_readout_submit.restype = C.c_size_t
        lib.ref_readout_submit.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_size_t]
        lib.ref_readout_drain.restype = C.c_size_t
        lib.ref_readout_drain.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        lib.ref_readout_dropped.restype = C.c_size_t
        lib.ref_readout_dropped.argtypes = [C.c_void_p]
        lib.ref_readout_peak.restype = C.c_size_t
        lib.ref_readout_peak.argtypes = [C.c_void_p]
        _LIBS["ref"] = lib
    return _LIBS["ref"]


# ---------------------------------------------------------------------------
# helpers


def fptr(a):
    return a.ctypes.data_as(c_f_p)


def dptr(a):
    return a.ctypes.data_as(c_d_p)


def hapke_struct(h):
    """h: mapping with the HapkeConfig keys (include/dvs/scene_types.hpp:204-214)."""
    return ohapke(*[float(h[k]) for k in ("b", "c", "hS", "hC", "thetap", "w", "B_S0", "B_C0", "phi")])


def physic_struct(p):
    s = ophysic()
    for k in PHYSIC_FLOAT_FIELDS:
        setattr(s, k, float(p[k]))
    for k in PHYSIC_INT_FIELDS:
        setattr(s, k, int(p[k]))
    return s


def state_struct(st):
    """st: dict with position, velocity, light, light_rate (3), rotation (4, xyzw), intensity, intensity_rate."""
    s = ostate()
    for k in ("position", "velocity", "light", "light_rate"):
        v = st.get(k, (0.0, 0.0, 0.0))
        setattr(s, k, of3(float(v[0]), float(v[1]), float(v[2])))
    q = st.get("rotation", (0.0, 0.0, 0.0, 1.0))
    for i in range(4):
        s.rotation[i] = float(q[i])
    s.intensity = float(st.get("intensity", 0.0))
    s.intensity_rate = float(st.get("intensity_rate", 0.0))
    return s


def intervals_array(intervals):
    arr = (ointerval * len(intervals))()
    for i, (a, b, t0, t1) in enumerate(intervals):
        arr[i].start = state_struct(a)
        arr[i].end = state_struct(b)
        arr[i].t0 = float(t0)
        arr[i].t1 = float(t1)
    return arr


class OracleScene:
    """Binary-BVH scene built by the oracle's restatement of BVHBuilder::build."""

    def __init__(self, vertices, normals, indices, camera, samples, hapke, albedos=None, max_leaf=64,
                 fp64=False, watertight=False):
        self.lib = load(fp64)
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        self.normals = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3).copy()
        nt = idx.shape[0]
        self.nodes = np.zeros(max(2 * nt, 1), dtype=NODE_DTYPE)
        n_nodes = C.c_int(0)
        self.root = self.lib.oracle_bvh_build(max_leaf, fptr(self.vertices), self.vertices.shape[0],
                                              idx.ctypes.data_as(C.POINTER(C.c_uint32)), nt,
                                              self.nodes.ctypes.data, C.byref(n_nodes))
        self.nodes = self.nodes[: n_nodes.value].copy()
        self.indices = idx
        self.albedos = None if albedos is None else np.ascontiguousarray(albedos, dtype=np.float32)
        self.camera = dict(camera)
        self.samples = int(samples)
        self.hapke = dict(hapke)
        s = oscene()
        s.nodes = self.nodes.ctypes.data
        s.vertices = self.vertices.ctypes.data
        s.normals = self.normals.ctypes.data
        s.indices = self.indices.ctypes.data
        s.albedos = self.albedos.ctypes.data if self.albedos is not None else None
        s.root = self.root
        s.width, s.height = int(camera["width"]), int(camera["height"])
        s.samples = self.samples
        s.fx, s.fy, s.cx, s.cy = (float(camera[k]) for k in ("fx", "fy", "cx", "cy"))
        s.hapke = hapke_struct(hapke)
        s.watertight = 1 if watertight else 0
        self.s = s

    @property
    def pixels(self):
        return self.s.width * self.s.height

    def with_camera(self, camera, samples=None):
        """The same tree and mesh seen by another camera (no rebuild)."""
        v = OracleScene.__new__(OracleScene)
        v.__dict__.update(self.__dict__)
        v.camera = dict(camera)
        v.samples = int(samples if samples is not None else self.samples)
        t = oscene.from_buffer_copy(self.s)
        t.width, t.height = int(camera["width"]), int(camera["height"])
        t.samples = v.samples
        t.fx, t.fy, t.cx, t.cy = (float(camera[k]) for k in ("fx", "fy", "cx", "cy"))
        v.s = t
        return v

    def render(self, pose, nthreads=0):
        n = self.pixels
        rad = np.zeros(n, np.float64)
        dep = np.zeros(n, np.float32)
        val = np.zeros(n, np.int32)
        st = state_struct(pose)
        self.lib.oracle_render(C.byref(self.s), C.byref(st), dptr(rad), fptr(dep),
                               val.ctypes.data_as(c_i_p), nthreads)
        return rad, dep, val

    def render_pixels(self, pose, pixels, nthreads=0):
        px = np.ascontiguousarray(pixels, dtype=np.int32)
        rad = np.zeros(px.size, np.float64)
        dep = np.zeros(px.size, np.float32)
        a, b = C.c_uint64(0), C.c_uint64(0)
        st = state_struct(pose)
        self.lib.oracle_render_pixels(C.byref(self.s), C.byref(st), px.ctypes.data_as(C.POINTER(C.c_int32)),
                                      px.size, dptr(rad), fptr(dep), nthreads, C.byref(a), C.byref(b))
        return rad, dep, a.value, b.value

    def render_margin(self, pose, pixels=None, eta=None, nthreads=0):
        """Radiance, depth and margin flags (MARGIN_OPTICAL) of the given
        pixels (all when None) at one pose."""
        px = np.arange(self.pixels, dtype=np.int32) if pixels is None else np.ascontiguousarray(pixels, np.int32)
        rad = np.zeros(px.size, np.float64)
        dep = np.zeros(px.size, np.float32)
        margin = np.zeros(px.size, np.uint8)
        st = state_struct(pose)
        self.lib.oracle_set_margin_eta(MARGIN_ETA if eta is None else eta)
        try:
            self.lib.oracle_render_pixels_margin(C.byref(self.s), C.byref(st),
                                                 px.ctypes.data_as(C.POINTER(C.c_int32)), px.size, dptr(rad),
                                                 fptr(dep), margin.ctypes.data_as(C.POINTER(C.c_uint8)), nthreads)
        finally:
            self.lib.oracle_set_margin_eta(0.0)
        return rad, dep, margin


class OracleSensor:
    """EventSensor restatement with deterministic physics."""

    def __init__(self, scene, physic, physic_effects=True, aer_delay=True, margin=False, eta=None, shift=None):
        """margin: also classify every pixel's margin class (margins())."""
        self.scene = scene
        self.lib = scene.lib
        self.phys = physic_struct(physic)
        self.h = self.lib.oracle_sensor_create(C.byref(scene.s), C.byref(self.phys), int(physic_effects),
                                               int(aer_delay))
        if not self.h:
            raise ValueError("invalid sensor capacity")
        self.max_events = int(physic["max_events_per_step"])
        self.eta = (MARGIN_ETA if eta is None else eta) if margin else 0.0
        if margin and self.lib.oracle_sensor_set_margin(self.h, MARGIN_SHIFT if shift is None else shift):
            raise ValueError("invalid margin threshold shift")

    def _classified(self, call, *args):
        self.lib.oracle_set_margin_eta(self.eta)
        try:
            return call(*args)
        finally:
            self.lib.oracle_set_margin_eta(0.0)

    def margins(self):
        """Per pixel (row-major): MARGIN_OPTICAL | MARGIN_CIRCUIT | MARGIN_DEPTH flags."""
        out = np.zeros(self.scene.pixels, np.uint8)
        self.lib.oracle_sensor_margins(self.h, out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_sensor_destroy(self.h)
            self.h = None

    def initialize(self, pose, t, nthreads=0):
        st = state_struct(pose)
        r = self._classified(self.lib.oracle_sensor_initialize, self.h, C.byref(st), float(t), nthreads)
        if r:
            raise RuntimeError("oracle initialize failed: %d" % r)

    def process(self, intervals, nthreads=0, capacity=None):
        arr = intervals_array(intervals)
        cap = capacity or (self.scene.pixels * self.max_events + 1_000_000)
        out = np.zeros(cap, dtype=EVENT_DTYPE)
        n = C.c_size_t(0)
        r = self._classified(self.lib.oracle_sensor_process, self.h, arr, len(intervals), out.ctypes.data, cap,
                             C.byref(n), nthreads)
        if r:
            raise RuntimeError({1: "pixel event capacity exceeded; reduce numerical window",
                                2: "invalid optical sample or BVH traversal overflow",
                                3: "sensor intervals must be positive and contiguous"}.get(r, "status %d" % r))
        return out[: n.value].copy()

    def drain(self):
        cap = 2_000_000
        out = np.zeros(cap, dtype=EVENT_DTYPE)
        n = C.c_size_t(0)
        self.lib.oracle_sensor_drain(self.h, out.ctypes.data, cap, C.byref(n))
        return out[: n.value].copy()

    def states(self):
        out = np.zeros(self.scene.pixels, dtype=STATE_DTYPE)
        self.lib.oracle_sensor_states(self.h, out.ctypes.data)
        return out

    def rays(self):
        return self.lib.oracle_sensor_rays(self.h, 0), self.lib.oracle_sensor_rays(self.h, 1)
