"""Host inputs of bin/dvs and bin/cam from Python: the YAML config, scene
bundles (mesh_*.bin + frames.bin) and the continuous trajectory, all through
the library's C-ABI (dvs_config_load, dvs_frames_load, dvs_trajectory_*), so
Python drives exactly the trajectory the apps use.

The bundle layout is the reference's (src/scene_data.cpp:93-193):
mesh_vertices.bin / mesh_normals.bin (N x 3 float32), mesh_indices.bin
(M x 3 uint32), frames.bin (24 float32 per frame: seconds, camera origin,
row-major 4x4 camera-to-world, light direction, light intensity).
"""
import ctypes as C
import math
import os

import numpy as np

from . import _capi
from ._capi import FRAME_DTYPE, INTERVAL_DTYPE, STATE_DTYPE, check

SCENE_KEYS = ("frame_count", "fps", "imu_fps", "cam_fps", "time_resolution", "blur_resolution",
              "supersample_factor", "translation", "rotation")


def _struct_dict(s):
    out = {}
    for k, _ in s._fields_:
        v = getattr(s, k)
        out[k] = list(v) if isinstance(v, C.Array) else v
    return out


def load_config(path):
    """Config(path) (src/scene_types.cpp:170-345): dict of camera, physic,
    hapke and scene blocks; ValueError with the reference's message."""
    cam, phys, hap, scene = _capi.Camera(), _capi.Physic(), _capi.Hapke(), _capi.SceneConfig()
    check(_capi.load().dvs_config_load(os.fsencode(path), C.byref(cam), C.byref(phys), C.byref(hap),
                                       C.byref(scene)))
    return {"camera": _struct_dict(cam), "physic": _struct_dict(phys), "hapke": _struct_dict(hap),
            "scene": _struct_dict(scene)}


def write_config(path, camera, physic, scene, hapke):
    """Writes a config file in the reference's YAML layout."""
    lines = ["intrinsic:"] + ["  %s: %r" % (k, camera[k]) for k in ("width", "height", "fx", "fy", "cx", "cy")]
    lines += ["physic:"] + ["  %s: %r" % (k, v) for k, v in physic.items()]
    sc = dict(scene)
    lines += ["scene:"]
    for k in ("frame_count", "fps", "imu_fps", "cam_fps", "time_resolution", "supersample_factor", "blur_resolution"):
        lines.append("  %s: %r" % (k, sc[k]))
    for k in ("translation", "rotation"):
        if k in sc:
            lines.append("  %s: [%s]" % (k, ", ".join(repr(float(v)) for v in sc[k])))
    lines += ["hapke:"] + ["  %s: %r" % (k, v) for k, v in hapke.items()]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def frames_array(times, origins, worlds, lights, intensities):
    """FRAME_DTYPE records from per-frame seconds, origins (3), row-major
    camera-to-world rotations (3x3), light directions (3) and intensities."""
    n = len(times)
    fr = np.zeros(n, FRAME_DTYPE)
    fr["frame_index"] = np.arange(n)
    fr["timestamp_seconds"] = np.asarray(times, np.float64)
    fr["camera_origin"] = np.asarray(origins, np.float32)
    fr["camera_world"] = np.asarray(worlds, np.float32).reshape(n, 9)
    fr["light_dir"] = np.asarray(lights, np.float32)
    fr["light_intensity"] = np.asarray(intensities, np.float32)
    return fr


def write_bundle(directory, vertices, normals, indices, frames):
    """Writes a scene bundle directory (mesh_*.bin + frames.bin)."""
    os.makedirs(directory, exist_ok=True)
    np.ascontiguousarray(vertices, np.float32).tofile(os.path.join(directory, "mesh_vertices.bin"))
    np.ascontiguousarray(normals, np.float32).tofile(os.path.join(directory, "mesh_normals.bin"))
    np.ascontiguousarray(indices, np.uint32).tofile(os.path.join(directory, "mesh_indices.bin"))
    n = len(frames)
    raw = np.zeros((n, 24), np.float32)
    raw[:, 0] = frames["timestamp_seconds"]
    raw[:, 1:4] = frames["camera_origin"]
    m4 = np.zeros((n, 4, 4), np.float32)
    m4[:, :3, :3] = frames["camera_world"].reshape(n, 3, 3)
    m4[:, 3, 3] = 1
    raw[:, 4:20] = m4.reshape(n, 16)
    raw[:, 20:23] = frames["light_dir"]
    raw[:, 23] = frames["light_intensity"]
    raw.tofile(os.path.join(directory, "frames.bin"))


def load_frames(directory):
    """frames.bin of a bundle as FRAME_DTYPE records."""
    n = C.c_size_t()
    lib = _capi.load()
    check(lib.dvs_frames_load(os.fsencode(directory), None, 0, C.byref(n)))
    out = np.zeros(n.value, FRAME_DTYPE)
    if n.value:
        check(lib.dvs_frames_load(os.fsencode(directory), out.ctypes.data, n.value, C.byref(n)))
    return out


def load_mesh(directory):
    v = np.fromfile(os.path.join(directory, "mesh_vertices.bin"), np.float32).reshape(-1, 3)
    nrm = np.fromfile(os.path.join(directory, "mesh_normals.bin"), np.float32).reshape(-1, 3)
    idx = np.fromfile(os.path.join(directory, "mesh_indices.bin"), np.uint32).reshape(-1, 3)
    return v, nrm, idx


class Trajectory:
    """CameraTrajectory(frames, scene config) (include/dvs/trajectory.hpp)."""

    def __init__(self, frames, scene):
        frames = np.ascontiguousarray(frames, FRAME_DTYPE)
        sc = _capi.SceneConfig()
        for k in SCENE_KEYS:
            v = scene.get(k, [0.0, 0.0, 0.0] if k in ("translation", "rotation") else 0)
            if k in ("translation", "rotation"):
                getattr(sc, k)[:] = [float(x) for x in v]
            else:
                setattr(sc, k, v)
        h = C.c_void_p()
        self._frames = frames
        check(_capi.load().dvs_trajectory_create(frames.ctypes.data if len(frames) else None, len(frames),
                                                 C.byref(sc), C.byref(h)))
        self.handle = h

    def range(self):
        a, b = C.c_float(), C.c_float()
        check(_capi.load().dvs_trajectory_range(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    def evaluate(self, t):
        """(OpticalState record, row-major 3x3 orientation) at float32 time t."""
        st = np.zeros(1, STATE_DTYPE)
        m = (C.c_float * 9)()
        check(_capi.load().dvs_trajectory_evaluate(self.handle, C.c_float(t), st.ctypes.data, m))
        return st[0], np.array(m[:], np.float32).reshape(3, 3)

    def close(self):
        if getattr(self, "handle", None):
            _capi.load().dvs_trajectory_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def native_batch(physic, time_resolution, adaptive=False):
    """Horizons per launch of bin/dvs (apps/main_dvs.cpp:94-98)."""
    batch = 200 if adaptive else 64
    if physic["refractory_time"] <= 0:
        return 1
    cap = max(1.0, (physic["max_events_per_step"] - 2) * float(np.float32(physic["refractory_time"])) /
              float(np.float32(time_resolution)))
    return max(1, min(batch, int(cap)))


def app_intervals(traj, frames, scene, physic):
    """The horizon batches bin/dvs feeds the native solver: (start state, t0)
    and a list of interval arrays, built with the app's float/double time
    arithmetic (apps/main_dvs.cpp:72-117)."""
    f32 = np.float32
    fps = float(f32(scene["fps"]))
    count = min(len(frames), int(scene["frame_count"]))

    def frame_time(f):
        ts = float(f["timestamp_seconds"])
        return f["frame_index"] / fps if math.isnan(ts) else ts

    end_time = float(f32(frame_time(frames[count - 1])))
    start_time = float(f32(frame_time(frames[0])))
    dt = float(f32(scene["time_resolution"]))
    total = int(math.ceil((end_time - start_time) / dt))
    batch = native_batch(physic, scene["time_resolution"])
    prev_state, _ = traj.evaluate(start_time)
    prev_t = start_time
    init = (prev_state.copy(), start_time)
    batches, step = [], 0
    while step < total:
        ivs = []
        for _ in range(batch):
            if step >= total:
                break
            step += 1
            t = min(end_time, start_time + step * dt)
            if t <= prev_t:
                break
            cur, _ = traj.evaluate(float(f32(t)))
            iv = np.zeros((), INTERVAL_DTYPE)
            iv["start"], iv["end"], iv["t0"], iv["t1"] = prev_state, cur, prev_t, t
            ivs.append(iv)
            prev_state, prev_t = cur, t
        if not ivs:
            break
        batches.append(np.array(ivs, INTERVAL_DTYPE))
    return init, batches, end_time
