"""bin/dvs and bin/cam end to end on the GPU: a synthetic scene bundle and
config in, events.bin / events.h5 / images / depth out.  The app's events
must equal, event for event, what the library API produces from the same
trajectory (dvs_trajectory_* through the Python package) with the app's
horizon batching (apps/main_dvs.cpp:72-126); the HDF5 file must carry the
same events in microseconds; bin/cam's depth must equal a direct render."""
import math
import os
import subprocess

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import DeviceScene, EventSensor, inputs, terrain, trajectory
from dvsrender4deepspace_gb300 import build as B
from dvsrender4deepspace_gb300.raycast import CamRayCaster
from tests.test_apps_host import read_hdf5, read_png, read_tiff_float

pytestmark = pytest.mark.gpu

CAMERA = dict(width=64, height=48, fx=60.0, fy=60.0, cx=32.0, cy=24.0)
PHYSIC = dict(threshold_pos=0.2, threshold_neg=0.2, threshold_std=0.03, threshold_min=0.01, refractory_time=200e-6,
              readout_bandwidth=5e6, readout_latency=18e-9, photon_shot_noise=1, random_seed=7,
              max_events_per_step=16, circuit_step=1e-6)
SCENE = dict(frame_count=3, fps=100.0, imu_fps=1000.0, cam_fps=100.0, time_resolution=1e-5, supersample_factor=2,
             blur_resolution=1e-3)
HAPKE = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)
EVENT_BIN = np.dtype([("t", "<f4"), ("x", "<i2"), ("y", "<i2"), ("p", "i1"), ("d", "<f4")])


@pytest.fixture(scope="module")
def bundle(tmp_path_factory):
    B.build()
    d = tmp_path_factory.mktemp("bundle")
    V, N, I = terrain.terrain_mesh(96, 11)
    light = trajectory.sun_direction(30, 40)
    eye = np.eye(3, dtype=np.float32)  # Blender camera: -Z looks down
    t = np.array([0.0, 0.01, 0.02])
    fr = inputs.frames_array(t, [(-100 + 500 * s, 20 * s, 400) for s in t], [eye] * 3, [light] * 3, [1000.0] * 3)
    inputs.write_bundle(d / "scene", V, N, I, fr)
    inputs.write_config(d / "config.yaml", CAMERA, PHYSIC, SCENE, HAPKE)
    return d


def run_app(name, bundle, out, *extra):
    r = subprocess.run([os.path.join(B.BIN, name), "--scene_dir", str(bundle / "scene"), "--config",
                        str(bundle / "config.yaml"), "--output", str(out), *extra], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr + r.stdout
    return r.stdout


def api_events(bundle, geometry=0, circuit="fp64"):
    """The same run through the library API with the app's batches."""
    cfg = inputs.load_config(bundle / "config.yaml")
    frames = inputs.load_frames(bundle / "scene")
    V, N, I = inputs.load_mesh(bundle / "scene")
    traj = inputs.Trajectory(frames, cfg["scene"])
    scene = DeviceScene(V, N, I, cfg["camera"], cfg["scene"]["supersample_factor"], cfg["hapke"], geometry=geometry)
    sensor = EventSensor(scene, cfg["physic"], circuit_precision=circuit)
    (state0, t0), batches, end_time = inputs.app_intervals(traj, frames, cfg["scene"], cfg["physic"])
    sensor.initialize(state0, t0)
    evs = [sensor.process_many(b) for b in batches]
    evs.append(sensor.drain())
    return np.concatenate(evs), end_time


def test_dvs_app_events_match_the_library(bundle, tmp_path):
    out = run_app("dvs", bundle, tmp_path / "bin", "--event_format", "bin")
    assert "Finished. Wrote" in out
    got = np.fromfile(tmp_path / "bin" / "events.bin", EVENT_BIN)
    want, end_time = api_events(bundle)
    assert len(want) > 50, len(want)
    assert len(got) == len(want)
    assert np.array_equal(got["t"], want["timestamp"].astype(np.float32))
    assert np.array_equal(got["x"], want["x"]) and np.array_equal(got["y"], want["y"])
    assert np.array_equal(got["p"], want["polarity"]) and np.array_equal(got["d"], want["depth"])
    for f in ("sensor_model.txt", "sensor_config.yaml", "camera_used.yaml", "source_config.yaml"):
        assert (tmp_path / "bin" / f).exists(), f
    meta = (tmp_path / "bin" / "sensor_model.txt").read_text()
    assert "optical_sampling=midpoint_rays_within_circuit_cells" in meta and "random_seed=7" in meta

    # events.h5 of the same run: microsecond timestamps, millisecond index
    run_app("dvs", bundle, tmp_path / "h5", "--event_format", "hdf5", "--solver", "native")
    h5 = read_hdf5(tmp_path / "h5" / "events.h5")
    order = np.argsort(want["timestamp"], kind="stable")
    assert np.array_equal(h5["t"], np.round(want["timestamp"][order] * 1e6).astype(np.int64))
    assert np.array_equal(h5["x"], want["x"][order]) and np.array_equal(h5["p"], want["polarity"][order])
    idx = h5["ms_to_idx"]
    end_ms = int(round(max(end_time, float(want["timestamp"].max())) * 1000))
    assert len(idx) == end_ms + 1
    ms = h5["t"] // 1000
    for m in range(len(idx)):
        assert idx[m] == np.searchsorted(ms, m, side="left")


def test_dvs_app_precision_flags_match_the_library(bundle, tmp_path):
    """bin/dvs --bvh / --circuit (GB300 additions) run the library's formats."""
    run_app("dvs", bundle, tmp_path, "--event_format", "bin", "--bvh", "half+watertight", "--circuit", "fp32-philox")
    got = np.fromfile(tmp_path / "events.bin", EVENT_BIN)
    want, _ = api_events(bundle, geometry=3, circuit="fp32-philox")
    assert len(want) > 50 and len(got) == len(want)
    assert np.array_equal(got["t"], want["timestamp"].astype(np.float32))
    assert np.array_equal(got["x"], want["x"]) and np.array_equal(got["p"], want["polarity"])


def test_dvs_app_adaptive_hdf5(bundle, tmp_path):
    out = run_app("dvs", bundle, tmp_path, "--event_format", "hdf5")  # auto selects adaptive optics
    assert "Finished. Wrote" in out
    meta = (tmp_path / "sensor_model.txt").read_text()
    assert "optical_sampling=adaptive_direct_ray_nodes_with_native_cell_fallback" in meta
    assert "optical_cache_capacity=" in meta and "optical_cache_capacity=0" not in meta
    h5 = read_hdf5(tmp_path / "events.h5")
    assert len(h5["t"]) > 0 and (np.diff(h5["t"]) >= 0).all()
    assert (h5["x"] >= 0).all() and (h5["x"] < CAMERA["width"]).all() and set(np.unique(h5["p"])) <= {0, 1}


def test_cam_blur_app(bundle, tmp_path):
    out = run_app("cam_blur", bundle, tmp_path)
    assert "Wrote 2 images" in out
    names = sorted(os.listdir(tmp_path / "blur_images"))
    assert names == ["0.000000.png", "0.010000.png"]
    img = read_png(tmp_path / "blur_images" / names[1])
    assert img.shape == (CAMERA["height"], CAMERA["width"]) and img.max() > 0


def test_cam_app_matches_direct_render(bundle, tmp_path):
    out = run_app("cam", bundle, tmp_path)
    n = math.ceil(0.02 * SCENE["cam_fps"])
    assert "Wrote %d images" % n in out
    pngs = sorted(os.listdir(tmp_path / "images"))
    tifs = sorted(os.listdir(tmp_path / "depth"))
    assert pngs == ["0.000000.png", "0.010000.png"] and tifs == ["0.000000.tif", "0.010000.tif"]
    cfg = inputs.load_config(bundle / "config.yaml")
    frames = inputs.load_frames(bundle / "scene")
    V, N, I = inputs.load_mesh(bundle / "scene")
    traj = inputs.Trajectory(frames, cfg["scene"])
    scene = DeviceScene(V, N, I, cfg["camera"], cfg["scene"]["supersample_factor"], cfg["hapke"])
    st, R = traj.evaluate(np.float32(0.01))
    img, dep = CamRayCaster(scene).render_state(st)
    depth = read_tiff_float(tmp_path / "depth" / "0.010000.tif").ravel()
    rel = np.abs(depth - dep) / np.maximum(np.abs(dep), 1e-30)
    assert (dep > 0).mean() > 0.9 and float(np.mean(rel > 1e-5)) < 0.01
    png = read_png(tmp_path / "images" / "0.010000.png")
    assert png.shape == (CAMERA["height"], CAMERA["width"]) and png.max() > 0
