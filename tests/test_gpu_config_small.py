"""The small config end to end: bin/dvs over its whole horizon loop
(apps/main_dvs.cpp:92-120) against the oracle sensor.

Config: a seeded 256x256-vertex fBm + crater terrain (130,050 triangles,
10 m spacing), the DAVIS346 camera at 346x260 (fx=fy=300, cx=173, cy=130)
on a 1 km nadir pass at 50 m/s, 50 frames at 100 fps (0.49 s, 10 us horizons,
1 us circuit cells: 49,000 horizons in 766 app batches), sun 30 degrees above
the horizon, the config's Hapke parameters, thresholds 0.2, one sub-ray, the
reference's FP64 circuit (the small config's plain method).  Deterministic
physics (no shot noise, mismatch or reset noise: the oracle has no device
random stream) and no AER bus (a bus couples every pixel's delivery times, so
a cropped oracle could not reproduce them); light intensity 1000, the
reference tests' value (the config's 1.0 is photon-starved and gives almost
no events).

bin/dvs runs the full sensor on the GPU.  The oracle runs the two 16x12 crops
of the same camera where the GPU's events are busiest (the crop's sub-rays
are the full camera's, bit for bit: the intrinsics are integers) through the
app's own batches.  The oracle here is the FP32 one -- the kernels' ray,
triangle and Hapke arithmetic in the same operation order, the FP64 circuit
-- so device and oracle differ only by the ulps of the transcendental
functions.  The FP64-geometry oracle is the wrong counterpart for a run this
long and slow: the ground moves seven pixels in 0.49 s, so a pixel's log
intensity crosses a threshold at a few units per second and a crossing time
moves by (radiance error) / (slope), which FP32 ray conditioning (~1e-6)
turns into microseconds; the FP64 classifier checks live in the light-pulse
tests and the bench's precision report.  The classifier's class here is the
circuit margin (thresholds moved by +-1e-4 change the polarity sequence).
Every other crop pixel's polarity sequence must equal the oracle's, with
timestamps within 1 us.
"""
import os
import subprocess

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import inputs, terrain, trajectory
from dvsrender4deepspace_gb300 import build as B
from oracle import oracle as O
from tests.test_gpu_apps import EVENT_BIN

pytestmark = pytest.mark.gpu

CAMERA = dict(width=346, height=260, fx=300.0, fy=300.0, cx=173.0, cy=130.0)
HAPKE = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)
PHYSIC = dict(threshold_pos=0.2, threshold_neg=0.2, threshold_std=0.0, threshold_min=0.01, refractory_time=200e-6,
              wavelength_nm=550, quantum_efficiency=0.3, pixel_pitch_um=15, fill_factor=0.2, f_number=2.0,
              lens_transmission=0.8, radiance_scale=0.001, temperature_k=300, subthreshold_kappa=0.8,
              receptor_capacitance_f=1e-15, reset_capacitance_f=20e-15, dark_current_a=1e-18, reset_leakage_a=0,
              photon_shot_noise=0, reset_thermal_noise=0, circuit_step=1e-6, readout_bandwidth=0.0,
              readout_latency=0.0, readout_queue_capacity=1000000, max_events_per_step=16, random_seed=114514)
SCENE = dict(frame_count=50, fps=100.0, imu_fps=1000.0, cam_fps=100.0, time_resolution=1e-5, supersample_factor=1,
             blur_resolution=1e-3)
CROP_W, CROP_H = 16, 12


def busiest_crops(ev, width, height, n=2):
    """(x0, y0) of the n non-overlapping 16x12 windows (on a 4-pixel grid)
    with the most pixels that have events.  A 1 km nadir pass at 50 m/s moves
    the ground about seven pixels in 0.49 s, so events gather along crater
    rims and shadow edges; fixed windows can hold none.  Every pixel of a
    chosen window is compared, with or without events."""
    active = np.zeros((height + 1, width + 1))
    active[1:, 1:][ev["y"], ev["x"]] = 1
    S = active.cumsum(0).cumsum(1)
    cands = []
    for y0 in range(0, height - CROP_H + 1, 4):
        for x0 in range(0, width - CROP_W + 1, 4):
            c = S[y0 + CROP_H, x0 + CROP_W] - S[y0, x0 + CROP_W] - S[y0 + CROP_H, x0] + S[y0, x0]
            cands.append((c, x0, y0))
    cands.sort(key=lambda c: -c[0])
    chosen = []
    for c, x0, y0 in cands:
        if all(abs(x0 - a) >= CROP_W or abs(y0 - b) >= CROP_H for a, b in chosen):
            chosen.append((x0, y0))
        if len(chosen) == n:
            break
    return chosen


def as_state(rec):
    return {k: tuple(float(v) for v in np.atleast_1d(rec[k])) if k not in ("intensity", "intensity_rate")
            else float(rec[k]) for k in rec.dtype.names}


def oracle_intervals(batch):
    return [(as_state(iv["start"]), as_state(iv["end"]), float(iv["t0"]), float(iv["t1"])) for iv in batch]


def test_small_config_through_bin_dvs_matches_the_oracle(tmp_path):
    B.build()
    V, N, I = terrain.terrain_mesh(256, 20260001)
    assert len(I) == 130050
    light = trajectory.sun_direction(30, 0)
    t = np.arange(50) / 100.0
    fr = inputs.frames_array(t, [(50.0 * s, 0.0, 1000.0) for s in t], [np.eye(3, dtype=np.float32)] * 50,
                             [light] * 50, [1000.0] * 50)
    inputs.write_bundle(tmp_path / "scene", V, N, I, fr)
    inputs.write_config(tmp_path / "config.yaml", CAMERA, PHYSIC, SCENE, HAPKE)
    out = tmp_path / "out"
    r = subprocess.run([os.path.join(B.BIN, "dvs"), "--scene_dir", str(tmp_path / "scene"), "--config",
                        str(tmp_path / "config.yaml"), "--output", str(out), "--event_format", "bin",
                        "--circuit", "fp64"], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stderr + r.stdout
    gpu = np.fromfile(out / "events.bin", EVENT_BIN)
    assert len(gpu) > 1000

    # the oracle through the app's own batches (float time arithmetic of apps/main_dvs.cpp:72-117)
    cfg = inputs.load_config(tmp_path / "config.yaml")
    frames = inputs.load_frames(tmp_path / "scene")
    traj = inputs.Trajectory(frames, cfg["scene"])
    (state0, t0), batches, end_time = inputs.app_intervals(traj, frames, cfg["scene"], cfg["physic"])
    assert len(batches) > 700
    o32 = O.OracleScene(V, N, I, CAMERA, 1, HAPKE)
    ivs = [oracle_intervals(b) for b in batches]
    total_pixels, total_margin, compared = 0, 0, 0
    for x0, y0 in busiest_crops(gpu, CAMERA["width"], CAMERA["height"]):
        crop = dict(CAMERA, width=16, height=12, cx=CAMERA["cx"] - x0, cy=CAMERA["cy"] - y0)
        ors = O.OracleSensor(o32.with_camera(crop), cfg["physic"], margin=True, eta=0.0)
        ors.initialize(as_state(state0), t0)
        oev = np.concatenate([ors.process(b) for b in ivs] + [ors.drain()])
        margins = ors.margins()
        mine = gpu[(gpu["x"] >= x0) & (gpu["x"] < x0 + 16) & (gpu["y"] >= y0) & (gpu["y"] < y0 + 12)]
        for px in range(16 * 12):
            x, y = x0 + px % 16, y0 + px // 16
            g = mine[(mine["x"] == x) & (mine["y"] == y)]
            o = oev[(oev["x"] == px % 16) & (oev["y"] == px // 16)]
            g, o = g[np.argsort(g["t"], kind="stable")], o[np.argsort(o["timestamp"], kind="stable")]
            total_pixels += 1
            if margins[px]:
                total_margin += 1
                continue
            assert list(g["p"]) == list(o["polarity"]), (x, y)
            if len(o):
                compared += 1
                # events.bin stores float32 seconds (dvs_writer.hpp:44-55): 6e-8 s at 0.5 s
                assert np.max(np.abs(g["t"].astype(np.float64) - o["timestamp"])) < 1e-6, (x, y)
    assert compared > 20, (compared, total_margin, total_pixels)
    assert total_margin < 0.2 * total_pixels, (compared, total_margin, total_pixels)
