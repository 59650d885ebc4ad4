"""The oracle's margin classifier, on the CPU.

The accuracy statement asks for radiance and depth within 1e-5 relative of
the FP64 oracle, with named exception classes instead of a tolerated
fraction.  The FP32 oracle evaluates the reference's arithmetic in the CUDA
kernels' FP32 operation order, so comparing it with the FP64 oracle checks
the classifier without a GPU: every pixel outside 1e-5 must fall in a class
(optical margin, conditioning, crack), and the classes must stay small and
land where the geometry says they should.
"""
import math

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import terrain, trajectory
from oracle import oracle as O

RTOL = 1e-5
HAPKE = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)
CAMERA = dict(width=128, height=96, fx=100.0, fy=100.0, cx=64.0, cy=48.0)
POSE = dict(position=(13.0, -7.0, 700.0), rotation=(0.02, -0.01, 0.3, math.sqrt(1 - 0.02**2 - 0.01**2 - 0.09)),
            light=trajectory.sun_direction(30, 40), intensity=1000)


def classify(V, N, I, camera, ss, pose, watertight=False):
    o32 = O.OracleScene(V, N, I, camera, ss, HAPKE, watertight=watertight)
    o64 = O.OracleScene(V, N, I, camera, ss, HAPKE, fp64=True, watertight=watertight)
    r64, d64, m = o64.render_margin(pose)
    r32, d32, _ = o32.render(pose)
    return r32, d32.astype(np.float64), r64, d64.astype(np.float64), m


def unclassified(r32, d32, r64, d64, m):
    rad_bad = (r64 > 0) & (np.abs(r32 - r64) > RTOL * r64)
    dep_bad = (d64 > 0) & (np.abs(d32 - d64) > RTOL * d64)
    miss_bad = (d64 < 0) != (d32 < 0)
    return np.flatnonzero((rad_bad | dep_bad | miss_bad) & (m == 0))


@pytest.mark.parametrize("ss", [1, 2, 4, 8])
def test_every_fp32_difference_is_classified(ss):
    V, N, I = terrain.terrain_mesh(96, 5)
    r32, d32, r64, d64, m = classify(V, N, I, CAMERA, ss, POSE)
    assert unclassified(r32, d32, r64, d64, m).size == 0
    differs = (r64 > 0) & (np.abs(r32 - r64) > RTOL * r64)
    assert differs.sum() >= 1               # the comparison has teeth on this scene
    assert (m > 0).mean() < 0.06            # the classes stay a small minority


def test_watertight_scene_needs_no_crack_class():
    V, N, I = terrain.terrain_mesh(96, 5)
    r32, d32, r64, d64, m = classify(V, N, I, CAMERA, 4, POSE, watertight=True)
    assert unclassified(r32, d32, r64, d64, m).size == 0
    assert not np.any(m & O.MARGIN_CRACK)


def test_classes_land_on_silhouettes_and_shadow_edges():
    """A half plane seen from above: pixels whose sub-rays straddle the plane's
    border are optical margin pixels, the plane's interior is in no class."""
    V = np.array([[-100, 0, 0], [100, 0, 0], [100, 100, 0], [-100, 100, 0]], np.float32)
    N = np.tile(np.float32([0, 0, 1]), (4, 1))
    I = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    cam = dict(width=64, height=48, fx=40.0, fy=40.0, cx=32.0, cy=24.0)
    pose = dict(position=(0.0, 0.0, 10.0), rotation=(0.0, 0.0, 0.0, 1.0), light=(0.0, 0.0, 1.0), intensity=1000)
    o64 = O.OracleScene(V, N, I, cam, 4, HAPKE, fp64=True)
    # move the border onto a sub-ray: y = 0 is the image row cy, sub-ray centers sit at +-1/8 pixel
    rad, dep, m = o64.render_margin(pose)
    m = m.reshape(48, 64)
    assert np.all(m[30:, :] == 0) and np.all(m[:18, 20:44] == 0)   # the lit interior and the empty sky
    # a border exactly between sub-ray rows: nudge the camera so it passes through one
    pose2 = dict(pose, position=(0.0, 10.0 / 40.0 / 8.0, 10.0))     # 1/8 pixel at 10 m: onto the sub-ray row
    rad2, dep2, m2 = o64.render_margin(pose2)
    m2 = m2.reshape(48, 64)
    assert np.any(m2[23:26, :] & O.MARGIN_OPTICAL)


def test_sensor_margins_flag_near_threshold_circuits():
    """The circuit class: a static pixel whose light ramps to just below a
    threshold is flagged, a pixel that crosses far above it is not."""
    V = np.array([[-100, -100, 0], [100, -100, 0], [100, 100, 0], [-100, 100, 0]], np.float32)
    N = np.tile(np.float32([0, 0, 1]), (4, 1))
    I = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    cam = dict(width=8, height=6, fx=6.0, fy=6.0, cx=4.0, cy=3.0)
    phys = dict(threshold_pos=0.2, threshold_neg=0.2, refractory_time=0, readout_bandwidth=0, readout_latency=0,
                threshold_std=0, threshold_min=0.01, wavelength_nm=550, quantum_efficiency=0.3, pixel_pitch_um=15,
                fill_factor=0.2, f_number=2.0, lens_transmission=0.8, radiance_scale=0.001, temperature_k=300,
                subthreshold_kappa=0.8, receptor_capacitance_f=1e-15, reset_capacitance_f=20e-15,
                dark_current_a=1e-18, reset_leakage_a=0, circuit_step=1e-5, photon_shot_noise=0,
                reset_thermal_noise=0, random_seed=1, max_events_per_step=64, readout_queue_capacity=100000)
    pose = dict(position=(0.0, 0.0, 10.0), rotation=(0.0, 0.0, 0.0, 1.0), light=(0.0, 0.0, 1.0), intensity=1000)

    def run(gain):
        s = O.OracleSensor(O.OracleScene(V, N, I, cam, 1, HAPKE), phys, margin=True)
        s.initialize(pose, 0.0)
        bright = dict(pose, intensity=1000 * gain)
        s.process([(pose, bright, 0.0, 0.05), (bright, bright, 0.05, 0.2)])
        return s.margins()

    # receptor log of a settled pixel follows log(light): exp(0.2) is the ON threshold ratio
    near = run(math.exp(0.2 - 2e-5))   # settles 2e-5 below the threshold: no event, but within 1e-4
    far = run(math.exp(0.5))           # crosses with a wide margin
    assert np.all(near & O.MARGIN_CIRCUIT)
    assert not np.any(far & O.MARGIN_CIRCUIT)
