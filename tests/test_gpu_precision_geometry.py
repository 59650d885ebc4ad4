"""Precision geometry through the C-ABI, flag by flag: FP16 child bounds
quantised outward against a per-node FP32 origin (HALF_BOUNDS: a conservative
filter, the leaves' triangles are still tested in FP32, so the hits are the
reference format's) and the watertight triangle test (WATERTIGHT; Woop,
Benthin and Wald 2013) on stored vertices.

Checked against the oracle (Moller-Trumbore or its watertight restatement:
hits do not depend on the tree, so radiance, depth and events agree as the
reference geometry agrees with the oracle), and against the reference
geometry: the two triangle tests differ only for sub-rays on an edge or a
silhouette, which the accuracy statement counts as a separate margin class.
"""
import math

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import CamRayCaster, DeviceScene, EventSensor, trajectory
from dvsrender4deepspace_gb300.raycast import HALF_BOUNDS, WATERTIGHT
from oracle import oracle as O
from tests.test_gpu_adaptive import same_events
from tests.test_gpu_parity import RTOL, outside_tolerance, pixel_sorted, plane_mesh, rel_err, terrain_scene
from tests.test_oracle_golden import DAVIS, DAVIS_HAPKE, davis_physic
from tests.test_oracle_golden import POSE as PLANE_POSE

pytestmark = pytest.mark.gpu

POSE = dict(position=(13.0, -7.0, 700.0), rotation=(0.02, -0.01, 0.3, math.sqrt(1 - 0.02**2 - 0.01**2 - 0.09)),
            light=trajectory.sun_direction(30, 40), intensity=1000)


BOTH = HALF_BOUNDS | WATERTIGHT


def precision_twin(ss=2, leaf=4, geometry=BOTH, **kw):
    V, N, I, camera, hap, ref = terrain_scene(ss=ss, leaf=leaf, **kw)
    return V, N, I, camera, hap, ref, DeviceScene(V, N, I, camera, ss, hap, leaf_size=leaf, geometry=geometry)


@pytest.mark.parametrize("geometry", [HALF_BOUNDS, WATERTIGHT, BOTH])
def test_precision_scene_info_and_node_bytes(geometry):
    V, N, I, camera, hap, ref, prec = precision_twin(geometry=geometry)
    a, b = ref.info(), prec.info()
    assert a["precision"] == 0 and b["precision"] == geometry
    assert a["nodes"] == b["nodes"] and a["depth"] == b["depth"] and a["leaf_size"] == b["leaf_size"]
    # 144-byte nodes with FP16 bounds; watertight scenes keep three 48-byte
    # copies of each triangle record (one per dominant axis of a ray)
    saved = (256 - 144) * a["nodes"] if geometry & HALF_BOUNDS else 0
    added = 2 * 48 * a["triangles"] if geometry & WATERTIGHT else 0
    assert abs((b["device_bytes"] - a["device_bytes"]) - (added - saved)) <= 512
    with pytest.raises(ValueError):
        DeviceScene(V, N, I, camera, 2, hap, geometry=4)


def test_half_bounds_change_nothing():
    """FP16 child bounds only widen boxes (outward rounding), so every ray
    reaches the same triangles: images and events equal the FP32 tree's."""
    V, N, I, camera, hap, ref, half = precision_twin(geometry=HALF_BOUNDS, leaf=0)
    _, _, _, _, _, ref0, _ = precision_twin(geometry=0, leaf=0)
    for a, b in zip(CamRayCaster(ref0).render_state(POSE), CamRayCaster(half).render_state(POSE)):
        assert float(np.mean(a != b)) < 1e-3 and float(np.mean(rel_err(b, a) > RTOL)) < 1e-3   # exact-t ties only


@pytest.mark.parametrize("leaf,geometry", [(0, BOTH), (8, BOTH), (0, WATERTIGHT), (0, HALF_BOUNDS)])
def test_precision_camera_matches_the_oracle(leaf, geometry):
    """Every pixel outside 1e-5 of either oracle is in a class of the FP64
    oracle's classifier; watertight scenes have no crack class."""
    V, N, I, camera, hap, ref, prec = precision_twin(leaf=leaf, geometry=geometry)
    img, dep = CamRayCaster(prec).render_state(POSE)
    wt = bool(geometry & WATERTIGHT)
    r64, d64, margin = O.OracleScene(V, N, I, camera, 2, hap, fp64=True, watertight=wt).render_margin(POSE)
    r32, d32, v32 = O.OracleScene(V, N, I, camera, 2, hap, watertight=wt).render(POSE)
    assert v32.all()
    for orad, odep in ((r32, d32), (r64, d64)):
        bad = outside_tolerance(img, dep, orad, odep)
        assert not np.any(bad & (margin == 0)), np.flatnonzero(bad & (margin == 0))[:10]
    if wt:
        assert not np.any(margin & O.MARGIN_CRACK)
    assert (margin > 0).mean() < 0.06
    assert (img > 0).mean() > 0.5 and (dep > 0).mean() > 0.8


def test_precision_geometry_differs_from_the_reference_only_at_edges():
    """Hit or shadow decisions change only for sub-rays within rounding of an
    edge or silhouette: few pixels, and the oracle shows the same class."""
    V, N, I, camera, hap, ref, prec = precision_twin()
    img_r, dep_r = CamRayCaster(ref).render_state(POSE)
    img_p, dep_p = CamRayCaster(prec).render_state(POSE)
    # the Moller-Trumbore oracle's classes (crack: within FP32 rounding of an edge)
    _, _, margin = O.OracleScene(V, N, I, camera, 2, hap, fp64=True).render_margin(POSE)
    differ = outside_tolerance(img_p, dep_p, img_r, dep_r)
    assert not np.any(differ & (margin == 0)), np.flatnonzero(differ & (margin == 0))[:10]
    mt = O.OracleScene(V, N, I, camera, 2, hap)
    wt = O.OracleScene(V, N, I, camera, 2, hap, watertight=True)
    a, b = wt.render(POSE), mt.render(POSE)
    assert not np.any(outside_tolerance(a[0], a[1], b[0], b[1]) & (margin == 0))


def test_precision_subray_and_temporal_packets_agree():
    """Both trace kernels of the precision format (sub-ray packets for one
    pose, temporal packets for nine) give bit-identical radiance."""
    V, N, I, camera, hap, ref, prec = precision_twin(ss=8)
    cam = CamRayCaster(prec)
    single, _ = cam.render_state(POSE)
    w = np.zeros(9, np.float32)
    w[4] = 1
    assert np.array_equal(cam.render_blur([POSE] * 9, w), single)
    assert (single > 0).mean() > 0.5


def test_precision_sensor_matches_the_watertight_oracle_on_moving_terrain():
    cam = dict(width=64, height=48, fx=60.0, fy=60.0, cx=32.0, cy=24.0)
    V, N, I, camera, hap, ref, prec = precision_twin(n=80, seed=9, camera=cam, ss=1)
    traj = trajectory.StraightPass((0.0, 0.0, 400.0), (50.0, 0.0, 0.0), trajectory.sun_direction(30), 1000.0)
    phys = davis_physic(threshold_std=0, photon_shot_noise=0, max_events_per_step=64, readout_bandwidth=0,
                        readout_latency=0, threshold_pos=0.05, threshold_neg=0.05, refractory_time=5e-5)
    s = EventSensor(prec, phys)
    s.initialize(traj.state(0.0), 0.0)
    ors = O.OracleSensor(O.OracleScene(V, N, I, camera, 1, hap, watertight=True), phys, margin=True)
    ors.initialize(traj.state(0.0), 0.0)
    gpu, ora = [], []
    t = 0.0
    for batch in range(3):
        ivs = trajectory.horizons(traj, t, 1e-4, 20)
        if batch == 1:
            a, b = traj.state(ivs[-1][3]), traj.state(ivs[-1][3] + 2e-3)
            ivs.append((dict(a, intensity_rate=8e6), dict(b, intensity_rate=-8e6), ivs[-1][3], ivs[-1][3] + 2e-3))
        t = ivs[-1][3]
        gpu.append(s.process_many(ivs))
        ora.append(ors.process(ivs))
    gpu.append(s.drain())
    ora.append(ors.drain())
    g, o = np.concatenate(gpu), np.concatenate(ora)
    assert len(o) > 50

    def per_pixel(ev):
        d = {}
        for e in ev:
            d.setdefault((int(e["x"]), int(e["y"])), []).append((float(e["timestamp"]), int(e["polarity"]),
                                                                 float(e["depth"])))
        return d
    pg, po = per_pixel(g), per_pixel(o)
    margins = ors.margins()
    unclassified, worst, worst_depth = 0, 0.0, 0.0
    for key in set(pg) | set(po):
        a, b = pg.get(key, []), po.get(key, [])
        flagged = margins[key[1] * cam["width"] + key[0]] != 0
        if [p for _, p, _ in a] != [p for _, p, _ in b]:
            unclassified += 0 if flagged else 1
            continue
        if flagged:
            continue
        for (ta, _, da), (tb, _, db) in zip(a, b):
            worst = max(worst, abs(ta - tb))
            worst_depth = max(worst_depth, abs(da - db) / max(abs(db), 1e-30))
    assert unclassified == 0
    assert (margins != 0).mean() < 0.05
    assert worst < 1e-6 and worst_depth < RTOL


def test_precision_adaptive_discontinuity_matches_native():
    """The adaptive solver's probe and exact-cell kernels in the precision
    format (the reference's discontinuity check, tests/test_sensor.cu:96-159):
    an intensity step is resolved with exactly traced cells, giving the
    native events."""
    V, N, I = plane_mesh()
    scene = DeviceScene(V, N, I, DAVIS, 1, DAVIS_HAPKE, geometry=BOTH)
    phys = davis_physic(threshold_std=0, photon_shot_noise=0, max_events_per_step=64, readout_bandwidth=0,
                        readout_latency=0, random_seed=42, circuit_step=1e-6)
    native, adaptive = EventSensor(scene, phys), EventSensor(scene, phys)
    native.initialize(PLANE_POSE, 0)
    adaptive.initialize(PLANE_POSE, 0)
    bright = dict(PLANE_POSE, intensity=2000)
    ivs = [(PLANE_POSE, PLANE_POSE, 0, .001), (bright, bright, .001, .002)]
    exact = native.process_many(ivs)
    cached = adaptive.process_adaptive(ivs, 1e-4)
    st = adaptive.refinement_statistics()
    assert st["native_cell_queries"] > 0 and st["fallback_pixels"] == 0
    assert len(exact) > 100
    same_events(pixel_sorted(exact), pixel_sorted(cached), tol=2e-12)
