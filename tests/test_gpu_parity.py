"""GPU parity: the CUDA path through the C-ABI against the CPU oracle, plus
the known answers of the reference's tests/test_render.cu and
tests/test_sensor.cu at the reference's own sizes.

Tolerances (the workload's accuracy statement): radiance and depth within
1e-5 relative of the oracle; per-pixel event counts and polarity sequences
identical except pixels within 1e-4 of a threshold (counted, bounded here
by a small fraction); timestamps within 1 us.
"""
import math

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import (CamRayCaster, CapacityError, DeviceScene, EventSensor, terrain,
                                       trajectory)
from oracle import oracle as O
from tests.test_oracle_golden import DAVIS, DAVIS_HAPKE, POSE, davis_physic

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def half_plane_mesh():
    V = np.array([[-100, 0, 0], [100, 0, 0], [100, 100, 0], [-100, 100, 0]], np.float32)
    N = np.tile(np.float32([0, 0, 1]), (4, 1))
    I = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    return V, N, I


def plane_mesh():
    V = np.array([[-100, -100, 0], [100, -100, 0], [100, 100, 0], [-100, 100, 0]], np.float32)
    N = np.tile(np.float32([0, 0, 1]), (4, 1))
    I = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    return V, N, I


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)


# ---- camera path (tests/test_render.cu:37-79) --------------------------------------------

def test_cam_half_plane_matches_oracle_and_reference_facts():
    V, N, I = half_plane_mesh()
    ss = 16
    scene = DeviceScene(V, N, I, DAVIS, ss, DAVIS_HAPKE)
    cam = CamRayCaster(scene)
    pose = dict(position=(0, 0, 10), rotation=(0, 0, 0, 1), light=(0, 0, 1), intensity=1000)
    img, dep = cam.render_state(pose)
    img2, dep2 = cam.render_state(pose)
    assert np.array_equal(img, img2) and np.array_equal(dep, dep2)  # repeat render identical
    osc = O.OracleScene(V, N, I, DAVIS, ss, DAVIS_HAPKE)
    orad, odep, oval = osc.render(pose)
    assert oval.all()
    hit = orad > 0
    assert np.array_equal(img > 0, hit)
    assert rel_err(img[hit], orad[hit].astype(np.float32)).max() < RTOL
    assert np.array_equal(dep == -1, odep == -1)
    d = odep != -1
    assert rel_err(dep[d], odep[d]).max() < RTOL
    W, H = DAVIS["width"], DAVIS["height"]
    col = int(DAVIS["cx"])
    assert img[col] > 0 and dep[col] > 0                                  # +world Y is the upper image
    assert img[(H - 1) * W + col] == 0 and dep[(H - 1) * W + col] == -1   # miss: 0 and -1
    row = round(DAVIS["cy"])
    rng_, hits = 0.0, 0
    for sy in range(ss):
        for sx in range(ss):
            px = (col + (sx + .5) / ss - .5 - DAVIS["cx"]) / DAVIS["fx"]
            py = (row + (sy + .5) / ss - .5 - DAVIS["cy"]) / DAVIS["fy"]
            if py <= 0:
                rng_ += 10 * math.sqrt(1 + px * px + py * py)
                hits += 1
    assert 0 < hits < ss * ss
    assert abs(dep[row * W + col] - rng_ / hits) < 1e-5                   # depth averages hit rays only


def terrain_scene(n=96, seed=5, camera=None, ss=2, fp64_oracle=False, leaf=4):
    V, N, I = terrain.terrain_mesh(n, seed)
    camera = camera or dict(width=128, height=96, fx=100.0, fy=100.0, cx=64.0, cy=48.0)
    hap = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)
    return (V, N, I, camera, hap, DeviceScene(V, N, I, camera, ss, hap, leaf_size=leaf))


def outside_tolerance(img, dep, orad, odep):
    """Pixels whose radiance or depth is outside RTOL of the oracle's, or whose hit/miss differs."""
    img, dep = np.asarray(img, np.float64), np.asarray(dep, np.float64)
    orad, odep = np.asarray(orad, np.float64), np.asarray(odep, np.float64)
    rad = (orad > 0) & (np.abs(img - orad) > RTOL * orad)
    dpt = (odep > 0) & (np.abs(dep - odep) > RTOL * odep)
    return rad | dpt | ((odep < 0) != (dep < 0)) | ((orad == 0) != (img == 0))


@pytest.mark.parametrize("ss", [2, 8])
def test_cam_terrain_matches_oracle(ss):
    """Radiance and depth within 1e-5 of both oracles at every pixel outside
    the named margin classes of the FP64 oracle's classifier (optical margin,
    conditioning, crack); the classes are counted and stay a small minority."""
    V, N, I, camera, hap, scene = terrain_scene(ss=ss)
    pose = dict(position=(13.0, -7.0, 700.0), rotation=(0.02, -0.01, 0.3, math.sqrt(1 - 0.02**2 - 0.01**2 - 0.09)),
                light=trajectory.sun_direction(30, 40), intensity=1000)
    img, dep = CamRayCaster(scene).render_state(pose)
    r64, d64, margin = O.OracleScene(V, N, I, camera, ss, hap, fp64=True).render_margin(pose)
    r32, d32, v32 = O.OracleScene(V, N, I, camera, ss, hap).render(pose)
    assert v32.all() and np.all(np.isfinite(r64))
    for orad, odep in ((r32, d32), (r64, d64)):
        bad = outside_tolerance(img, dep, orad, odep)
        assert not np.any(bad & (margin == 0)), np.flatnonzero(bad & (margin == 0))[:10]
    assert (margin > 0).mean() < 0.06
    assert (img > 0).mean() > 0.5 and (dep > 0).mean() > 0.8


def test_leaf_size_changes_the_tree_not_the_image():
    """Nearest hits and occlusion do not depend on how the tree is cut: the
    default (binned SAH, 2 triangles per leaf), 1/8-triangle leaves and the
    Morton-radix tree render the same image up to edge ties."""
    pose = dict(position=(13.0, -7.0, 700.0), rotation=(0.0, 0.0, 0.0, 1.0),
                light=trajectory.sun_direction(30, 40), intensity=1000)
    images = {}
    for leaf in (0, 1, 8):
        V, N, I, camera, hap, scene = terrain_scene(leaf=leaf)
        info = scene.info()
        assert info["leaf_size"] == (leaf or 2) and info["builder"] == 0
        images[leaf] = CamRayCaster(scene).render_state(pose)
    morton = DeviceScene(V, N, I, camera, 2, hap, builder=1)
    info = morton.info()
    assert info["builder"] == 1 and info["sah_node_visits"] > 1 and info["sah_triangle_tests"] > 0
    images["morton"] = CamRayCaster(morton).render_state(pose)
    for key in (1, 8, "morton"):
        for a, b in zip(images[0], images[key]):
            assert float(np.mean(rel_err(a, b) > RTOL)) < 1e-3


def test_motion_blur_exposure_is_the_weighted_sum_of_renders():
    """dvs_cam_render_blur (all poses in one launch) equals the float
    accumulation, in pose order, of one render per pose
    (apps/main_cam_blur.cpp:66-73)."""
    V, N, I, camera, hap, scene = terrain_scene()
    cam = CamRayCaster(scene)
    light = trajectory.sun_direction(30, 40)
    for n_poses in (1, 5, 40):
        poses = [dict(position=(13.0 + 0.5 * j, -7.0 + 0.1 * j, 700.0 - j), rotation=(0.0, 0.0, 0.0, 1.0),
                      light=light, intensity=1000) for j in range(n_poses)]
        w = np.full(n_poses, 1.0 / n_poses, np.float32)
        w[-1] = np.float32(1.0) - np.float32(w[:-1].sum()) if n_poses > 1 else 1.0
        acc = np.zeros(scene.pixels, np.float32)
        for p, wj in zip(poses, w):
            acc = acc + cam.render_state(p)[0] * np.float32(wj)
        got = cam.render_blur(poses, w)
        assert got.dtype == np.float32 and float(np.mean(got != acc)) < 1e-3, n_poses
        assert float(np.mean(rel_err(got, acc) > RTOL)) < 1e-3
    with pytest.raises(ValueError):
        cam.render_blur([poses[0]], np.array([np.nan], np.float32))


def test_subray_packets_equal_temporal_packets():
    """A single-pose render (sub-ray packets: one warp per pixel, lanes on its
    sub-rays, ordered FP64 sums) and a nine-pose exposure (temporal packets:
    one warp over a pixel's poses) give bit-identical radiance for the same
    pose."""
    V, N, I, camera, hap, scene = terrain_scene(ss=8)
    cam = CamRayCaster(scene)
    pose = dict(position=(13.0, -7.0, 700.0), rotation=(0.02, -0.01, 0.3, math.sqrt(1 - 0.02**2 - 0.01**2 - 0.09)),
                light=trajectory.sun_direction(30, 40), intensity=1000)
    single, _ = cam.render_state(pose)
    for k in (0, 4, 8):
        w = np.zeros(9, np.float32)
        w[k] = 1
        blur = cam.render_blur([pose] * 9, w)
        assert np.array_equal(blur, single), k
    assert (single > 0).mean() > 0.5


# ---- sensor path (tests/test_sensor.cu:66-93,160-173) ----------------------------------

def plane_sensor(**over):
    V, N, I = plane_mesh()
    scene = DeviceScene(V, N, I, DAVIS, 1, DAVIS_HAPKE)
    phys = davis_physic(threshold_std=0, photon_shot_noise=0, max_events_per_step=64, readout_bandwidth=0,
                        readout_latency=0, random_seed=42)
    phys.update(over)
    return scene, phys


def test_sensor_static_then_interior_pulse():
    scene, phys = plane_sensor()
    s = EventSensor(scene, phys)
    s.initialize(POSE, 0)
    assert len(s.process((POSE, POSE, 0, 0.002))) == 0                      # no startup burst
    start = dict(POSE, intensity_rate=8e6)
    end = dict(POSE, intensity_rate=-8e6)
    ev = s.process((start, end, 0.002, 0.004))
    on, off = int((ev["polarity"] == 1).sum()), int((ev["polarity"] == 0).sum())
    assert on > 0 and off > 0                                               # pulse between equal endpoints
    assert np.all(ev["depth"] >= 10) and np.all(ev["timestamp"] > 0.002) and np.all(ev["timestamp"] <= 0.004)
    # halving circuit_step converges (tests/test_sensor.cu:160-166)
    scene2, phys2 = plane_sensor(circuit_step=0.5e-6)
    r = EventSensor(scene2, phys2)
    r.initialize(POSE, 0)
    r.process((POSE, POSE, 0, 0.002))
    ev2 = r.process((start, end, 0.002, 0.004))
    # The reference asserts equal counts on its small sensor; on the full 346x260 plane a
    # pixel whose pulse peak lies within a hair of a threshold may gain or lose its last
    # crossing with the step (a margin pixel of the accuracy statement): allow two.
    a, b = pixel_sorted(ev), pixel_sorted(ev2)
    ka = a["y"].astype(np.int64) * DAVIS["width"] + a["x"]
    kb = b["y"].astype(np.int64) * DAVIS["width"] + b["x"]
    ca = np.bincount(ka, minlength=DAVIS["width"] * DAVIS["height"])
    cb = np.bincount(kb, minlength=DAVIS["width"] * DAVIS["height"])
    differ = np.flatnonzero(ca != cb)
    assert len(differ) <= 2 and np.all(np.abs(ca[differ] - cb[differ]) == 1), differ
    same_a, same_b = ~np.isin(ka, differ), ~np.isin(kb, differ)
    assert np.max(np.abs(b["timestamp"][same_b] - a["timestamp"][same_a])) < 2e-6


def test_sensor_pulse_matches_oracle_full_resolution():
    scene, phys = plane_sensor()
    s = EventSensor(scene, phys)
    s.initialize(POSE, 0)
    start = dict(POSE, intensity_rate=8e6)
    end = dict(POSE, intensity_rate=-8e6)
    ivs = [(POSE, POSE, 0, 0.001), (start, end, 0.001, 0.003)]
    ev = s.process_many(ivs)
    V, N, I = plane_mesh()
    osc = O.OracleScene(V, N, I, DAVIS, 1, DAVIS_HAPKE)
    ors = O.OracleSensor(osc, phys)
    ors.initialize(POSE, 0)
    oev = ors.process(ivs)
    assert len(ev) == len(oev) > 0
    # The uniform plane gives many pixels the same crossing time up to the last
    # bits, so the (t, y, x) readout order of near-ties may differ; compare in
    # pixel order.
    ev, oev = pixel_sorted(ev), pixel_sorted(oev)
    for f in ("x", "y", "polarity"):
        np.testing.assert_array_equal(ev[f], oev[f])
    dt = np.abs(ev["timestamp"] - oev["timestamp"])
    assert np.max(dt) < 1e-6          # the stated timestamp tolerance
    assert np.median(dt) < 1e-15      # almost every crossing is the same double
    assert np.max(rel_err(ev["depth"], oev["depth"])) < RTOL


def test_fp32_circuit_precision_mode_against_the_fp64_oracle():
    """Precision mode (FP32 receptor/contrast arithmetic, FP64 times and
    crossing solves) on the pulse case: the same per-pixel polarity sequences
    as the FP64 oracle except pixels within 1e-4 of a threshold, timestamps
    within the stated 1 us."""
    scene, phys = plane_sensor()
    start = dict(POSE, intensity_rate=8e6)
    end = dict(POSE, intensity_rate=-8e6)
    ivs = [(POSE, POSE, 0, 0.001), (start, end, 0.001, 0.003)]
    s = EventSensor(scene, phys, circuit_precision="fp32")
    s.initialize(POSE, 0)
    ev = s.process_many(ivs)
    V, N, I = plane_mesh()
    ors = O.OracleSensor(O.OracleScene(V, N, I, DAVIS, 1, DAVIS_HAPKE, fp64=True), phys, margin=True)
    ors.initialize(POSE, 0)
    oev = ors.process(ivs)
    assert len(oev) > 1000
    report = compare_event_streams(ev, oev, ors.margins(), DAVIS["width"])
    assert report["unclassified_mismatches"] == 0, report
    assert report["max_timestamp_error_s"] < 1e-6, report
    with pytest.raises(ValueError):
        EventSensor(scene, phys, circuit_precision="fp16")


def pixel_sorted(ev):
    return ev[np.lexsort((ev["timestamp"], ev["x"], ev["y"]))]


def cell_count(t0, t1, circuit_step):
    """Circuit cells of one interval, generate_pixels' bound (event_sensor.cu:37)."""
    return math.ceil((t1 - t0) / float(np.float32(circuit_step)))


@pytest.mark.parametrize("circuit", ["fp64", "fp32"])
def test_sensor_with_reference_leak_against_the_fp64_oracle(circuit):
    """A leaking reference (reset_leakage_a > 0, pixel_model.hpp:46-59): the
    segment ends at the leak extremum and the crossing time comes from the
    48-step bisection, both FP64, out of line in the FP32 circuit.  A 64x48
    crop of the DAVIS camera through the interior pulse against the FP64 oracle:
    identical polarity sequences outside the margin classes, timestamps within
    1 us."""
    V, N, I = plane_mesh()
    crop = dict(DAVIS, width=64, height=48, cx=DAVIS["cx"] - 141, cy=DAVIS["cy"] - 106)
    scene = DeviceScene(V, N, I, crop, 1, DAVIS_HAPKE)
    phys = davis_physic(threshold_std=0, photon_shot_noise=0, max_events_per_step=64, readout_bandwidth=0,
                        readout_latency=0, random_seed=42, reset_leakage_a=1.3e-14)  # reference leak ~20 /s
    start, end = dict(POSE, intensity_rate=8e6), dict(POSE, intensity_rate=-8e6)
    ivs = [(POSE, POSE, 0, 0.001), (start, end, 0.001, 0.003)]
    s = EventSensor(scene, phys, circuit_precision=circuit)
    s.initialize(POSE, 0)
    ev = s.process_many(ivs)
    ors = O.OracleSensor(O.OracleScene(V, N, I, crop, 1, DAVIS_HAPKE, fp64=True), phys, margin=True)
    ors.initialize(POSE, 0)
    oev = ors.process(ivs)
    assert len(oev) > 1000
    report = compare_event_streams(ev, oev, ors.margins(), crop["width"])
    assert report["unclassified_mismatches"] == 0, report
    assert report["max_timestamp_error_s"] < 1e-6, report


@pytest.mark.parametrize("circuit", ["fp64", "fp32", "fp32-philox"])
@pytest.mark.parametrize("shot,reset", [(0, 0), (1, 0), (1, 1)])
def test_sensor_batch_invariance(shot, reset, circuit):
    """Batching cannot change the events, with photon shot noise and kTC reset
    noise (reset_thermal_noise, drawn after each refractory period; out of line
    in the FP32 circuits) on or off, for every circuit and noise stream."""
    scene, phys = plane_sensor(photon_shot_noise=shot, reset_thermal_noise=reset)
    bright = dict(POSE, intensity=2000)
    ivs = [(POSE, POSE, 0, 0.001), (bright, bright, 0.001, 0.002), (POSE, POSE, 0.002, 0.003)]
    grouped = EventSensor(scene, phys, circuit_precision=circuit)
    separate = EventSensor(scene, phys, circuit_precision=circuit)
    grouped.initialize(POSE, 0)
    separate.initialize(POSE, 0)
    individual = np.concatenate([separate.process(iv) for iv in ivs])
    allev = grouped.process_many(ivs)
    assert len(allev) == len(individual) > 0
    for f in ("timestamp", "x", "y", "polarity"):
        np.testing.assert_array_equal(allev[f], individual[f])


def test_philox_precision_mode_noise():
    """circuit_precision = 2 (FP32 circuit, counter-based Philox noise keyed
    by seed, pixel and cell index): batching cannot change the draws, a seed
    repeats, row bands reproduce the full sensor, and the event rate agrees
    with the XORWOW stream's within sampling error."""
    from dvsrender4deepspace_gb300 import shard
    scene, phys = plane_sensor(photon_shot_noise=1, threshold_pos=0.03, threshold_neg=0.03, refractory_time=0,
                               threshold_std=0.02)
    dim = dict(POSE, intensity=20)  # about 1e-2 photo-electrons per 1 us cell: shot noise dominates
    ivs = [(dim, dim, 0, 0.0005), (dim, dim, 0.0005, 0.001), (dim, dim, 0.001, 0.002)]

    def run(mode, split, seed=42, rows=(0, 0)):
        s = EventSensor(scene, dict(phys, random_seed=seed), circuit_precision=mode, row_begin=rows[0],
                        row_end=rows[1])
        s.initialize(dim, 0)
        ev = np.concatenate([s.process(iv) for iv in ivs]) if split else s.process_many(ivs)
        return np.concatenate([ev, s.drain()])

    a, b = run("fp32-philox", False), run("fp32-philox", True)
    assert len(a) == len(b) > 1000
    for f in ("timestamp", "x", "y", "polarity"):
        np.testing.assert_array_equal(a[f], b[f])
    c = run("fp32-philox", False, seed=43)
    assert len(c) != len(a) or not np.array_equal(c["timestamp"], a["timestamp"])
    bands = [run("fp32-philox", False, rows=r) for r in shard.row_bands(DAVIS["height"], 2)]
    merged = pixel_sorted(shard.merge_runs(bands))
    want = pixel_sorted(a)
    assert len(merged) == len(want)
    for f in ("timestamp", "x", "y", "polarity"):
        np.testing.assert_array_equal(merged[f], want[f])
    x = run("fp32", False)
    assert abs(len(x) - len(a)) < 6 * math.sqrt(len(x)) + 0.05 * len(x), (len(x), len(a))
    with pytest.raises(ValueError):
        s = EventSensor(scene, phys, circuit_precision="fp32-philox")
        s.initialize(dim, 0)
        s.process_adaptive(ivs, 1e-2)


def test_seeded_shot_noise_repeatable():
    # tests/test_sensor.cu:168-173
    scene, phys = plane_sensor(photon_shot_noise=1, threshold_pos=0.03, threshold_neg=0.03, refractory_time=0)
    a, b = EventSensor(scene, phys), EventSensor(scene, phys)
    a.initialize(POSE, 0)
    b.initialize(POSE, 0)
    ea = a.process((POSE, POSE, 0, 0.001))
    eb = b.process((POSE, POSE, 0, 0.001))
    assert len(ea) > 0 and len(ea) == len(eb)
    for f in ("timestamp", "x", "y", "polarity"):
        np.testing.assert_array_equal(ea[f], eb[f])


def test_back_to_back_enqueues_equal_processing():
    """Batches enqueued without collecting in between (the device-timed loop of
    the benchmark) advance the pixel circuits exactly as processed batches:
    each upload finishes reading the pinned staging before the next batch
    overwrites it.  The last batch's events are those of processing."""
    cam = dict(width=64, height=48, fx=60.0, fy=60.0, cx=32.0, cy=24.0)
    V, N, I, camera, hap, scene = terrain_scene(n=80, seed=9, camera=cam, ss=2)
    traj = trajectory.StraightPass((0.0, 0.0, 400.0), (50.0, 0.0, 0.0), trajectory.sun_direction(30), 1000.0)
    phys = davis_physic(threshold_std=0.02, photon_shot_noise=1, max_events_per_step=64, readout_bandwidth=0,
                        readout_latency=0, threshold_pos=0.05, threshold_neg=0.05, random_seed=3)
    batches, t = [], 0.0
    for k in range(6):
        ivs = trajectory.horizons(traj, t, 1e-4, 8)
        t = ivs[-1][3]
        batches.append(ivs)
    # a light pulse closes the last batch, so it carries events
    p0, p1 = traj.state(t), traj.state(t + 2e-3)
    batches[-1].append((dict(p0, intensity_rate=8e6), dict(p1, intensity_rate=-8e6), t, t + 2e-3))
    a, b = EventSensor(scene, phys), EventSensor(scene, phys)
    a.initialize(traj.state(0.0), 0.0)
    b.initialize(traj.state(0.0), 0.0)
    for ivs in batches[:-1]:
        a.enqueue(ivs)
    a.enqueue(batches[-1])
    last_a = a.collect()
    for ivs in batches[:-1]:
        b.process_many(ivs)
    last_b = b.process_many(batches[-1])
    sa, ra = a.read_state()
    sb, rb = b.read_state()
    assert np.array_equal(sa, sb) and np.array_equal(ra, rb)
    assert len(last_a) == len(last_b) > 0
    for f in ("timestamp", "x", "y", "polarity", "depth"):
        np.testing.assert_array_equal(last_a[f], last_b[f])


def test_capacity_error_and_rejections():
    scene, phys = plane_sensor(max_events_per_step=1, refractory_time=0, threshold_pos=0.01, threshold_neg=0.01,
                               threshold_min=0.001)
    s = EventSensor(scene, phys)
    s.initialize(POSE, 0)
    start = dict(POSE, intensity_rate=8e6)
    end = dict(POSE, intensity_rate=-8e6)
    with pytest.raises(CapacityError):
        s.process((start, end, 0, 0.002))
    t = EventSensor(scene, plane_sensor()[1])
    with pytest.raises(ValueError):
        t.process((POSE, POSE, 0, 0.001))          # not initialized
    t.initialize(POSE, 0)
    with pytest.raises(ValueError):
        t.process((POSE, POSE, 0.001, 0.002))      # not contiguous
    with pytest.raises(ValueError):
        t.process((POSE, POSE, 0, 2.0))            # > 1e6 cells in one batch


def test_ray_counters_and_stats():
    scene, phys = plane_sensor()
    s = EventSensor(scene, phys, timing=True)
    s.initialize(POSE, 0)
    s.reset_stats()
    s.process_many([(POSE, POSE, 0, 0.0001), (POSE, POSE, 0.0001, 0.0002)])
    st = s.stats()
    n = DAVIS["width"] * DAVIS["height"]
    cells = cell_count(0, 0.0001, 1e-6) + cell_count(0.0001, 0.0002, 1e-6)  # 101 + 101: float circuit_step
    assert st["primary_rays"] == n * cells
    assert st["shadow_rays"] > 0 and st["circuit_cells"] == n * cells
    assert st["optics_ms"] > 0 and st["circuit_ms"] > 0


def test_sensor_matches_oracle_on_moving_terrain():
    cam = dict(width=64, height=48, fx=60.0, fy=60.0, cx=32.0, cy=24.0)
    V, N, I, camera, hap, scene = terrain_scene(n=80, seed=9, camera=cam, ss=1)
    traj = trajectory.StraightPass((0.0, 0.0, 400.0), (50.0, 0.0, 0.0), trajectory.sun_direction(30), 1000.0)
    phys = davis_physic(threshold_std=0, photon_shot_noise=0, max_events_per_step=64, readout_bandwidth=0,
                        readout_latency=0, threshold_pos=0.05, threshold_neg=0.05, refractory_time=5e-5)
    s = EventSensor(scene, phys)
    s.initialize(traj.state(0.0), 0.0)
    osc = O.OracleScene(V, N, I, camera, 1, hap)
    ors = O.OracleSensor(osc, phys, margin=True)
    ors.initialize(traj.state(0.0), 0.0)
    gpu, ora = [], []
    t = 0.0
    for batch in range(3):
        ivs = trajectory.horizons(traj, t, 1e-4, 20)
        if batch == 1:  # a 2 ms light pulse inside the moving pass
            a, b = traj.state(ivs[-1][3]), traj.state(ivs[-1][3] + 2e-3)
            ivs.append((dict(a, intensity_rate=8e6), dict(b, intensity_rate=-8e6), ivs[-1][3], ivs[-1][3] + 2e-3))
        t = ivs[-1][3]
        gpu.append(s.process_many(ivs))
        ora.append(ors.process(ivs))
    gpu.append(s.drain())
    ora.append(ors.drain())
    g, o = np.concatenate(gpu), np.concatenate(ora)
    assert len(o) > 50
    report = compare_event_streams(g, o, ors.margins(), cam["width"])
    assert report["unclassified_mismatches"] == 0, report
    assert report["max_timestamp_error_s"] < 1e-6, report
    # the classes accumulate over the pass's 6,000 cells: a pixel is flagged if any cell is a margin cell
    assert report["margin_pixels"] < 0.15 * cam["width"] * cam["height"], report


def compare_event_streams(g, o, margins, width):
    """Per-pixel polarity sequences of two event streams: pixels whose sequences
    differ must be margin pixels of the oracle's classifier; timestamps of the
    other pixels' events are compared in order."""
    def per_pixel(ev):
        d = {}
        for e in ev:
            d.setdefault((int(e["x"]), int(e["y"])), []).append((float(e["timestamp"]), int(e["polarity"])))
        return d
    pg, po = per_pixel(g), per_pixel(o)
    mismatched, unclassified, worst = 0, 0, 0.0
    for key in set(pg) | set(po):
        a, b = pg.get(key, []), po.get(key, [])
        flagged = margins[key[1] * width + key[0]] != 0
        if [p for _, p in a] != [p for _, p in b]:
            mismatched += 1
            unclassified += 0 if flagged else 1
            continue
        if a and not flagged:
            worst = max(worst, max(abs(x - y) for (x, _), (y, _) in zip(a, b)))
    return {"pixels_with_events": len(set(pg) | set(po)), "mismatched_pixels": mismatched,
            "unclassified_mismatches": unclassified, "margin_pixels": int((margins != 0).sum()),
            "max_timestamp_error_s": worst}


def test_packet_shape_and_autotuner_do_not_change_events():
    """Cells per warp, one or two sub-rays per lane and the autotuner's
    choice change how rays share warps, not what each ray computes: the
    events of a moving, pulsed terrain pass (4 sub-rays per pixel) are the
    same for every shape."""
    cam = dict(width=64, height=48, fx=60.0, fy=60.0, cx=32.0, cy=24.0)
    V, N, I, camera, hap, scene = terrain_scene(n=80, seed=9, camera=cam, ss=2)
    traj = trajectory.StraightPass((0.0, 0.0, 400.0), (50.0, 0.0, 0.0), trajectory.sun_direction(30), 1000.0)
    phys = davis_physic(threshold_std=0, max_events_per_step=64, readout_bandwidth=0, readout_latency=0,
                        threshold_pos=0.05, threshold_neg=0.05, refractory_time=5e-5, random_seed=5)

    def run(shape):
        s = EventSensor(scene, phys)
        s.initialize(traj.state(0.0), 0.0)
        out, t, tuned = [], 0.0, None
        for batch in range(2):
            ivs = trajectory.horizons(traj, t, 1e-4, 20)
            a, b = traj.state(ivs[-1][3]), traj.state(ivs[-1][3] + 2e-3)
            ivs.append((dict(a, intensity_rate=8e6), dict(b, intensity_rate=-8e6), ivs[-1][3], ivs[-1][3] + 2e-3))
            t = ivs[-1][3]
            if shape == "auto" and batch == 0:
                tuned = s.autotune(ivs)
            elif shape != "auto" and batch == 0:
                s.set_tuning(*shape)
            out.append(s.process_many(ivs))
        out.append(s.drain())
        return np.concatenate(out), tuned

    ref, _ = run((32, 2))
    assert len(ref) > 100
    for shape in ((32, 1), (4, 2), (8, 1), (16, 4), "auto"):
        ev, tuned = run(shape)
        assert len(ev) == len(ref), shape
        for f in ref.dtype.names:
            assert np.array_equal(ev[f], ref[f]), (shape, f)
        if tuned:
            assert tuned["rays_per_lane"] in (1, 2, 4) and tuned["cells_per_warp"] in (4, 8, 16, 32)
            assert tuned["candidates"] >= 4 and tuned["best_ms"] > 0
            # second stage: the circuit-step chunk over the batch's default chunk -- here 2048 cells
            # (the 512 MB radiance bound at 64x48 pixels) of the 4000-cell batch: 2048, 1024, 512, 256
            assert tuned["chunk_cells"] == 2048 and tuned["chunk_candidates"] == 4
            assert tuned["cells_per_chunk"] in (256, 512, 1024, 2048) and tuned["chunk_best_ms"] > 0
    s = EventSensor(scene, phys)
    with pytest.raises(ValueError):
        s.set_tuning(3, 2)
    with pytest.raises(ValueError):
        s.set_tuning(8, 3)


def test_row_band_sensors_reproduce_the_full_sensor():
    """One GPU's share of a split sensor (dvs_sensor_options.row_begin/row_end)
    gives exactly the full sensor's events of those rows."""
    from dvsrender4deepspace_gb300 import shard
    scene, phys = plane_sensor(photon_shot_noise=1, threshold_pos=0.05, threshold_neg=0.05)
    start, end = dict(POSE, intensity_rate=8e6), dict(POSE, intensity_rate=-8e6)
    ivs = [(POSE, POSE, 0, .0005), (start, end, .0005, .0015)]
    full = EventSensor(scene, phys)
    full.initialize(POSE, 0)
    want = full.process_many(ivs)
    got = []
    for r0, r1 in shard.row_bands(DAVIS["height"], 3):
        band = EventSensor(scene, phys, row_begin=r0, row_end=r1)
        band.initialize(POSE, 0)
        ev = band.process_many(ivs)
        assert np.all((ev["y"] >= r0) & (ev["y"] < r1))
        got.append(ev)
    merged = shard.merge_runs(got)
    assert len(merged) == len(want) > 0
    a, b = pixel_sorted(merged), pixel_sorted(want)
    for f in ("timestamp", "x", "y", "polarity", "depth"):
        np.testing.assert_array_equal(a[f], b[f])
