"""Multi-sensor batches (dvs_batch_*): many sensors over one terrain advanced
together -- one persistent trace launch and one circuit launch per step, the
step captured into a CUDA graph and replayed.  Every member's events must be
the events of the same sensor processed alone (bit for bit: the batch kernels
run the one-sensor kernels' per-item code), through idle members, shape
changes and graph replays, for each circuit precision and geometry format."""
import numpy as np
import pytest

from dvsrender4deepspace_gb300 import DeviceScene, EventSensor, SensorBatch, terrain, trajectory
from dvsrender4deepspace_gb300.raycast import HALF_BOUNDS, WATERTIGHT
from tests.test_oracle_golden import davis_physic

pytestmark = pytest.mark.gpu

HAPKE = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)
CAMERAS = [(dict(width=64, height=48, fx=60.0, fy=60.0, cx=32.0, cy=24.0), 2),
           (dict(width=96, height=64, fx=80.0, fy=80.0, cx=48.0, cy=32.0), 2),
           (dict(width=40, height=40, fx=50.0, fy=50.0, cx=20.0, cy=20.0), 4),
           (dict(width=50, height=30, fx=40.0, fy=40.0, cx=25.0, cy=15.0), 2)]


def physic(**over):
    p = davis_physic(threshold_std=0.02, photon_shot_noise=1, max_events_per_step=64, readout_bandwidth=0,
                     readout_latency=0, threshold_pos=0.05, threshold_neg=0.05, refractory_time=5e-5,
                     random_seed=7)
    p.update(over)
    return p


def passes():
    out = []
    for k in range(len(CAMERAS)):
        out.append(trajectory.StraightPass((15.0 * k, -10.0 * k, 350.0 + 40 * k), (40.0 + 10 * k, 5.0 * k, 0.0),
                                           trajectory.sun_direction(30 + 5 * k, 20 * k), 1000.0))
    return out


def make_sensors(base, cameras, phys, circuit):
    sensors = []
    for (cam, ss), traj in zip(cameras, passes()):
        s = EventSensor(base.view(cam, ss), phys, circuit_precision=circuit)
        s.initialize(traj.state(0.0), 0.0)
        sensors.append(s)
    return sensors


def schedule(n_members, steps, idle, pulse=True):
    """Per step, per member: its intervals (10 horizons of 10 us; empty when
    idle); with `pulse`, member 0 gets a light pulse interval at step 1."""
    trajs = passes()
    t = [0.0] * n_members
    out = []
    for k in range(steps):
        row = []
        for m in range(n_members):
            if (k, m) in idle:
                row.append([])
                continue
            ivs = trajectory.horizons(trajs[m], t[m], 1e-5, 10)
            if pulse and k == 1 and m == 0:   # a light pulse inside the pass
                a, b = trajs[m].state(ivs[-1][3]), trajs[m].state(ivs[-1][3] + 2e-4)
                ivs.append((dict(a, intensity_rate=4e6), dict(b, intensity_rate=-4e6), ivs[-1][3], ivs[-1][3] + 2e-4))
            t[m] = ivs[-1][3]
            row.append(ivs)
        out.append(row)
    return out


def run_alone(base, cameras, phys, circuit, plan):
    sensors = make_sensors(base, cameras, phys, circuit)
    got = [[] for _ in sensors]
    for row in plan:
        for m, ivs in enumerate(row):
            if ivs:
                got[m].append(sensors[m].process_many(ivs))
    return [np.concatenate(g) if g else np.zeros(0) for g in got]


def run_batch(base, cameras, phys, circuit, plan):
    sensors = make_sensors(base, cameras, phys, circuit)
    batch = SensorBatch(sensors)
    got = [[] for _ in sensors]
    for row in plan:
        for m, ev in enumerate(batch.process(row)):
            if row[m]:
                got[m].append(ev)
    return [np.concatenate(g) if g else np.zeros(0) for g in got], batch.stats(), sensors


def assert_same(alone, batched):
    total = 0
    for a, b in zip(alone, batched):
        assert len(a) == len(b)
        total += len(a)
        for f in ("timestamp", "x", "y", "polarity", "depth"):
            np.testing.assert_array_equal(a[f], b[f])
    return total


@pytest.fixture(scope="module")
def base():
    V, N, I = terrain.terrain_mesh(80, 9)
    return DeviceScene(V, N, I, CAMERAS[0][0], CAMERAS[0][1], HAPKE)


@pytest.mark.parametrize("circuit", ["fp64", "fp32", "fp32-philox"])
def test_batch_members_equal_alone_through_idle_steps(base, circuit):
    plan = schedule(4, 4, idle={(2, 1), (3, 1), (3, 3)})
    phys = physic()
    alone = run_alone(base, CAMERAS, phys, circuit, plan)
    batched, stats, _ = run_batch(base, CAMERAS, phys, circuit, plan)
    assert assert_same(alone, batched) > 100
    # four shapes: plain, member 0's pulse interval, then two different idle sets
    assert stats["steps"] == 4 and stats["graph_launches"] == 4 and stats["graph_captures"] == 4
    assert stats["persistent_launches"] >= 4 and stats["trace_items"] > 0 and stats["step_ms"] > 0


def test_batch_replays_one_graph_and_counts_rays(base):
    plan = schedule(4, 5, idle=set(), pulse=False)
    phys = physic()
    alone = run_alone(base, CAMERAS, phys, "fp32", plan)
    batched, stats, sensors = run_batch(base, CAMERAS, phys, "fp32", plan)
    assert_same(alone, batched)
    assert stats["graph_captures"] == 1 and stats["graph_launches"] == 5
    for s, (cam, ss) in zip(sensors, CAMERAS):   # 5 steps x 10 cells, counted on the device
        assert s.stats()["primary_rays"] >= cam["width"] * cam["height"] * ss * ss * 10 * 5


def test_batch_one_ray_per_lane_when_a_member_has_odd_subrays(base):
    cams = CAMERAS[:2] + [(dict(width=32, height=24, fx=30.0, fy=30.0, cx=16.0, cy=12.0), 1)]
    plan = schedule(3, 2, idle=set())
    phys = physic()
    alone = run_alone(base, cams, phys, "fp64", plan)
    batched, stats, _ = run_batch(base, cams, phys, "fp64", plan)
    assert_same(alone, batched)


@pytest.mark.parametrize("geometry", [HALF_BOUNDS, HALF_BOUNDS | WATERTIGHT])
def test_batch_over_precision_geometry(geometry):
    V, N, I = terrain.terrain_mesh(80, 9)
    base = DeviceScene(V, N, I, CAMERAS[0][0], CAMERAS[0][1], HAPKE, geometry=geometry)
    plan = schedule(4, 2, idle={(1, 2)})
    phys = physic()
    alone = run_alone(base, CAMERAS, phys, "fp32-philox", plan)
    batched, _, _ = run_batch(base, CAMERAS, phys, "fp32-philox", plan)
    assert assert_same(alone, batched) > 0


def test_batch_rejects_mixed_members(base):
    phys = physic()
    V, N, I = terrain.terrain_mesh(40, 3)
    other = DeviceScene(V, N, I, CAMERAS[0][0], 2, HAPKE)
    a = EventSensor(base, phys)
    b = EventSensor(other, phys)
    c = EventSensor(base.view(*CAMERAS[1]), phys, circuit_precision="fp32")
    with pytest.raises(ValueError):
        SensorBatch([a, b])          # two geometries
    with pytest.raises(ValueError):
        SensorBatch([a, c])          # two circuit precisions
    with pytest.raises(ValueError):
        SensorBatch([a, a])          # one sensor twice
    with pytest.raises(ValueError):
        SensorBatch([])
