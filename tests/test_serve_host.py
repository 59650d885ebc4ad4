"""Host-side logic of the serving loop (CPU): admission under the HBM budget,
the SRPT and fair policies, batch-sized cursors and job completion, with
stand-ins for the device scene and sensor that record what the server asks
of them (the device path itself is covered by tests/test_gpu_serve.py)."""
import numpy as np
import pytest

from dvsrender4deepspace_gb300 import serve


class FakeView:
    def __init__(self, log, camera):
        self.log, self.camera = log, camera

    def close(self):
        self.log.append(("close_view", self.camera["width"]))


class FakeScene:
    def __init__(self, log):
        self.log = log

    def view(self, camera, supersample):
        self.log.append(("view", camera["width"], supersample))
        return FakeView(self.log, camera)


class FakeSensor:
    """Advances a clock over the enqueued intervals; one event per batch."""
    instances = []

    def __init__(self, scene, physic, circuit_precision="fp64"):
        self.scene, self.t, self.batches, self.closed = scene, None, [], False
        self.rays = 0
        self.circuit = circuit_precision
        FakeSensor.instances.append(self)

    def initialize(self, state, t):
        self.t = t

    def enqueue(self, ivs):
        assert ivs["t0"][0] == self.t, "batches must be contiguous"
        self.t = float(ivs["t1"][-1])
        self.batches.append(len(ivs))
        self.rays += len(ivs)

    def collect(self):
        return np.zeros(1, dtype=[("timestamp", "f8")])

    def drain(self):
        return np.zeros(0, dtype=[("timestamp", "f8")])

    def stats(self):
        return {"primary_rays": self.rays, "shadow_rays": 0}

    def device_bytes(self):
        return 1

    def close(self):
        self.closed = True


@pytest.fixture
def fake(monkeypatch):
    FakeSensor.instances = []
    monkeypatch.setattr(serve, "EventSensor", FakeSensor)
    log = []
    return log, [FakeScene(log), FakeScene(log)]


def jobs_of(spec):
    """spec: (arrival, width, duration) per job; 1 us cells, 10 us horizons."""
    out = []
    for i, (arrival, w, dur) in enumerate(spec):
        cam = dict(width=w, height=w, fx=w, fy=w, cx=w / 2, cy=w / 2)
        path = serve.T.StraightPass((0.0, 0.0, 500.0), (10.0, 0.0, 0.0), serve.T.sun_direction(30), 1000.0)
        out.append(serve.Job(i, arrival, i % 2, cam, 1, dur, 1e-5, path, dict(circuit_step=1e-6)))
    return out


def test_every_job_completes_with_contiguous_batches(fake):
    log, scenes = fake
    jobs = jobs_of([(0.0, 64, 1e-3), (0.0, 32, 3e-4), (0.0, 16, 2.05e-4)])
    srv = serve.Server(scenes, 1 << 40, horizons_per_step=8, policy="fair")
    done = srv.run(jobs, realtime=False)
    for j, s in zip(done, FakeSensor.instances):
        want = int(np.ceil(j.duration / 1e-5 - 1e-9))
        assert sum(s.batches) == want and all(b <= 8 for b in s.batches), (s.batches, want)
        assert s.closed and j.finished >= j.admitted and len(j.events) == len(s.batches)
        assert j.rays == want
    assert srv.used == 0 and srv.steps == max(len(s.batches) for s in FakeSensor.instances)
    assert sorted(e for e in log if e[0] == "close_view") == sorted(("close_view", j.camera["width"]) for j in jobs)


def test_srpt_finishes_short_jobs_first(fake):
    log, scenes = fake
    # one long job and three short ones, all eligible at once; the fill admits the long
    # job's batch only when nothing shorter is left
    jobs = jobs_of([(0.0, 64, 2e-3), (0.0, 16, 1e-4), (0.0, 16, 2e-4), (0.0, 16, 1.5e-4)])
    srv = serve.Server(scenes, 1 << 40, horizons_per_step=10, policy="srpt", fill_samples=16 * 16 * 10 * 10 * 3)
    done = srv.run(jobs, realtime=False)
    order = sorted(done, key=lambda j: j.finished)
    assert [j.job_id for j in order][-1] == 0             # the long job finishes last
    assert order[0].job_id == 1                            # the shortest first
    fair = serve.Server(scenes, 1 << 40, horizons_per_step=10, policy="fair")
    FakeSensor.instances = []
    done_fair = fair.run(jobs_of([(0.0, 64, 2e-3), (0.0, 16, 1e-4), (0.0, 16, 2e-4), (0.0, 16, 1.5e-4)]),
                         realtime=False)
    assert all(len(j.events) > 0 for j in done_fair)


def test_admission_respects_the_budget(fake):
    log, scenes = fake
    jobs = jobs_of([(0.0, 128, 3e-4), (0.0, 128, 3e-4), (0.0, 128, 3e-4)])
    srv = serve.Server(scenes, 0, horizons_per_step=10)
    need = srv.estimate_bytes(jobs[0])
    srv = serve.Server(scenes, 2 * need, horizons_per_step=10)   # two at a time
    srv.run(jobs, realtime=False)
    assert srv.peak_active == 2 and srv.peak_used <= 2 * need and srv.used == 0
    with pytest.raises(ValueError):
        serve.Server(scenes, need - 1).run(jobs_of([(0.0, 128, 1e-4)]), realtime=False)
    with pytest.raises(ValueError):
        serve.Server(scenes, 1 << 30, policy="lifo")


def test_synthetic_stream_is_seeded_and_in_range():
    a = serve.synthetic_stream(40, 7, 8, duration_scale=0.01)
    b = serve.synthetic_stream(40, 7, 8, duration_scale=0.01)
    assert [(j.arrival, j.camera["width"], j.duration, j.terrain) for j in a] == \
           [(j.arrival, j.camera["width"], j.duration, j.terrain) for j in b]
    assert all(0.05 * 0.01 <= j.duration <= 2.0 * 0.01 for j in a)
    assert {j.camera["width"] for j in a} <= {64, 346, 640, 1280} and all(0 <= j.terrain < 8 for j in a)
    arrivals = np.array([j.arrival for j in a])
    assert np.all(np.diff(arrivals) > 0) and 0.05 < arrivals[-1] < 0.6   # ~200 jobs per second
