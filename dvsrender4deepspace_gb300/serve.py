"""Continuous-batching server for render + DVS jobs on one GPU.

Jobs (a camera, a trajectory over one terrain of a pool, a physic block and
a simulated duration) arrive over time.  The server keeps every admitted
job's state on the device -- a scene view over its terrain's shared BVH
(dvs_scene_view_create: one device copy per terrain), its sensor's circuit
state, RNG and event buffers -- and advances admitted jobs in scheduler
steps: a step enqueues the next horizon batch of each chosen job on that
job's own CUDA stream (dvs_sensor_enqueue, asynchronous, so the jobs' kernels
overlap on the GPU), then collects those jobs' ready events.  A job that
reaches its duration is drained and released; arrivals are admitted whenever
their device memory fits under the HBM budget (continuous batching:
admission happens between steps, while other jobs are in flight).

Which admitted jobs a step advances is the policy: "srpt" takes jobs in
order of least remaining work (pixel-cell samples) until the step holds
fill_samples of work, so short jobs that arrive while a long one runs finish
first (preemption at batch granularity; the long job's state stays
resident); "fair" advances every admitted job each step.  Each job's events
depend only on its own inputs, so a job yields the same events alone, in any
mix and under either policy.

The reference has no serving layer (one process per sequence,
tools/run_sequences.py:247-256); this is the GB300 addition.
"""
import dataclasses
import math
import time
from typing import Any, Optional

import numpy as np

from . import trajectory as T
from .raycast import EventSensor, interval_array

EVENT_SLAB_BYTES = 8 + 1 + 24   # per pixel and event slot: time, polarity, compacted event
READOUT_EVENT_BYTES = 2 * 16 + 16 + 24  # per event slot of the device readout: sort keys x2, completions, output
STATE_BYTES = 5 * 8 + 1 + 48 + 4  # per pixel: FP64 circuit state, reset flag, XORWOW, event count
RADIANCE_CHUNK_CAP = 512 << 20    # the sensor's largest radiance chunk


@dataclasses.dataclass
class Job:
    job_id: int
    arrival: float              # seconds after the start of the stream
    terrain: int                # index into the server's scene pool
    camera: dict
    supersample: int
    duration: float             # simulated seconds
    time_resolution: float      # horizon length, seconds
    path: Any                   # trajectory with .state(t) -> optical-state dict
    physic: dict
    admitted: float = math.nan
    finished: float = math.nan
    events: Optional[np.ndarray] = None
    rays: int = 0
    device_bytes: int = 0

    @property
    def latency(self):
        return self.finished - self.arrival

    @property
    def pixels(self):
        return int(self.camera["width"]) * int(self.camera["height"])


class _Active:
    def __init__(self, job, scene, sensor, reserved):
        self.job, self.scene, self.sensor, self.reserved = job, scene, sensor, reserved
        self.cursor = 0.0
        self.chunks = []
        # horizons of the job, counted once.  A job covers duration / time_resolution
        # whole horizons; a ratio a rounding above an integer (a float time_resolution)
        # adds none.  bin/dvs keeps the reference app's plain ceil, which then runs one
        # more, very short horizon up to its end time (apps/main_dvs.cpp:82-84); served
        # jobs have no such app counterpart, so they stop at the last whole horizon.
        self.total_h = max(1, math.ceil(job.duration / job.time_resolution - 1e-9))
        self.done_h = 0


class Server:
    """scenes: base DeviceScene per terrain of the pool (their BVHs stay
    resident); hbm_budget: device bytes the admitted jobs may hold."""

    def __init__(self, scenes, hbm_budget, horizons_per_step=64, max_active=64, policy="srpt",
                 fill_samples=1 << 26, circuit="fp32-philox"):
        """circuit: the jobs' pixel circuit -- "fp32-philox" (the default:
        FP32 receptor arithmetic, FP64 times and root solves, and the
        counter-based Philox photon counts, whose no-event path has no FP64
        instruction -- the circuit is what bounds supersample-1 jobs), "fp32"
        (the same arithmetic with the reference's XORWOW stream, whose
        curand_poisson runs in FP64) or the reference's "fp64"."""
        if policy not in ("srpt", "fair"):
            raise ValueError("policy must be srpt or fair")
        if circuit not in ("fp64", "fp32", "fp32-philox"):
            raise ValueError("circuit must be fp64, fp32 or fp32-philox")
        self.circuit = circuit
        self.scenes = list(scenes)
        self.budget = int(hbm_budget)
        self.horizons = int(horizons_per_step)
        self.max_active = int(max_active)
        self.policy = policy
        self.fill = int(fill_samples)
        self.used = 0
        self.peak_used = 0
        self.peak_active = 0
        self.steps = 0

    def estimate_bytes(self, job):
        """Device bytes a job holds: circuit state, event slabs, its radiance
        chunk and batch buffers, and its view's pixel order."""
        n = job.pixels
        cells = self.horizons * max(1, math.ceil(job.time_resolution / job.physic.get("circuit_step", 1e-6) - 1e-9))
        chunk = min(RADIANCE_CHUNK_CAP, (4 if self.circuit != "fp64" else 8) * n * min(2048, cells))
        slots = int(job.physic.get("max_events_per_step", 16))
        ring = 0
        if job.physic.get("readout_bandwidth", 0) > 0:  # the device readout's pending ring (a power of two)
            ring = 24 * (1 << max(0, int(min(job.physic.get("readout_queue_capacity", 1), 1 << 24)) - 1).bit_length())
        return (n * (STATE_BYTES + (EVENT_SLAB_BYTES + READOUT_EVENT_BYTES) * slots + 4) + chunk + ring
                + cells * 256 + (4 << 20))

    @staticmethod
    def _cells_per_horizon(job):
        return max(1, math.ceil(job.time_resolution / job.physic.get("circuit_step", 1e-6) - 1e-9))

    def _remaining_samples(self, a):
        j = a.job
        return j.pixels * j.supersample ** 2 * (a.total_h - a.done_h) * self._cells_per_horizon(j)

    def _step_samples(self, a):
        j = a.job
        horizons = min(self.horizons, a.total_h - a.done_h)
        return j.pixels * j.supersample ** 2 * horizons * self._cells_per_horizon(j)

    def _choose(self, active):
        if self.policy == "fair":
            return list(active)
        chosen, work = [], 0
        for a in sorted(active, key=lambda a: (self._remaining_samples(a), a.job.arrival, a.job.job_id)):
            if chosen and work + self._step_samples(a) > self.fill:
                continue
            chosen.append(a)
            work += self._step_samples(a)
        return chosen

    def _admit(self, job, now):
        scene = self.scenes[job.terrain].view(job.camera, job.supersample)
        sensor = EventSensor(scene, job.physic, circuit_precision=self.circuit)
        sensor.initialize(job.path.state(0.0), 0.0)
        reserved = self.estimate_bytes(job)
        a = _Active(job, scene, sensor, reserved)
        job.admitted = now
        self.used += reserved
        self.peak_used = max(self.peak_used, self.used)
        return a

    def _release(self, a, now):
        job = a.job
        a.chunks.append(a.sensor.drain())
        st = a.sensor.stats()
        job.rays = int(st["primary_rays"] + st["shadow_rays"])
        job.device_bytes = max(a.reserved, a.sensor.device_bytes())
        job.events = np.concatenate(a.chunks) if a.chunks else np.zeros(0)
        job.finished = now
        a.sensor.close()
        a.scene.close()
        self.used -= a.reserved

    def run(self, jobs, realtime=True):
        """Serves the jobs; with realtime, a job is eligible from its arrival
        time on (the scheduler sleeps when idle), else all are eligible at
        once.  Returns the jobs with events, times and ray counts filled."""
        pending = sorted(jobs, key=lambda j: (j.arrival if realtime else 0.0, j.job_id))
        active = []
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        while pending or active:
            t = now()
            while (pending and len(active) < self.max_active and (not realtime or pending[0].arrival <= t)
                   and self.used + self.estimate_bytes(pending[0]) <= self.budget):
                active.append(self._admit(pending.pop(0), t))
            if not active:
                if pending and self.estimate_bytes(pending[0]) > self.budget:
                    raise ValueError("job %d needs more device memory than the budget" % pending[0].job_id)
                if pending and realtime:
                    time.sleep(max(0.0, pending[0].arrival - now()))
                continue
            self.peak_active = max(self.peak_active, len(active))
            chosen = self._choose(active)
            for a in chosen:  # launch each chosen job's next batch; nothing waits here
                j = a.job
                count = min(self.horizons, a.total_h - a.done_h)
                ivs = T.horizons(j.path, a.cursor, j.time_resolution, count)
                a.sensor.enqueue(interval_array(ivs))
                a.cursor = ivs[-1][3]
                a.done_h += count
            self.steps += 1
            done = set()
            for a in chosen:
                a.chunks.append(a.sensor.collect())
                if a.done_h >= a.total_h:
                    self._release(a, now())
                    done.add(id(a))
            active = [a for a in active if id(a) not in done]
        return jobs


def latency_summary(jobs):
    lat = np.array([j.latency for j in jobs])
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "max_ms": float(lat.max() * 1e3)}


def synthetic_stream(n_jobs, seed, n_terrains, rate_hz=200.0, durations=(0.05, 2.0), duration_scale=1.0,
                     resolutions=((64, 48), (346, 260), (640, 480), (1280, 720)), supersample=1,
                     time_resolution=1e-5, physic=None, intensity=1000.0):
    """Seeded Poisson stream of jobs: resolutions uniform over the list,
    durations log-uniform (times duration_scale), terrain uniform over the
    pool, each a straight nadir pass at 0.5-5 km and 10-200 m/s."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    light = T.sun_direction(30.0, 35.0)
    for i in range(n_jobs):
        t += rng.exponential(1.0 / rate_hz)
        w, h = resolutions[rng.integers(len(resolutions))]
        f = 0.75 * w  # a 67 degree field of view
        cam = dict(width=w, height=h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0)
        dur = float(np.exp(rng.uniform(np.log(durations[0]), np.log(durations[1])))) * duration_scale
        alt = float(rng.uniform(500.0, 5000.0))
        speed = float(rng.uniform(10.0, 200.0))
        heading = float(rng.uniform(0, 2 * np.pi))
        start = (float(rng.uniform(-500, 500)), float(rng.uniform(-500, 500)), alt)
        vel = (speed * math.cos(heading), speed * math.sin(heading), 0.0)
        jobs.append(Job(i, t, int(rng.integers(n_terrains)), cam, supersample, dur, time_resolution,
                        T.StraightPass(start, vel, light, intensity), dict(physic or {})))
    return jobs
