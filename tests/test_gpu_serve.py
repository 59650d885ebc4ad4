"""Serving loop on the GPU: jobs of different resolutions and lengths over a
pool of terrains share the device; every job's events are the same alone,
all together, and under a memory budget that admits them a few at a time
(continuous admission as others finish).  Scene views share their terrain's
device geometry."""
import math

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import CamRayCaster, DeviceScene, serve, terrain, trajectory

pytestmark = pytest.mark.gpu

HAPKE = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)
PHYSIC = dict(threshold_pos=0.2, threshold_neg=0.2, threshold_std=0.03, threshold_min=0.01, refractory_time=100e-6,
              readout_bandwidth=5e6, readout_latency=18e-9, photon_shot_noise=1, random_seed=3,
              max_events_per_step=16, circuit_step=1e-6, wavelength_nm=550, quantum_efficiency=0.3,
              pixel_pitch_um=15, fill_factor=0.2, f_number=2.0, lens_transmission=0.8, radiance_scale=0.001,
              temperature_k=300, subthreshold_kappa=0.8, receptor_capacitance_f=1e-15, reset_capacitance_f=20e-15,
              dark_current_a=1e-18, reset_leakage_a=0, reset_thermal_noise=0, readout_queue_capacity=100000)


@pytest.fixture(scope="module")
def pool():
    scenes = []
    for n, seed in ((64, 1), (96, 2)):
        V, N, I = terrain.terrain_mesh(n, seed)
        scenes.append(DeviceScene(V, N, I, dict(width=8, height=8, fx=8.0, fy=8.0, cx=4.0, cy=4.0), 1, HAPKE))
    return scenes


class FlickerPass(trajectory.StraightPass):
    """A straight pass under a bright light whose intensity oscillates at
    1 kHz: the photoreceptor (time constant ~30 us at this light level)
    follows it, so every lit pixel crosses its thresholds within a
    millisecond."""

    def state(self, t):
        s = super().state(t)
        w = 2 * math.pi * 1000.0
        s["intensity"] = self.intensity * (1.0 + 0.6 * math.sin(w * t))
        s["intensity_rate"] = self.intensity * 0.6 * w * math.cos(w * t)
        return s


def jobs():
    light = trajectory.sun_direction(30, 40)
    spec = [((64, 48), 0, 8e-4), ((96, 72), 1, 3e-4), ((128, 96), 0, 5e-4), ((64, 48), 1, 2e-3),
            ((96, 72), 0, 1e-3), ((128, 96), 1, 4e-4)]
    out = []
    for i, ((w, h), terr, dur) in enumerate(spec):
        cam = dict(width=w, height=h, fx=0.8 * w, fy=0.8 * w, cx=w / 2, cy=h / 2)
        path = FlickerPass((-50.0 + 10 * i, 5.0 * i, 500.0 + 50 * i), (300.0, 40.0 * i, 0.0), light, 1e5)
        out.append(serve.Job(i, 0.001 * i, terr, cam, 1 + i % 2, dur, 1e-5, path, dict(PHYSIC, random_seed=10 + i)))
    return out


def events_by_job(done):
    return {j.job_id: j.events for j in done}


def test_jobs_give_the_same_events_alone_and_in_the_mix(pool):
    alone = {}
    for j in jobs():
        srv = serve.Server(pool, hbm_budget=8 << 30, horizons_per_step=16, max_active=1)
        alone.update(events_by_job(srv.run([j], realtime=False)))
    assert sum(len(e) for e in alone.values()) > 100
    mixed_server = serve.Server(pool, hbm_budget=8 << 30, horizons_per_step=16, max_active=8)
    mixed = events_by_job(mixed_server.run(jobs(), realtime=False))
    assert mixed_server.peak_active == 6
    budget = max(mixed_server.estimate_bytes(j) for j in jobs()) * 2 + 1
    tight_server = serve.Server(pool, hbm_budget=budget, horizons_per_step=16, max_active=8)
    tight = events_by_job(tight_server.run(jobs(), realtime=False))
    assert 1 <= tight_server.peak_active < 6 and tight_server.peak_used <= budget
    fair = events_by_job(serve.Server(pool, hbm_budget=8 << 30, horizons_per_step=16, policy="fair",
                                      fill_samples=1).run(jobs(), realtime=False))
    for k, ev in alone.items():
        for other in (mixed[k], tight[k], fair[k]):
            assert len(other) == len(ev)
            for f in ev.dtype.names:
                assert np.array_equal(other[f], ev[f]), (k, f)


def test_realtime_stream_latency(pool):
    js = jobs()
    done = serve.Server(pool, hbm_budget=8 << 30, horizons_per_step=16).run(js, realtime=True)
    lat = serve.latency_summary(done)
    assert all(j.finished >= j.admitted >= j.arrival - 1e-3 for j in done)
    assert 0 < lat["p50_ms"] <= lat["p99_ms"] <= lat["max_ms"]
    assert all(j.rays > 0 and j.device_bytes > 0 for j in done)


def test_scene_views_share_geometry(pool):
    base = pool[1]
    cam = dict(width=96, height=72, fx=77.0, fy=77.0, cx=48.0, cy=36.0)
    view = base.view(cam, 2)
    V, N, I = terrain.terrain_mesh(96, 2)
    own = DeviceScene(V, N, I, cam, 2, HAPKE)
    pose = dict(position=(3.0, -2.0, 600.0), rotation=(0.0, 0.0, 0.0, 1.0), light=trajectory.sun_direction(30, 40),
                intensity=1000)
    a, da = CamRayCaster(view).render_state(pose)
    b, db = CamRayCaster(own).render_state(pose)
    assert np.array_equal(a, b) and np.array_equal(da, db)
    assert view.info()["device_bytes"] < own.info()["device_bytes"] // 10
    view2 = base.view(cam, 1)
    del view
    c, _ = CamRayCaster(view2).render_state(pose)  # geometry outlives the first view
    assert (c > 0).mean() > 0.5
    assert math.isfinite(float(c.sum()))
