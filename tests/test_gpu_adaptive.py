"""GPU adaptive optics against the native path, the reference's own checks
(tests/test_sensor.cu:94-159) at the DAVIS346 resolution with one spatial
sample: static reuse is exact, an interior pulse converges, a discontinuity
is resolved with local exact cells, and the convergence gate rejects a window
before any pixel or RNG state changes."""
import numpy as np
import pytest

from dvsrender4deepspace_gb300 import EventSensor
from tests.test_gpu_parity import pixel_sorted, plane_sensor
from tests.test_oracle_golden import DAVIS, POSE

pytestmark = pytest.mark.gpu
N_PIX = DAVIS["width"] * DAVIS["height"]


def same_events(a, b, tol=0.0):
    assert len(a) == len(b)
    for f in ("x", "y", "polarity"):
        np.testing.assert_array_equal(a[f], b[f])
    if len(a):
        assert np.max(np.abs(a["timestamp"] - b["timestamp"])) <= tol


@pytest.mark.parametrize("shot", [0, 1])
def test_adaptive_static_reuses_optics_exactly(shot):
    scene, phys = plane_sensor(photon_shot_noise=shot, circuit_step=1e-6)
    native, adaptive = EventSensor(scene, phys), EventSensor(scene, phys)
    native.initialize(POSE, 0)
    adaptive.initialize(POSE, 0)
    ivs = [(POSE, POSE, 0, .001), (POSE, POSE, .001, .002)]
    exact = native.process_many(ivs)
    cached = adaptive.process_adaptive(ivs, .001)
    st = adaptive.refinement_statistics()
    assert st["fallback_pixels"] == 0 and st["maximum_knots"] == 5
    same_events(exact, cached)
    assert adaptive.adaptive_cache_capacity() in (128, 256, 512)


def test_adaptive_interior_pulse_converges():
    scene, phys = plane_sensor(photon_shot_noise=0, circuit_step=1e-6)
    native, adaptive = EventSensor(scene, phys), EventSensor(scene, phys)
    native.initialize(POSE, 0)
    adaptive.initialize(POSE, 0)
    start, end = dict(POSE, intensity_rate=8e6), dict(POSE, intensity_rate=-8e6)
    ivs = [(start, end, 0, .002)]
    exact = pixel_sorted(native.process_many(ivs))
    cached = adaptive.process_adaptive(ivs, 1e-4)
    st = adaptive.refinement_statistics()
    assert st["fallback_pixels"] < N_PIX
    assert len(cached) > 0
    cached = pixel_sorted(cached)
    key = lambda e: (e["y"].astype(np.int64) * DAVIS["width"] + e["x"])
    ke, kc = key(exact), key(cached)
    different, worst = 0, 0.0
    ue, ce = np.unique(ke, return_counts=True)
    uc, cc = np.unique(kc, return_counts=True)
    ne, nc = dict(zip(ue, ce)), dict(zip(uc, cc))
    for p in set(ne) | set(nc):
        if ne.get(p, 0) != nc.get(p, 0):
            different += 1
            continue
        a, b = exact[ke == p], cached[kc == p]
        np.testing.assert_array_equal(a["polarity"], b["polarity"])
        worst = max(worst, float(np.max(np.abs(a["timestamp"] - b["timestamp"]))))
    assert different < N_PIX * .001
    assert worst < 3 * 1e-6


def test_adaptive_discontinuity_uses_local_exact_cells():
    scene, phys = plane_sensor(photon_shot_noise=0, circuit_step=1e-6)
    native, adaptive = EventSensor(scene, phys), EventSensor(scene, phys)
    native.initialize(POSE, 0)
    adaptive.initialize(POSE, 0)
    bright = dict(POSE, intensity=2000)
    ivs = [(POSE, POSE, 0, .001), (bright, bright, .001, .002)]
    exact = native.process_many(ivs)
    cached = adaptive.process_adaptive(ivs, 1e-4)
    st = adaptive.refinement_statistics()
    assert st["native_cell_queries"] > 0 and st["fallback_pixels"] == 0
    same_events(pixel_sorted(exact), pixel_sorted(cached), tol=2e-12)


def test_convergence_gate_rejects_before_state_changes():
    scene, phys = plane_sensor(photon_shot_noise=1, circuit_step=1e-6)
    checked, fresh = EventSensor(scene, phys), EventSensor(scene, phys)
    checked.initialize(POSE, 0)
    fresh.initialize(POSE, 0)
    flash = dict(POSE, intensity=20000)  # strictly between the five initial probes
    ivs = [(POSE, POSE, 0, .0003), (flash, flash, .0003, .0004), (POSE, POSE, .0004, .002)]
    assert checked.process_adaptive(ivs, .5, check_convergence=True) is None
    conv = checked.last_convergence()
    assert conv["pixels"] == 1024 and conv["maximum_log_voltage_error"] > 0
    retried = checked.process_many(ivs)
    exact = fresh.process_many(ivs)
    same_events(exact, retried)
    assert len(exact) > 0


def test_adaptive_rejects_invalid_requests():
    scene, phys = plane_sensor(photon_shot_noise=0)
    s = EventSensor(scene, phys)
    s.initialize(POSE, 0)
    with pytest.raises(ValueError):
        s.process_adaptive([(POSE, POSE, 0, .001)], 0.0)          # tolerance must be positive
    with pytest.raises(ValueError):
        s.process_adaptive([(POSE, POSE, 0, .05)], 1e-3)          # window beyond the event capacity bound
    scene2, phys2 = plane_sensor(refractory_time=0)
    t = EventSensor(scene2, phys2)
    t.initialize(POSE, 0)
    with pytest.raises(ValueError):
        t.process_adaptive([(POSE, POSE, 0, .001)], 1e-3)         # needs a refractory period
