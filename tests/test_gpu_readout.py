"""The device readout FIFO (dvs_device_readout_*, and the sensors' default
readout) against the reference's FIFO (src/event_readout.cpp:6-34).

Pinned three ways: the reference's own outputs in tests/golden/readout.npz
(four bandwidth / latency / capacity regimes, two of them dropping events),
the host restatement (dvs_readout_*, serial) on large random streams with and
without drops, and whole sensors with the device and the host readout.
Order, x, y, polarity, drops and peak are exact; delivery times are the same
FP64 sums grouped as a scan -- they differ from the serial chain of additions
by at most the chain's rounding (below 1e-11 s here) -- and are compared to
1 ns.  Arrival times on a coarse grid are used only without FIFO delay: with
a saturated bus they would put delivery and arrival times on one grid, where
the serial FIFO's exact comparisons depend on that rounding.
"""
import os

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import EventSensor
from dvsrender4deepspace_gb300._capi import EVENT_DTYPE
from dvsrender4deepspace_gb300.raycast import EventReadout
from tests.test_gpu_parity import plane_sensor
from tests.test_oracle_golden import POSE

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "readout.npz")


def same_stream(got, want, delayed):
    assert len(got) == len(want)
    for f in ("x", "y", "polarity", "depth"):
        np.testing.assert_array_equal(got[f], want[f])
    if delayed:
        np.testing.assert_allclose(got["timestamp"], want["timestamp"], rtol=0, atol=1e-9)
    else:
        np.testing.assert_array_equal(got["timestamp"], want["timestamp"])


def test_device_readout_reproduces_the_reference_fixtures():
    g = np.load(GOLDEN)
    for k in range(4):
        bw, lat, cap = g["s%d_cfg" % k]
        r = EventReadout(bw, lat, int(cap), device=True, max_batch=4096)
        for b in range(3):
            out = r.submit(g["s%d_in%d" % (k, b)], float(g["s%d_now%d" % (k, b)]))
            same_stream(out, g["s%d_out%d" % (k, b)], bw > 0)
        same_stream(r.drain(), g["s%d_drain" % k], bw > 0)
        assert r.dropped() == int(g["s%d_dropped" % k])
        assert r.peak_queue() == int(g["s%d_peak" % k])


def random_events(rng, n, t0, t1, width=1280, height=720, ties=False):
    ev = np.zeros(n, EVENT_DTYPE)
    t = rng.uniform(t0, t1, n)
    if ties:  # many events at the same instants: (y, x) breaks the ties
        t = np.round(t * 1e5) / 1e5
    ev["timestamp"] = t
    ev["x"] = rng.integers(0, width, n)
    ev["y"] = rng.integers(0, height, n)
    ev["polarity"] = rng.integers(0, 2, n)
    ev["depth"] = rng.uniform(10, 1000, n).astype(np.float32)
    return ev


@pytest.mark.parametrize("bandwidth,latency,capacity,ties", [
    (0.0, 0.0, 1000, True),           # no FIFO delay: (t, y, x) order only
    (5e6, 18e-9, 1_000_000, False),   # the configs' bus: never full
    (2e5, 1e-6, 1_000_000, False),    # saturated bus: long busy periods, no drops
    (1e5, 1e-6, 300, False),          # small queue: drops (serial pass on the device)
])
def test_device_readout_equals_the_host_fifo(bandwidth, latency, capacity, ties):
    rng = np.random.default_rng(17)
    dev = EventReadout(bandwidth, latency, capacity, device=True, max_batch=200_000)
    host = EventReadout(bandwidth, latency, capacity)
    t = 0.0
    for batch in range(6):
        n = int(rng.integers(1, 150_000)) if batch != 3 else 0
        ev = random_events(rng, n, t, t + 0.01, ties=ties)
        t += 0.01
        same_stream(dev.submit(ev, t), host.submit(ev, t), bandwidth > 0)
        assert dev.dropped() == host.dropped() and dev.peak_queue() == host.peak_queue()
    same_stream(dev.drain(), host.drain(), bandwidth > 0)
    if capacity == 300:
        assert host.dropped() > 0


@pytest.mark.parametrize("bandwidth,latency,capacity", [
    (0.0, 0.0, 1000),                # no FIFO delay
    (1e12, 0.0, 1 << 24),            # unbounded bus: the parallel path, nothing pending
    (5e9, 18e-9, 1_000_000),         # busy bus, no drops: completions carried across batches
    (5e8, 1e-6, 20_000),             # saturated bus with drops (serial pass)
])
def test_device_readout_packed_keys_equal_the_host_fifo(bandwidth, latency, capacity):
    """Batches of one 64 us window of a 1280x720 sensor at t ~ 1 s (the
    readout workload's shape): the varying bits of t, y and x fit one 64-bit
    key, so the device sorts on the packed key (the wide batches of the test
    above take the two-key sort)."""
    rng = np.random.default_rng(23)
    dev = EventReadout(bandwidth, latency, capacity, device=True, max_batch=300_000)
    host = EventReadout(bandwidth, latency, capacity)
    t = 1.0
    for batch in range(5):
        n = int(rng.integers(1, 250_000)) if batch != 2 else 1
        ev = random_events(rng, n, t, t + 64e-6, ties=batch == 3 and bandwidth == 0)  # ties: (y, x) decides
        t += 64e-6
        same_stream(dev.submit(ev, t), host.submit(ev, t), bandwidth > 0)
        assert dev.dropped() == host.dropped() and dev.peak_queue() == host.peak_queue()
    same_stream(dev.drain(), host.drain(), bandwidth > 0)
    if capacity == 20_000:
        assert host.dropped() > 0


def test_device_readout_refuses_oversized_batches():
    r = EventReadout(1e6, 0.0, 100, device=True, max_batch=16)
    with pytest.raises(ValueError):
        r.submit(random_events(np.random.default_rng(1), 17, 0.0, 1.0), 1.0)


def test_sensor_device_readout_equals_host_readout():
    """A sensor with the device FIFO (the default) and one with the host FIFO
    deliver the same events through a finite bus."""
    scene, phys = plane_sensor(readout_bandwidth=2e6, readout_latency=1e-6, readout_queue_capacity=5000,
                               threshold_pos=0.05, threshold_neg=0.05)
    start, end = dict(POSE, intensity_rate=8e6), dict(POSE, intensity_rate=-8e6)
    ivs = [(POSE, POSE, 0, 0.001), (start, end, 0.001, 0.003), (POSE, POSE, 0.003, 0.004)]
    dev, host = EventSensor(scene, phys), EventSensor(scene, phys, host_readout=True)
    for s in (dev, host):
        s.initialize(POSE, 0)
    got = [dev.process(iv) for iv in ivs] + [dev.drain()]
    want = [host.process(iv) for iv in ivs] + [host.drain()]
    assert sum(len(w) for w in want) > 1000
    for a, b in zip(got, want):
        same_stream(a, b, True)
    sd, sh = dev.stats(), host.stats()
    assert sd["dropped"] == sh["dropped"] and sd["peak_queue"] == sh["peak_queue"]
    assert sd["events_delivered"] == sh["events_delivered"]
