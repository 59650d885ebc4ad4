"""Multi-GPU event path on CPU ranks (gloo, world size 2): each rank owns a
band of sensor rows, the raw event runs are merged on rank 0 and read out
through one FIFO; the result must equal the single-sensor stream.  The
per-band events come from the oracle (pixels are independent), so this
exercises the sharding, the merge and the bus without a GPU."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from dvsrender4deepspace_gb300 import shard  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_row_bands_cover_rows_once():
    for h, w in ((260, 2), (260, 3), (720, 8), (5, 8)):
        bands = shard.row_bands(h, w)
        assert bands[0][0] == 0 and bands[-1][1] == h
        assert all(a[1] == b[0] for a, b in zip(bands, bands[1:]))
        sizes = [b[1] - b[0] for b in bands]
        assert max(sizes) - min(sizes) <= 1


def oracle_raw_events():
    from tests.test_oracle_golden import POSE, _plane_sensor
    from oracle import oracle as O
    sc, phys = _plane_sensor(crop=(48, 32))
    s = O.OracleSensor(sc, phys)  # readout bandwidth 0: the raw crossing events
    s.initialize(POSE, 0)
    start, end = dict(POSE, intensity_rate=8e6), dict(POSE, intensity_rate=-8e6)
    ivs = [(POSE, POSE, 0, .001), (start, end, .001, .003)]
    return s.process(ivs), sc.s.height, ivs[-1][3]


def _worker(rank, world, port, q):
    try:
        os.environ["MASTER_ADDR"] = "127.0.0.1"
        os.environ["MASTER_PORT"] = str(port)
        dist.init_process_group("gloo", rank=rank, world_size=world)
        raw, height, now = oracle_raw_events()
        r0, r1 = shard.row_bands(height, world)[rank]
        mine = raw[(raw["y"] >= r0) & (raw["y"] < r1)]
        bus = shard.ShardedReadout(dist, 2e5, 1e-5, 64)
        ready = bus.submit(mine, now)
        tail = bus.drain()
        if rank == 0:
            from dvsrender4deepspace_gb300.raycast import EventReadout
            single = EventReadout(2e5, 1e-5, 64)
            want = np.concatenate([single.submit(raw, now), single.drain()])
            got = np.concatenate([ready, tail])
            ok = len(got) == len(want) and all(np.array_equal(got[f], want[f]) for f in want.dtype.names)
            q.put((ok, len(want), bus.dropped(), single.dropped()))
        dist.barrier()
        dist.destroy_process_group()
    except Exception as e:  # report to the parent instead of hanging it
        q.put((False, repr(e), -1, -1))


def test_two_rank_merge_matches_single_sensor():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, n, dropped, single_dropped = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
    assert ok, n
    assert n > 0 and dropped == single_dropped > 0  # the small FIFO drops the same events
