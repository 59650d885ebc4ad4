"""One sensor over several GPUs.

Pixels are independent (each has its own circuit state, RNG stream and event
slab), so rank r of a world of N simulates the rows of band r
(``dvs_sensor_options.row_begin/row_end``) with the scene replicated on every
GPU.  The only coupling is the readout bus: the reference's FIFO serializes
the events of all pixels (src/event_readout.cpp:13-26), so the ranks' raw
event runs (readout bypassed) are gathered on rank 0, merged into (t, y, x)
order and read out there.  With the readout bandwidth at 0 the merge alone
reproduces the single-GPU stream.  No GPU collective is involved: the event
runs travel through the host process group.
"""
import numpy as np

from ._capi import EVENT_DTYPE


def row_bands(height, world):
    """Contiguous row ranges, one per rank, sizes differing by at most one."""
    base, extra = divmod(int(height), int(world))
    out, r0 = [], 0
    for r in range(world):
        r1 = r0 + base + (1 if r < extra else 0)
        out.append((r0, r1))
        r0 = r1
    return out


def merge_runs(runs):
    """Merges event arrays into one array ordered by (timestamp, y, x)."""
    runs = [np.asarray(r, EVENT_DTYPE) for r in runs if len(r)]
    if not runs:
        return np.zeros(0, EVENT_DTYPE)
    ev = np.concatenate(runs)
    return ev[np.lexsort((ev["x"], ev["y"], ev["timestamp"]))]


class ShardedReadout:
    """The readout bus of a sensor split over the ranks of a process group.

    submit() is collective: every rank passes its raw events of one batch;
    rank 0 returns the events delivered by `now`, the other ranks an empty
    array."""

    def __init__(self, dist, bandwidth, latency, capacity, group=None):
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.bus = None
        if self.rank == 0:
            from .raycast import EventReadout
            self.bus = EventReadout(bandwidth, latency, capacity)

    def _gather(self, events):
        runs = [None] * self.world if self.rank == 0 else None
        self.dist.gather_object(np.asarray(events, EVENT_DTYPE), runs, dst=0, group=self.group)
        return runs

    def submit(self, events, now):
        runs = self._gather(events)
        if self.rank != 0:
            return np.zeros(0, EVENT_DTYPE)
        return self.bus.submit(merge_runs(runs), now)

    def drain(self):
        return self.bus.drain() if self.rank == 0 else np.zeros(0, EVENT_DTYPE)

    def dropped(self):
        return self.bus.dropped() if self.rank == 0 else 0
