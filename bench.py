"""Benchmark of the DVS hot path on one GB300 (or N, one rank per GPU).

Workload (default "precision"): Prophesee 1280x720 (fx=fy=1000, cx=640,
cy=360) over a seeded 4096x4096-vertex fBm+crater heightfield (33.5M
triangles, 10 m spacing), supersample 16 (config/prophesee.yaml), a 2 s
descent from 3 km to 500 m, 1 us horizons and circuit cells.  A step is one
native batch of 64 horizons (apps/main_dvs.cpp:294-296) = 64 us of simulated
time.  The scene (several GB) is far larger than L2, so no flush is needed.

value  = primary + shadow rays traced per second of device time (CUDA events
         on the sensor's stream around K enqueued steps; inputs resident).
e2e    = the same metric through dvs_sensor_process_events with host
         intervals in and host events out (copies and readout included).
cpu_baseline / --impl reference = the oracle port (the reference has no CPU
         renderer) timed with all host threads on a bounded sample of the
         same workload's pixel-cells.
Multi-GPU: one rank per GPU, each an independent job (the reference runs one
sequence per GPU, tools/run_sequences.py:247-256): weak scaling, no
collective on the data path.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# dvs_bvh_params.precision flags: 1 = FP16 child bounds, 2 = watertight triangle test
GEOMETRY = {"reference": 0, "half": 1, "watertight": 2, "half+watertight": 3}
# dvs_bvh_params.builder
BUILDERS = {"sah": 0, "morton": 1}
BUILDERS_TEXT = {0: "binned SAH splits", 1: "Morton radix splits"}

WORKLOADS = {
    # configs: precision (1280x720), small (346x260 DAVIS, plain method)
    "precision": dict(grid=4096, seed=20260003, camera=dict(width=1280, height=720, fx=1000.0, fy=1000.0, cx=640.0,
                                                            cy=360.0),
                      ss=16, z0=3000.0, z1=500.0, duration=2.0, ground_speed=80.0, sun_elevation=30.0,
                      intensity=1000.0, time_resolution=1e-6, batch=64,
                      # precision traversal: quantised FP16 child bounds and the watertight FP32 triangle
                      # test; FP32 receptor arithmetic with Philox noise
                      geometry="half+watertight", circuit="fp32-philox"),
    # one trajectory of the batching config: 1024^2 terrain (2.09M triangles), ss 4, 10 us horizons
    "orbit": dict(grid=1024, seed=20260002, camera=dict(width=346, height=260, fx=300.0, fy=300.0, cx=173.0,
                                                        cy=130.0),
                  ss=4, z0=1500.0, z1=1500.0, duration=2.0, ground_speed=100.0, sun_elevation=30.0,
                  intensity=1000.0, time_resolution=1e-5, batch=64,
                  geometry="reference", circuit="fp32"),  # FP32 pixel state, FP64 timestamps
    "small": dict(grid=256, seed=20260001, camera=dict(width=346, height=260, fx=300.0, fy=300.0, cx=173.0, cy=130.0),
                  ss=1, z0=1000.0, z1=1000.0, duration=0.49, ground_speed=50.0, sun_elevation=30.0, intensity=1.0,
                  time_resolution=1e-5, batch=64, geometry="reference", circuit="fp64"),
    # the large config: 8192^2 terrain (134M triangles), 1280x720, 4^2 sub-rays, a 10 s level traverse
    # 300 m above the highest terrain of its corridor at 80 m/s, sun 5 deg above the horizon (long
    # shadows, dense events), physic effects and the AER readout on; FP32 receptor arithmetic with
    # FP64 timestamps and crossing solves
    "large": dict(grid=8192, seed=20260005, camera=dict(width=1280, height=720, fx=1000.0, fy=1000.0, cx=640.0,
                                                        cy=360.0),
                  ss=4, altitude_agl=300.0, duration=10.0, ground_speed=80.0, sun_elevation=5.0, intensity=1000.0,
                  time_resolution=1e-6, batch=64, geometry="half+watertight", circuit="fp32"),
}
HAPKE = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)
PHYSIC = dict(threshold_pos=0.2, threshold_neg=0.2, refractory_time=200e-6, readout_bandwidth=5e6,
              readout_latency=18e-9, threshold_std=0.03, threshold_min=0.01, wavelength_nm=550,
              quantum_efficiency=0.3, pixel_pitch_um=15, fill_factor=0.2, f_number=2.0, lens_transmission=0.8,
              radiance_scale=0.001, temperature_k=300, subthreshold_kappa=0.8, receptor_capacitance_f=1e-15,
              reset_capacitance_f=20e-15, dark_current_a=1e-18, reset_leakage_a=0, circuit_step=1e-6,
              photon_shot_noise=1, reset_thermal_noise=0, random_seed=114514, max_events_per_step=16,
              readout_queue_capacity=1000000)
METRIC = "DVS events/s and Mrays/s at 1280x720 on 1 GB300; serving p99 latency vs plain path"
# ncu counters of one full-size trace_cells_kernel launch (one native batch),
# by (workload, BVH format, BVH builder, cells per warp, rays per lane): warp
# instructions (smsp__inst_executed.sum) per traced ray (primary + shadow, as
# the sensor counted them), and DRAM bytes read + written
# (dram__bytes_read.sum + dram__bytes_write.sum) per pixel-cell.  Radiance
# writes still held in L2 when the kernel ends are not in the DRAM count.
TRACE_WARP_INSTRUCTIONS_PER_RAY = {
    ("precision", "half+watertight", "sah", 32, 2): 1466157173123 / 29471262019,
    ("orbit", "reference", "sah", 32, 2): 79970172908 / 1768685229,
}
TRACE_DRAM_BYTES_PER_PIXEL_CELL = {
    ("precision", "half+watertight", "sah", 32, 2): (66908416 + 219526144) / (921600 * 64),
    ("orbit", "reference", "sah", 32, 2): (14630400 + 178991360) / (89960 * 640),
}
# ncu DRAM counters (dram__bytes_read.sum + dram__bytes_write.sum) of the 44
# launches of one device-readout batch of 4,194,304 events (the readout
# workload's batch), per event: the sort's passes, the FIFO scan and the release.
READOUT_DRAM_BYTES_PER_EVENT = (1489862912 + 310624256) / 4194304
GB300_SMS = 152


def readout_roofline(peak, n_events=1 << 22, batches=4):
    """The device readout FIFO on a large synthetic batch: n_events events of
    a 1280x720 sensor within one 64 us batch.  The configs' 5e6 s^-1 bus would
    saturate and drop at that density (the serial path); an unbounded bus
    (1e12 s^-1) keeps the parallel path -- radix sort, max-plus scan,
    occupancy, release.  Device time from CUDA events around the kernels.
    Algorithmic bytes per event: the event read once and delivered once."""
    from dvsrender4deepspace_gb300._capi import EVENT_DTYPE
    from dvsrender4deepspace_gb300.raycast import EventReadout
    rng = np.random.default_rng(5)
    r = EventReadout(1e12, 0.0, 1 << 24, device=True, max_batch=n_events)
    times, t = [], 1.0
    for b in range(batches + 1):
        ev = np.zeros(n_events, EVENT_DTYPE)
        ev["timestamp"] = t + rng.uniform(0.0, 64e-6, n_events)
        ev["x"] = rng.integers(0, 1280, n_events)
        ev["y"] = rng.integers(0, 720, n_events)
        ev["polarity"] = rng.integers(0, 2, n_events)
        t += 64e-6
        out = r.submit(ev, t)
        assert len(out) == n_events
        if b:  # the first batch warms the kernels and sizes the sort grid
            times.append(r.last_ms())
    ms = statistics.median(times)
    alg = n_events * 2 * 24.0
    return {"bound": "hbm", "kernel": "device readout (radix sort, max-plus scan, release)",
            "achieved": alg / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / peak,
            "ms_per_batch": ms, "events_per_batch": n_events, "events_per_s": n_events / (ms / 1e3),
            "algorithmic_bytes": alg, "traffic": READOUT_DRAM_BYTES_PER_EVENT * n_events,
            "traffic_gbs": READOUT_DRAM_BYTES_PER_EVENT * n_events / (ms / 1e3) / 1e9}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def make_workload(name, rank=0):
    from dvsrender4deepspace_gb300 import terrain, trajectory
    w = WORKLOADS[name]
    V, N, I = terrain.terrain_mesh(w["grid"], w["seed"])
    light = trajectory.sun_direction(w["sun_elevation"], 35.0)
    # each rank flies its own job over the same terrain (offset start)
    x0 = -2000.0 + 1000.0 * rank if w["grid"] >= 1024 else 0.0
    z0, z1 = w.get("z0"), w.get("z1")
    if w.get("altitude_agl"):  # level flight above the highest terrain of the flight corridor (+-300 m)
        x1 = x0 + w["ground_speed"] * w["duration"]
        corridor = (V[:, 0] > x0 - 300) & (V[:, 0] < x1 + 300) & (np.abs(V[:, 1]) < 300)
        z0 = z1 = float(V[corridor, 2].max()) + w["altitude_agl"]
    traj = trajectory.Descent((x0, 0.0), z0, z1, w["duration"], w["ground_speed"], light, w["intensity"])
    return w, V, N, I, traj


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(name, V, N, I, traj, w, budget_s=15.0, threads=0, osc=None, build_s=None, fp64=False):
    """Oracle port on a bounded sample of the workload's pixel-cells: the
    optics only (primary + shadow rays with Hapke shading; the circuit, a
    negligible share of the CPU time, is not in the sample), in the
    reference's FP32 ray arithmetic or, with fp64, the FP64 oracle's.
    Returns Mrays/s and the sample description."""
    from oracle import oracle as O
    cam = w["camera"]
    if osc is None:
        t_build = time.time()
        osc = O.OracleScene(V, N, I, cam, w["ss"], HAPKE, max_leaf=64, fp64=fp64)
        build_s = time.time() - t_build
    rng = np.random.default_rng(7)
    n_pix = cam["width"] * cam["height"]
    nthreads = threads or os.cpu_count()
    total_rays, total_t, cells = 0, 0.0, 0
    batch = 1024
    while total_t < budget_s and cells < 10000:
        t = cells * w["time_resolution"]
        pix = rng.choice(n_pix, size=batch, replace=False).astype(np.int32)
        t0 = time.perf_counter()
        _, _, prim, shad = osc.render_pixels(traj.state(t), pix, nthreads)
        total_t += time.perf_counter() - t0
        total_rays += prim + shad
        cells += 1
    return {"value": total_rays / total_t / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
            "scope": "optics only (rays + Hapke), %s oracle port" % ("FP64" if fp64 else "FP32"),
            "sample": "%d pixel-cells (%d random pixels x %d cell times, ss=%d), %.1f s of CPU work; oracle "
                      "binary BVH (leaf 64) built in %.1f s" % (batch * cells, batch, cells, w["ss"], total_t, build_s)}


def precision_errors(V, N, I, traj, w, scene, geometry, circuit, budget_pixels=2048, threads=0, o64=None):
    """The precision config's accuracy statement, measured: the GPU path's
    radiance and depth on a seeded sample of the config's pixels (one pose,
    all sub-rays) against the FP64 oracle, and its events on a crop of the
    config's camera through a light pulse against the FP64 oracle sensor
    (deterministic physics: no shot noise, no threshold mismatch, no FIFO
    delay -- the oracle cannot reproduce device random streams)."""
    from dvsrender4deepspace_gb300 import CamRayCaster, EventSensor
    from oracle import oracle as O
    nthreads = threads or os.cpu_count()
    cam = w["camera"]
    if o64 is None:
        o64 = O.OracleScene(V, N, I, cam, w["ss"], HAPKE, max_leaf=64, fp64=True,
                            watertight=bool(GEOMETRY[geometry] & 2))
    out = {"oracle": "FP64 (geometry, rays, Hapke in double; binary BVH leaf 64)",
           "geometry": geometry, "circuit_precision": circuit}
    # radiance and depth: one pose, seeded pixel sample, with the oracle's
    # margin classes (optical margin, conditioning, crack) named per pixel
    pose = traj.state(0.0)
    img, dep = CamRayCaster(scene).render_state(pose)
    rng = np.random.default_rng(11)
    pix = rng.choice(cam["width"] * cam["height"], size=budget_pixels, replace=False).astype(np.int32)
    t_cls = time.time()
    orad, odep, margin = o64.render_margin(pose, pix, nthreads=nthreads)
    out["classifier_seconds"] = time.time() - t_cls
    g_rad, g_dep = img.reshape(-1)[pix].astype(np.float64), dep.reshape(-1)[pix].astype(np.float64)
    lit = orad > 0
    rel = np.where(lit, np.abs(g_rad - orad) / np.where(lit, orad, 1.0), 0.0)
    hit = odep > 0
    drel = np.where(hit, np.abs(g_dep - odep) / np.where(hit, odep, 1.0), 0.0)
    plain = margin == 0
    classes = {"optical": int(np.count_nonzero(margin & O.MARGIN_OPTICAL)),
               "conditioning": int(np.count_nonzero(margin & O.MARGIN_CONDITIONING)),
               "crack": int(np.count_nonzero(margin & O.MARGIN_CRACK))}
    out["radiance"] = {"pixels": int(lit.sum()), "max_rel": float(rel[lit].max()),
                       "p99_rel": float(np.quantile(rel[lit], .99)), "above_1e-5": int((rel > 1e-5).sum()),
                       "margin_pixels": int((~plain).sum()), "margin_classes": classes,
                       "non_margin_above_1e-5": int(((rel > 1e-5) & plain).sum()),
                       "max_rel_non_margin": float(rel[lit & plain].max())}
    out["depth"] = {"pixels": int(hit.sum()), "max_rel": float(drel[hit].max()),
                    "p99_rel": float(np.quantile(drel[hit], .99)), "above_1e-5": int((drel > 1e-5).sum()),
                    "non_margin_above_1e-5": int(((drel > 1e-5) & plain).sum()),
                    "misses_agree_non_margin": bool(np.all(((g_dep < 0) == (odep < 0)) | ~plain))}
    # events: a 16x12 crop through a 0.5 ms light pulse (500 cells of 1 us), at the
    # fully lit window nearest the image centre (with a low sun the centre can lie in
    # shadow, where a pulse gives no events), else at the centre
    lit = np.pad((img.reshape(cam["height"], cam["width"]) > 0).astype(np.int64), ((1, 0), (1, 0)))
    S = lit.cumsum(0).cumsum(1)
    x0, y0 = cam["width"] // 2 - 8, cam["height"] // 2 - 6

    def fully_lit(xx, yy):
        return S[yy + 12, xx + 16] - S[yy, xx + 16] - S[yy + 12, xx] + S[yy, xx] == 16 * 12
    best = (0, x0, y0) if fully_lit(x0, y0) else None
    for yy in range(0, cam["height"] - 12 + 1, 4):
        for xx in range(0, cam["width"] - 16 + 1, 4):
            if best is None or (xx - x0) ** 2 + (yy - y0) ** 2 < best[0]:
                if fully_lit(xx, yy):
                    best = ((xx - x0) ** 2 + (yy - y0) ** 2, xx, yy)
    if best is not None:
        x0, y0 = best[1], best[2]
    crop = dict(cam, width=16, height=12, cx=cam["cx"] - x0, cy=cam["cy"] - y0)
    phys = dict(PHYSIC, photon_shot_noise=0, threshold_std=0, readout_bandwidth=0, readout_latency=0,
                max_events_per_step=64)
    sensor = EventSensor(scene.view(crop, w["ss"]), phys, circuit_precision=circuit)
    ors = O.OracleSensor(o64.with_camera(crop), phys, margin=True)
    sensor.initialize(pose, 0.0)
    ors.initialize(pose, 0.0, nthreads)
    a, b = dict(pose, intensity_rate=1.6e8), dict(traj.state(5e-4), intensity_rate=-1.6e8)
    ivs = [(a, b, 0.0, 5e-4)]
    t0 = time.time()
    gev = np.concatenate([sensor.process_many(ivs), sensor.drain()])
    oev = np.concatenate([ors.process(ivs, nthreads), ors.drain()])
    cpu_s = time.time() - t0
    margins = ors.margins()

    def per_pixel(ev):
        d = {}
        for e in ev:
            d.setdefault((int(e["x"]), int(e["y"])), []).append((float(e["timestamp"]), int(e["polarity"])))
        return d
    pg, po = per_pixel(gev), per_pixel(oev)
    same, unclassified, worst = 0, 0, 0.0
    for key in set(pg) | set(po):
        x, y = pg.get(key, []), po.get(key, [])
        flagged = margins[key[1] * crop["width"] + key[0]] != 0
        if [p for _, p in x] == [p for _, p in y]:
            same += 1
            if x and not flagged:
                worst = max(worst, max(abs(u - v) for (u, _), (v, _) in zip(x, y)))
        elif not flagged:
            unclassified += 1
    n_px = len(set(pg) | set(po))
    out["events"] = {"crop": "16x12 at (%d, %d)" % (x0, y0), "interval": "0.5 ms pulse, 500 cells",
                     "gpu_events": int(len(gev)), "oracle_events": int(len(oev)), "pixels_with_events": n_px,
                     "pixels_same_polarity_sequence": same, "margin_pixels": int((margins != 0).sum()),
                     "non_margin_sequence_mismatches": unclassified,
                     "max_timestamp_error_s_non_margin": worst, "oracle_seconds": cpu_s}
    return out


def bench_config(args, w, n_triangles, world):
    """The workload's `config` block, the same for both arms."""
    return {"workload": args.workload, "pixels": w["camera"]["width"] * w["camera"]["height"],
            "width": w["camera"]["width"], "height": w["camera"]["height"], "supersample": w["ss"],
            "terrain_grid": w["grid"], "triangles": int(n_triangles), "horizons_per_step": w["batch"],
            "time_resolution": w["time_resolution"], "circuit_step": PHYSIC["circuit_step"],
            "shot_noise": "philox" if args.circuit == "fp32-philox" else "curand_xorwow",
            "sun_elevation_deg": w["sun_elevation"], "intensity": w["intensity"],
            "l2": "inputs larger than L2 (129 MB): the triangle and shading records alone are %.2f GB"
                  % (n_triangles * (48 * (3 if GEOMETRY[args.geometry] & 2 else 1) + 64) / 1e9),
            "parallelism": "dp%d (independent jobs)" % world, "geometry": args.geometry,
            "bvh_builder": args.builder, "circuit_precision": args.circuit}


def run_reference(args):
    from oracle import oracle as O
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    w, V, N, I, traj = make_workload(args.workload)
    t_build = time.time()
    osc = O.OracleScene(V, N, I, w["camera"], w["ss"], HAPKE, max_leaf=64)   # built once for all steps
    build_s = time.time() - t_build
    res = []
    for step in range(args.warmup + args.steps):
        cb = cpu_baseline(args.workload, V, N, I, traj, w, budget_s=max(2.0, 60.0 / (args.warmup + args.steps)),
                          osc=osc, build_s=build_s)
        if step >= args.warmup:
            res.append(cb)
    value = statistics.median(r["value"] for r in res)
    cbl = dict(res[-1])
    cbl["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args, w, len(I), world),
            "cpu_baseline": cbl, "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gb300(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from dvsrender4deepspace_gb300 import DeviceScene, EventSensor, interval_array, trajectory
    from dvsrender4deepspace_gb300.build import build
    if rank == 0:
        build()
    if world > 1:
        torch.distributed.barrier()
    w, V, N, I, traj = make_workload(args.workload, rank)
    t_setup = time.time()
    scene = DeviceScene(V, N, I, w["camera"], w["ss"], HAPKE, leaf_size=args.leaf,
                        geometry=GEOMETRY[args.geometry], builder=BUILDERS[args.builder])
    info = scene.info()
    sensor = EventSensor(scene, PHYSIC, timing=True, cells_per_chunk=args.chunk, cells_per_warp=args.cw,
                         circuit_precision=args.circuit)
    sensor.initialize(traj.state(0.0), 0.0)
    setup_s = time.time() - t_setup
    dt, B = w["time_resolution"], w["batch"]
    t_cursor = [0.0]

    def next_batch():
        ivs = trajectory.horizons(traj, t_cursor[0], dt, B)
        t_cursor[0] = ivs[-1][3]
        return interval_array(ivs)

    tuning = None
    if args.rays:
        sensor.set_tuning(args.cw, args.rays)
    for k in range(args.warmup):
        b = next_batch()
        if k == 0 and args.autotune:
            tuning = sensor.autotune(b)
        sensor.process_many(b)
    # ---- device-resident timed region (value)
    batches = [next_batch() for _ in range(args.steps)]
    stream = torch.cuda.ExternalStream(sensor.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sensor.reset_stats()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for b in batches:
            sensor.enqueue(b)
        stop.record(stream)
        torch.cuda.synchronize()
    dev_ms = start.elapsed_time(stop)
    sensor.collect()  # the last batch's events; also gathers the per-kernel CUDA-event timings
    st = sensor.stats()
    rays = st["primary_rays"] + st["shadow_rays"]
    # ---- end to end through the C-ABI with host buffers (e2e)
    e2e_batches = [next_batch() for _ in range(args.steps)]
    events_total, d2h = 0, 0
    torch.cuda.synchronize()
    sensor.reset_stats()
    t0 = time.perf_counter()
    for b in e2e_batches:
        ev = sensor.process_many(b)
        events_total += len(ev)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    st2 = sensor.stats()
    rays2 = st2["primary_rays"] + st2["shadow_rays"]
    gen2 = st2["events_generated"]
    # ---- adaptive optical solver over a longer window (the app's solver for
    # long sequences, apps/main_dvs.cpp:54,106-113): simulated seconds per wall
    # second and events per wall second, 200 horizons per call
    adaptive = None
    if args.adaptive_ms > 0:
        ab = 200
        n_calls = int(math.ceil(args.adaptive_ms * 1e-3 / (float(np.float32(dt)) * ab) - 1e-9))
        asensor, acircuit = sensor, args.circuit
        if args.circuit == "fp32-philox":
            # the adaptive solver keeps the reference's XORWOW stream: a sensor with FP32
            # arithmetic and that stream, started where the native run stopped
            acircuit = "fp32"
            asensor = EventSensor(scene, PHYSIC, timing=True, cells_per_chunk=args.chunk, cells_per_warp=args.cw,
                                  circuit_precision=acircuit)
            asensor.initialize(traj.state(t_cursor[0]), t_cursor[0])
        sim0, ev_a, rejected = t_cursor[0], 0, 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(n_calls):
            ivs = trajectory.horizons(traj, t_cursor[0], dt, ab)
            arr = interval_array(ivs)
            r = asensor.process_adaptive(arr, 1e-2, check_convergence=(k == 0))
            if r is None:  # rejected window: the native solver takes it
                rejected += 1
                r = asensor.process_many(arr)
            t_cursor[0] = ivs[-1][3]
            ev_a += len(r)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        adaptive = {"simulated_s": t_cursor[0] - sim0, "wall_s": wall,
                    "simulated_s_per_wall_s": (t_cursor[0] - sim0) / wall, "events": ev_a,
                    "events_per_s": ev_a / wall, "calls": n_calls, "horizons_per_call": ab,
                    "rejected_windows": rejected, "refinement": asensor.refinement_statistics(),
                    "knot_capacity": asensor.adaptive_cache_capacity(), "circuit_precision": acircuit}
    # max over ranks
    vals = torch.tensor([dev_ms, e2e_s, rays, rays2, st2["events_delivered"]], dtype=torch.float64, device="cuda")
    if world > 1:
        import torch.distributed as dist
        mx = vals.clone()
        dist.all_reduce(mx[:2], op=dist.ReduceOp.MAX)
        sm = vals.clone()
        dist.all_reduce(sm[2:], op=dist.ReduceOp.SUM)
        vals = torch.cat([mx[:2], sm[2:]])
    dev_ms, e2e_s, rays_all, rays2_all, delivered_all = vals.tolist()
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0
    value = rays_all / (dev_ms / 1e3) / 1e6
    e2e_value = rays2_all / e2e_s / 1e6
    n_pix = w["camera"]["width"] * w["camera"]["height"]
    optics_ms = st["optics_ms"] / max(1, st["optics_launches"])
    # dominant kernel: trace_cells (optics).  Algorithmic bytes per launch: the
    # per-pixel-cell radiance it must write (4 B float for the FP32 circuits,
    # 8 B double for the FP64 one) -- the HBM-minimal traffic of an
    # issue-bound traversal (the scene is read from L1/L2).
    cells_per_launch = st["circuit_cells"] / max(1, st["circuit_launches"]) / max(1, n_pix)
    chunk_bytes = 8.0 if args.circuit == "fp64" else 4.0
    alg_bytes = n_pix * cells_per_launch * chunk_bytes
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (optics_ms / 1e3) / 1e9 if optics_ms > 0 else None
    circuit_ms = st["circuit_ms"] / max(1, st["circuit_launches"])
    # circuit bytes per launch, as each mode moves them: the radiance chunk, the
    # state round trip (five FP64 fields and the reset flag; the XORWOW states
    # only when a stream is drawn: Philox keeps none), the per-pixel event count
    xorwow = args.circuit != "fp32-philox" and (PHYSIC["photon_shot_noise"] or PHYSIC["reset_thermal_noise"])
    state_bytes = 5 * 8 + 1 + (48 if xorwow else 0)
    circuit_bytes = n_pix * cells_per_launch * chunk_bytes + n_pix * state_bytes * 2 + n_pix * 4 * 2
    # the trace kernel is issue-bound: its roofline is the SMs' instruction issue
    # rate (4 warp instructions per clock per SM), from the warp instructions
    # per ray that ncu counted for this kernel and format, at the sampled clock
    rays_per_launch = rays / max(1, st["optics_launches"])
    issue = None
    shape = ((tuning["cells_per_warp"], tuning["rays_per_lane"]) if tuning else (args.cw or 32, args.rays or 2))
    counted = (args.workload, args.geometry, args.builder) + shape
    ipr = TRACE_WARP_INSTRUCTIONS_PER_RAY.get(counted)
    sm_mhz = clocks.summary()["sm_mhz"]
    if ipr and optics_ms > 0 and sm_mhz:
        issue_peak = GB300_SMS * 4 * sm_mhz * 1e6
        issue_achieved = ipr * rays_per_launch / (optics_ms / 1e3)
        issue = {"bound": "issue", "kernel": "trace_cells_kernel", "achieved": issue_achieved / 1e12,
                 "peak": issue_peak / 1e12, "unit": "T warp-instructions/s", "frac": issue_achieved / issue_peak,
                 "warp_instructions_per_ray": ipr, "sm_mhz": sm_mhz,
                 "note": "issue rate of %d SMs x 4 schedulers at the sampled clock; instructions per ray from "
                         "ncu smsp__inst_executed.sum of this kernel and format" % GB300_SMS}
    cb = None
    o64 = None
    if not args.no_cpu_baseline:
        cb = cpu_baseline(args.workload, V, N, I, traj, w, budget_s=15.0)
        # beside it, the FP64 oracle of the same optics (the precision report's oracle)
        from oracle import oracle as O
        t_build = time.time()
        o64 = O.OracleScene(V, N, I, w["camera"], w["ss"], HAPKE, max_leaf=64, fp64=True,
                            watertight=bool(GEOMETRY[args.geometry] & 2))
        b64 = time.time() - t_build
        cb64 = cpu_baseline(args.workload, V, N, I, traj, w, budget_s=8.0, osc=o64, build_s=b64, fp64=True)
        cb["fp64_oracle"] = {"value": cb64["value"], "unit": cb64["unit"], "cores": cb64["cores"],
                             "sample": cb64["sample"]}
    errors = None
    if args.workload in ("precision", "large") and not args.no_precision_report and rank == 0:
        errors = precision_errors(V, N, I, traj, w, scene, args.geometry, args.circuit, o64=o64)
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": bench_config(args, w, len(I), world),
        "scene": {"device_gb": info["device_bytes"] / 1e9,
                  "bvh": "8-wide, %s, leaf %d, depth %d" % (BUILDERS_TEXT[info["builder"]], info["leaf_size"],
                                                            info["depth"]),
                  "sah_node_visits": info["sah_node_visits"], "sah_triangle_tests": info["sah_triangle_tests"]},
        "rays_per_step": rays / args.steps,
        "rays": {"primary_per_step": st["primary_rays"] / args.steps, "shadow_per_step": st["shadow_rays"] / args.steps,
                 "primary_mrays_s": st["primary_rays"] / (dev_ms / 1e3) / 1e6 if world == 1 else None,
                 "shadow_mrays_s": st["shadow_rays"] / (dev_ms / 1e3) / 1e6 if world == 1 else None},
        "events_per_s": delivered_all / e2e_s,
        "events_generated_per_step": gen2 / args.steps,
        "e2e": {"value": e2e_value, "unit": "Mrays/s",
                "h2d_bytes_per_step": B * 176, "d2h_bytes_per_step": int(events_total * 24 / args.steps)},
        "gpu_launches": int(st["launches"]),
        "kernel_ms": {"optics_per_launch": optics_ms, "circuit_per_launch": circuit_ms,
                      "events_total": st["events_ms"]},
        "roofline": {"bound": "hbm", "kernel": "trace_cells_kernel", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": (TRACE_DRAM_BYTES_PER_PIXEL_CELL[counted] * n_pix * cells_per_launch
                                 if counted in TRACE_DRAM_BYTES_PER_PIXEL_CELL else None),
                     "algorithmic_bytes": alg_bytes,
                     "peak_source": "measured" if peaks else "fallback",
                     "note": "traversal is instruction-issue bound (roofline_issue); bytes = radiance written "
                             "per launch"},
        "roofline_issue": issue,
        "roofline_circuit": {"bound": "hbm", "kernel": "circuit_kernel",
                             "achieved": circuit_bytes / (circuit_ms / 1e3) / 1e9 if circuit_ms > 0 else None,
                             "peak": peak, "unit": "GB/s", "algorithmic_bytes": circuit_bytes},
        "roofline_readout": readout_roofline(peak) if not args.no_readout_leg else None,
        "clocks": clocks.summary(), "setup_s": setup_s, "bvh_build_s": info["build_seconds"], "tuning": tuning,
        "adaptive": adaptive,
        "cpu_baseline": cb,
        "precision_errors": errors,
    }
    if line["roofline_circuit"]["achieved"]:
        line["roofline_circuit"]["frac"] = line["roofline_circuit"]["achieved"] / peak
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


SERVING_GRIDS = (512, 768, 1024, 1536, 2048, 2560, 3072, 4096)


def run_serving(args):
    """Serving workload: a seeded Poisson stream (200 req/s) of render+DVS
    jobs -- resolutions uniform over 64x48 / 346x260 / 640x480 / 1280x720,
    durations log-uniform, terrains uniform over a pool of 8 heightfields of
    512^2 ... 4096^2 vertices -- admitted under a 150 GB HBM budget by the
    continuous-batching server, against the plain path (the same jobs one at
    a time, first come first served).  Durations are the stream's 0.05-2 s
    scaled by --serving-scale (default 0.01: 0.5-20 ms of simulated time per
    job, 1 us circuit cells) so that the stream completes in about a minute."""
    import torch
    from dvsrender4deepspace_gb300 import DeviceScene, serve, terrain
    from dvsrender4deepspace_gb300.build import build
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    build()
    t_setup = time.time()
    scenes = []
    for k, g in enumerate(SERVING_GRIDS):
        V, N, I = terrain.terrain_mesh(g, 20260100 + k)
        scenes.append(DeviceScene(V, N, I, dict(width=8, height=8, fx=8.0, fy=8.0, cx=4.0, cy=4.0), 1, HAPKE))
    setup_s = time.time() - t_setup
    phys = dict(PHYSIC)

    def stream():
        return serve.synthetic_stream(args.serving_jobs, 20260104, len(scenes), rate_hz=200.0,
                                      duration_scale=args.serving_scale, physic=phys, intensity=1000.0)

    # warm-up: one small job per terrain through the server (first-use allocations, module load)
    warm = [j for j in stream() if j.camera["width"] == 64][:2]
    circuit = args.circuit
    serve.Server(scenes, 150 << 30, circuit=circuit).run(warm, realtime=False)
    results = {}
    for mode, max_active, policy in (("served", 64, "srpt"), ("served_fair", 64, "fair"), ("plain", 1, "fair")):
        jobs = stream()
        srv = serve.Server(scenes, 150 << 30, horizons_per_step=64, max_active=max_active, policy=policy,
                           circuit=circuit)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with ClockSampler(local) as clocks:
            done = srv.run(jobs, realtime=True)
            torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        events = sum(len(j.events) for j in done)
        rays = sum(j.rays for j in done)
        res = serve.latency_summary(done)
        res.update({"jobs": len(done), "makespan_s": wall, "events": events, "events_per_s": events / wall,
                    "mrays_per_s": rays / wall / 1e6, "peak_active": srv.peak_active,
                    "peak_device_gb": srv.peak_used / 1e9, "scheduler_steps": srv.steps,
                    "clocks": clocks.summary()})
        results[mode] = res
    line = {"metric": METRIC, "value": results["served"]["p99_ms"], "unit": "ms (p99 request latency)",
            "n_gpus": 1, "steps": args.serving_jobs, "warmup": len(warm), "ms_per_step": None,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "serving", "jobs": args.serving_jobs, "rate_hz": 200.0,
                       "resolutions": ["64x48", "346x260", "640x480", "1280x720"],
                       "durations_s": [0.05 * args.serving_scale, 2.0 * args.serving_scale],
                       "terrain_grids": list(SERVING_GRIDS), "hbm_budget_gb": 150, "supersample": 1,
                       "time_resolution": 1e-5, "circuit_step": PHYSIC["circuit_step"],
                       "circuit_precision": circuit},
            "served": results["served"], "served_fair": results["served_fair"], "plain": results["plain"],
            "p99_speedup_vs_plain": results["plain"]["p99_ms"] / results["served"]["p99_ms"],
            "throughput_vs_plain": results["served"]["events_per_s"] / max(1e-9, results["plain"]["events_per_s"]),
            "setup_s": setup_s}
    print(json.dumps(line))
    return 0


READOUT_KERNELS_PER_SUBMIT = 2 + 12 * 3 + 3 + 3  # keys, packing, 12 x (histogram, scan, scatter), FIFO, release


def readout_events(rng, n, t):
    """One batch of the readout workload: n events of a 1280x720 sensor within
    64 us from t, uniform over pixels, polarities and times."""
    from dvsrender4deepspace_gb300._capi import EVENT_DTYPE
    ev = np.zeros(n, EVENT_DTYPE)
    ev["timestamp"] = t + rng.uniform(0.0, 64e-6, n)
    ev["x"] = rng.integers(0, 1280, n)
    ev["y"] = rng.integers(0, 720, n)
    ev["polarity"] = rng.integers(0, 2, n)
    return ev


def run_readout(args, n_events=1 << 22):
    """Readout workload: the device FIFO (dvs_device_readout_*) alone on batches
    of 4,194,304 events of a 1280x720 sensor within 64 us each, through an
    unbounded bus (1e12 s^-1, no latency) so that every batch takes the
    parallel path (radix sort by (t, y, x), max-plus scan, occupancy, release);
    the configs' 5e6 s^-1 bus would saturate at that density and take the
    serial drop path.  `value` is events per second of device time (CUDA
    events around the submit's kernels); `e2e` the same through the host call
    with the events in host memory (upload, kernels, download of the delivered
    events).  The reference arm times the oracle's serial FIFO (stable sort
    and queue, the reference's event_readout.cpp) on one batch."""
    import torch
    from dvsrender4deepspace_gb300.build import build
    from dvsrender4deepspace_gb300.raycast import EventReadout
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    if args.steps < 1:
        raise SystemExit("--steps must be at least 1")
    torch.cuda.set_device(local)
    build()
    rng = np.random.default_rng(5)
    batches = [readout_events(rng, n_events, 1.0 + 64e-6 * b) for b in range(args.warmup + args.steps)]
    r = EventReadout(1e12, 0.0, 1 << 24, device=True, max_batch=n_events)

    def submit(b):
        t0 = time.perf_counter()
        out = r.submit(batches[b], 1.0 + 64e-6 * (b + 1))
        dt = time.perf_counter() - t0
        if len(out) != n_events:
            raise RuntimeError("device readout delivered %d of %d events" % (len(out), n_events))
        return dt

    for b in range(args.warmup):  # the first batch also sizes the sort grid
        submit(b)
    dev_ms, wall = [], 0.0
    with ClockSampler(local) as clocks:  # started before and stopped after the timed batches
        torch.cuda.synchronize()
        for b in range(args.warmup, len(batches)):
            wall += submit(b)
            dev_ms.append(r.last_ms())
    ms = sum(dev_ms) / max(1, len(dev_ms))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    alg = n_events * 2 * 24.0
    cb = None
    if not args.no_cpu_baseline:
        cb = readout_cpu_baseline(batches[:1])
    n = args.steps
    line = {"metric": METRIC, "value": n_events / (ms / 1e3), "unit": "events/s", "n_gpus": 1, "steps": n,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "readout", "events_per_batch": n_events, "width": 1280, "height": 720,
                       "batch_window_s": 64e-6, "bandwidth": 1e12, "latency": 0.0, "capacity": 1 << 24,
                       "l2": "inputs larger than L2: each batch's events are 100.7 MB on the device, "
                             "its sort buffers 3 x 67 MB"},
            # per batch: the events as 24-byte device records plus the count and time in; the
            # released events as 24-byte device records plus four status words (24 B) out
            "e2e": {"value": n_events * n / wall, "unit": "events/s", "h2d_bytes_per_step": n_events * 24 + 16,
                    "d2h_bytes_per_step": n_events * 24 + 24},
            "roofline": {"bound": "hbm", "kernel": "device readout (radix sort, max-plus scan, release)",
                         "achieved": alg / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (ms / 1e3) / 1e9 / peak, "traffic": READOUT_DRAM_BYTES_PER_EVENT * n_events,
                         "traffic_gbs": READOUT_DRAM_BYTES_PER_EVENT * n_events / (ms / 1e3) / 1e9,
                         "algorithmic_bytes": alg,
                         "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
            "gpu_launches": READOUT_KERNELS_PER_SUBMIT * n, "clocks": clocks.summary(), "cpu_baseline": cb}
    print(json.dumps(line))
    return 0


def run_readout_reference(args, n_events=1 << 22):
    """The readout workload's reference arm: the oracle's serial FIFO (the
    reference's event_readout.cpp restated) on the host, one batch per step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    rng = np.random.default_rng(5)
    res = []
    for b in range(args.warmup + args.steps):
        cb = readout_cpu_baseline([readout_events(rng, n_events, 1.0 + 64e-6 * b)], first=b)
        if b >= args.warmup:
            res.append(cb)
    value = statistics.median(r["value"] for r in res)
    cbl = dict(res[-1], value=value)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": n_events / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "readout", "events_per_batch": n_events, "width": 1280, "height": 720,
                       "batch_window_s": 64e-6, "bandwidth": 1e12, "latency": 0.0, "capacity": 1 << 24},
            "cpu_baseline": cbl,
            "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def readout_cpu_baseline(batches, first=0):
    """The oracle's serial FIFO (the reference's event_readout.cpp: stable sort
    by (t, y, x), then the queue) on the host, one thread."""
    import ctypes as C
    from oracle import oracle as O
    lib = O.load(False)
    s, n = 0.0, 0
    for b, ev in enumerate(batches):
        oev = np.zeros(len(ev), O.EVENT_DTYPE)
        for f in O.EVENT_DTYPE.names:
            oev[f] = ev[f]
        out = np.zeros(len(ev), O.EVENT_DTYPE)
        got = C.c_size_t()
        r = lib.oracle_readout_create(1e12, 0.0, 1 << 24)
        t0 = time.perf_counter()
        lib.oracle_readout_submit(r, oev.ctypes.data, len(oev), 1.0 + 64e-6 * (first + b + 1), out.ctypes.data,
                                  len(out), C.byref(got))
        s += time.perf_counter() - t0
        lib.oracle_readout_destroy(r)
        n += len(ev)
        if got.value != len(ev):
            raise RuntimeError("oracle readout delivered %d of %d events" % (got.value, len(ev)))
    return {"value": n / s, "unit": "events/s", "cores": 1, "kind": "port",
            "sample": "%d events (one batch), %.1f s of CPU work" % (n, s)}


def batching_members(n, seed, light, intensity):
    """The batching config's trajectories: constant-altitude arcs with altitude
    U(0.5, 5) km, speed U(10, 200) m/s, heading U(0, 360) deg, yaw rate
    U(-5, 5) deg/s, starting points spread over the 10 km terrain, and lengths
    U{20..400} frames (seeded)."""
    from dvsrender4deepspace_gb300 import trajectory
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        out.append((trajectory.Orbit((rng.uniform(-3000, 3000), rng.uniform(-3000, 3000)), rng.uniform(500, 5000),
                                     rng.uniform(10, 200), math.radians(rng.uniform(0, 360)),
                                     math.radians(rng.uniform(-5, 5)), light, intensity),
                    int(rng.integers(20, 401))))
    return out


def run_batching(args):
    """Batching config: 64 independent trajectories over one 1024^2 terrain
    (346x260, 16 sub-rays, 10 us horizons, FP32 pixel state, FP64 timestamps),
    every step one multi-sensor batch step (one persistent trace launch, one
    circuit launch, captured into a CUDA graph and replayed).  Trajectory k of
    F_k frames stays active for ceil(F_k / 400 * K) of the K timed steps, so
    members drop out unevenly and the step is re-captured for each new shape.
    Beside it, the same members advanced one sensor at a time (the plain path)."""
    import torch
    from dvsrender4deepspace_gb300 import DeviceScene, EventSensor, SensorBatch, interval_array, terrain, trajectory
    from dvsrender4deepspace_gb300.build import build
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if rank == 0:
        build()
    if world > 1:
        torch.distributed.init_process_group("nccl")
        torch.distributed.barrier()
    w = WORKLOADS["orbit"]
    V, N, I = terrain.terrain_mesh(w["grid"], w["seed"])
    light = trajectory.sun_direction(w["sun_elevation"], 35.0)
    members = batching_members(args.batch_members, 20260005 + rank, light, w["intensity"])
    t_setup = time.time()
    base = DeviceScene(V, N, I, w["camera"], w["ss"], HAPKE, leaf_size=args.leaf, geometry=GEOMETRY[args.geometry],
                       builder=BUILDERS[args.builder])
    info = base.info()
    setup_s = time.time() - t_setup
    dt, H = w["time_resolution"], args.batch_horizons
    K, Wm = args.steps, args.warmup
    active_steps = [int(math.ceil(frames / 400.0 * K)) for _, frames in members]

    def make(view, count):
        sensors = []
        for traj, _ in members[:count]:
            s = EventSensor(view, PHYSIC, cells_per_warp=args.cw, circuit_precision=args.circuit)
            s.initialize(traj.state(0.0), 0.0)
            sensors.append(s)
        return sensors

    def plan(step, cursors, timed, horizons, count):
        rows = []
        for m, (traj, _) in enumerate(members[:count]):
            if timed and step >= active_steps[m]:
                rows.append([])
                continue
            ivs = trajectory.horizons(traj, cursors[m], dt, horizons)
            cursors[m] = ivs[-1][3]
            rows.append(interval_array(ivs))
        return rows

    def rays_of(sensors):
        return sum(s.stats()["primary_rays"] + s.stats()["shadow_rays"] for s in sensors)

    def events_of(sensors):
        return sum(s.stats()["events_delivered"] for s in sensors)

    def measure(view, horizons, count=None):
        count = count or len(members)
        results = {}
        for mode in ("batch", "loop"):
            sensors = make(view, count)
            batch = SensorBatch(sensors) if mode == "batch" else None
            cursors = [0.0] * count
            for k in range(Wm):
                rows = plan(k, cursors, False, horizons, count)
                if batch:
                    batch.process(rows)
                else:
                    for s, r in zip(sensors, rows):
                        s.process_many(r)
            rays0, ev0 = rays_of(sensors), events_of(sensors)
            st0 = batch.stats() if batch else None
            # the timed steps' intervals, generated beforehand (host Python, not the path)
            timed_rows = [plan(k, cursors, True, horizons, count) for k in range(K)]
            if world > 1:
                torch.distributed.barrier()
            with ClockSampler(local) as clocks:  # started before and stopped after the timed region
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for k in range(K):
                    rows = timed_rows[k]
                    if batch:
                        batch.process(rows)
                    else:
                        for s, r in zip(sensors, rows):
                            if len(r):
                                s.process_many(r)
                torch.cuda.synchronize()
                wall = time.perf_counter() - t0
            if world > 1:
                torch.distributed.barrier()
            rays, events = rays_of(sensors) - rays0, events_of(sensors) - ev0
            res = {"wall_s": wall, "rays": rays, "events": events, "mrays_per_s_wall": rays / wall / 1e6,
                   "events_per_s": events / wall, "clocks": clocks.summary()}
            if batch:
                st = batch.stats()
                dev_ms = st["step_ms"] - st0["step_ms"]
                res.update({"device_ms": dev_ms, "mrays_per_s_device": rays / (dev_ms / 1e3) / 1e6,
                            "graph_launches": st["graph_launches"] - st0["graph_launches"],
                            "graph_captures": st["graph_captures"] - st0["graph_captures"],
                            "persistent_launches": st["persistent_launches"] - st0["persistent_launches"],
                            "host_ms": st["host_ms"] - st0["host_ms"],
                            "capture_ms": st["capture_ms"] - st0["capture_ms"],
                            "trace_items": st["trace_items"] - st0["trace_items"]})
                batch.close()
            results[mode] = res
            for s in sensors:
                s.close()
        return results

    results = measure(base, H)
    # the same trajectories as small members (64x48, one sub-ray, 64 horizons a step):
    # per-member work is then a few launches' worth, where one persistent launch and
    # one graph per step replace per-member launches and synchronisations
    small_cam = dict(width=64, height=48, fx=60.0, fy=60.0, cx=32.0, cy=24.0)
    small = measure(base.view(small_cam, 1), 64) if args.batch_small else None
    # members at the 1280x720 config's camera and 16^2 sub-rays (4 trajectories, 4 horizons a step):
    # each member's step already fills the GPU, so this is where batching has nothing to add
    prec_cam = WORKLOADS["precision"]["camera"]
    prec = (measure(base.view(prec_cam, WORKLOADS["precision"]["ss"]), 4, count=args.batch_precision_members)
            if args.batch_precision_members > 0 else None)
    b, l = results["batch"], results["loop"]
    vals = torch.tensor([b["device_ms"], b["wall_s"], b["rays"], l["wall_s"], l["rays"], b["events"]],
                        dtype=torch.float64, device="cuda")
    if world > 1:
        mx = vals.clone()
        torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
        sm = vals.clone()
        torch.distributed.all_reduce(sm, op=torch.distributed.ReduceOp.SUM)
        dev_ms, b_wall, l_wall = mx[0].item(), mx[1].item(), mx[3].item()
        b_rays, l_rays, b_events = sm[2].item(), sm[4].item(), sm[5].item()
    else:
        dev_ms, b_wall, l_wall = b["device_ms"], b["wall_s"], l["wall_s"]
        b_rays, l_rays, b_events = b["rays"], l["rays"], b["events"]
    if rank != 0:
        return 0
    from dvsrender4deepspace_gb300 import INTERVAL_DTYPE
    n_launch = sum(min(K, a) for a in active_steps)
    cells_per_horizon = int(round(float(np.float32(dt)) / float(np.float32(PHYSIC["circuit_step"]))))
    cb = None
    if not args.no_cpu_baseline:
        cb = cpu_baseline("orbit", V, N, I, members[0][0], w, budget_s=15.0)
    line = {"metric": METRIC, "value": b_rays / (dev_ms / 1e3) / 1e6, "unit": "Mrays/s", "n_gpus": world,
            "steps": K, "warmup": Wm, "ms_per_step": dev_ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "batching", "members": len(members), "frames": [f for _, f in members],
                       "active_steps": active_steps, "width": w["camera"]["width"], "height": w["camera"]["height"],
                       "supersample": w["ss"], "terrain_grid": w["grid"], "triangles": int(info["triangles"]),
                       "horizons_per_step": H, "time_resolution": dt, "circuit_precision": args.circuit,
                       "geometry": args.geometry, "parallelism": "dp%d (independent batches)" % world,
                       "l2": "inputs larger than L2 (radiance chunks %.1f GB)"
                             % (len(members) * H * 10 * w["camera"]["width"] * w["camera"]["height"]
                                * (4 if args.circuit.startswith("fp32") else 8) / 1e9)},
            # per active member-step: its intervals and their circuit cells (24 B each) in, its
            # events (24 B each on the device side) and status words out
            "e2e": {"value": b_rays / b_wall / 1e6, "unit": "Mrays/s",
                    "h2d_bytes_per_step": int(n_launch * H * (INTERVAL_DTYPE.itemsize + cells_per_horizon * 24) / K),
                    "d2h_bytes_per_step": int((b_events * 24 + n_launch * 8) / K)},
            "events_per_s": b_events / b_wall,
            "batch": results["batch"], "per_sensor_loop": results["loop"],
            "small_members": None if small is None else {
                "camera": "64x48", "supersample": 1, "horizons_per_step": 64, "batch": small["batch"],
                "per_sensor_loop": small["loop"],
                "batch_vs_loop_wall": small["batch"]["mrays_per_s_wall"] / max(1e-9, small["loop"]["mrays_per_s_wall"]),
                "events_batch_vs_loop": small["batch"]["events_per_s"] / max(1e-9, small["loop"]["events_per_s"])},
            "precision_members": None if prec is None else {
                "camera": "1280x720", "supersample": WORKLOADS["precision"]["ss"], "members": args.batch_precision_members,
                "horizons_per_step": 4, "batch": prec["batch"], "per_sensor_loop": prec["loop"],
                "batch_vs_loop_wall": prec["batch"]["mrays_per_s_wall"] / max(1e-9, prec["loop"]["mrays_per_s_wall"]),
                "events_batch_vs_loop": prec["batch"]["events_per_s"] / max(1e-9, prec["loop"]["events_per_s"]),
                "target_events_vs_plain": 5.0},
            "batch_vs_loop_wall": (b_rays / b_wall) / max(1e-9, l_rays / l_wall),
            "gpu_launches": int(2 * K + 3 * n_launch),
            "clocks": results["batch"]["clocks"], "setup_s": setup_s, "cpu_baseline": cb}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="precision",
                    choices=sorted(WORKLOADS) + ["serving", "batching", "readout"])
    ap.add_argument("--batch-members", type=int, default=64)
    ap.add_argument("--batch-horizons", type=int, default=16, help="horizons per member per batching step")
    ap.add_argument("--batch-precision-members", type=int, default=4,
                    help="members at the 1280x720 config's camera and sub-rays (0: skip that leg)")
    ap.add_argument("--no-batch-small", dest="batch_small", action="store_false",
                    help="skip the batching workload's small-member leg (64x48, one sub-ray)")
    ap.add_argument("--serving-jobs", type=int, default=48)
    ap.add_argument("--serving-scale", type=float, default=0.01)
    ap.add_argument("--leaf", type=int, default=0)
    ap.add_argument("--builder", default="sah", choices=sorted(BUILDERS),
                    help="split rule of the BVH: binned SAH splits (default) or Morton radix splits")
    ap.add_argument("--geometry", default=None, choices=sorted(GEOMETRY),
                    help="BVH format: FP32 or FP16 (half) child bounds; Moller-Trumbore or watertight triangles")
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--cw", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-readout-leg", action="store_true", help="skip the device readout's large-batch leg")
    ap.add_argument("--no-precision-report", action="store_true",
                    help="skip the precision workload's error report against the FP64 oracle")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the autotuner (packet shape, then circuit-step chunk) on the first warm-up batch")
    ap.add_argument("--rays", type=int, default=0, help="sub-rays per lane: 1, 2 or 4 (0 = default)")
    ap.add_argument("--adaptive-ms", type=float, default=2.0,
                    help="also run the adaptive optical solver over this many simulated milliseconds")
    ap.add_argument("--circuit", default=None, choices=["fp64", "fp32", "fp32-philox"],
                    help="pixel-circuit arithmetic: fp64 (reference) or fp32 (precision mode)")
    args = ap.parse_args()
    w = WORKLOADS.get("orbit" if args.workload == "batching" else args.workload, {})
    if args.geometry is None:
        args.geometry = w.get("geometry", "reference")   # each workload's configured BVH format
    if args.circuit is None:  # serving: the FP32 circuit with the counter-based noise stream
        args.circuit = "fp32-philox" if args.workload == "serving" else w.get("circuit", "fp64")
    if args.impl == "reference":
        if args.workload in ("serving", "batching"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving or multi-sensor "
                                                                  "batching layer"}))
            return 0
        if args.workload == "readout":
            return run_readout_reference(args)
        return run_reference(args)
    if args.workload == "readout":
        return run_readout(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "batching":
        return run_batching(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
