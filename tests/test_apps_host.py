"""Host side of the drop-in apps (no GPU): the YAML config, scene bundles,
the continuous trajectory (known answers of tests/test_render.cu:115-131),
the event writers (tests/test_writer.cpp:11-18) and the image writers, and
the command-line error paths of bin/dvs and bin/cam.  Files written by the
C++ code are read back here with independent readers (HDF5 by its file
format specification, PNG through zlib, TIFF by its tags)."""
import math
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import build as B
from dvsrender4deepspace_gb300 import inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DAVIS_CAMERA = dict(width=346, height=260, fx=226.3802, fy=226.15, cx=173.6471, cy=133.7327)
PHYSIC = dict(threshold_pos=0.28, threshold_neg=0.28, threshold_std=0.03, threshold_min=0.01, refractory_time=200e-6,
              wavelength_nm=550, quantum_efficiency=0.3, pixel_pitch_um=15, fill_factor=0.2, f_number=2.0,
              lens_transmission=0.8, radiance_scale=0.001, temperature_k=300, subthreshold_kappa=0.8,
              receptor_capacitance_f=1e-15, reset_capacitance_f=20e-15, dark_current_a=1e-18, reset_leakage_a=0,
              photon_shot_noise=1, reset_thermal_noise=0, circuit_step=1e-6, readout_bandwidth=5e6,
              readout_latency=18e-9, readout_queue_capacity=1000000, max_events_per_step=16, random_seed=114514)
SCENE = dict(frame_count=201, fps=24.0, imu_fps=200, cam_fps=30, time_resolution=1e-5, supersample_factor=16,
             blur_resolution=1e-3)
HAPKE = dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=0.453786, w=0.324, B_S0=2.42, B_C0=0.0, phi=0.3)


@pytest.fixture(scope="module")
def built():
    B.build()
    return B


def f32(x):
    return float(np.float32(x))


# ---- config -----------------------------------------------------------------------
def test_config_round_trip(tmp_path):
    p = tmp_path / "davis.yaml"
    inputs.write_config(p, DAVIS_CAMERA, PHYSIC, SCENE, HAPKE)
    c = inputs.load_config(p)
    assert c["camera"]["width"] == 346 and c["camera"]["fy"] == f32(226.15)
    for k, v in PHYSIC.items():
        assert c["physic"][k] == (v if isinstance(v, int) else f32(v)), k
    for k, v in HAPKE.items():
        assert c["hapke"][k] == f32(v), k
    assert c["scene"]["frame_count"] == 201 and c["scene"]["time_resolution"] == f32(1e-5)
    assert c["scene"]["translation"] == [0, 0, 0] and c["scene"]["rotation"] == [0, 0, 0]


def test_config_grammar_and_defaults(tmp_path):
    text = """# comment line
intrinsic:   # trailing comment
  width: 64\r
  height: 48
  fx: 50
  fy: 50
  cx: 32
  cy: 24
physic:
  threshold_pos: 0.2
  threshold_neg: 0.3
  refractory_time: 0
  readout_bandwidth: 0
  readout_latency: 0
scene:
  frame_count: 2
  fps: 10
  imu_fps: 100
  cam_fps: 10
  time_resolution: 1e-4
  supersample_factor: 1
  blur_resolution: 1e-3
  translation: [1, 2.5, -3]
  rotation: [0.1, 0, 0]
hapke:
  b: 0.3
  c: 0.4
  hS: 0.06
  hC: 1.0
  thetap: 0.349066
  w: 0.25
  B_S0: 1.0
  B_C0: 0
  phi: 0.3
"""
    p = tmp_path / "c.yaml"
    p.write_text(text)
    c = inputs.load_config(p)
    assert c["physic"]["threshold_neg"] == f32(0.3) and c["physic"]["quantum_efficiency"] == f32(0.3)  # default
    assert c["physic"]["random_seed"] == 114514 and c["physic"]["max_events_per_step"] == 16
    assert c["scene"]["translation"] == [1.0, 2.5, -3.0] and c["scene"]["rotation"][0] == f32(0.1)


@pytest.mark.parametrize("edit, message", [
    (lambda t: t.replace("scene:", "scenery:"), "Missing top-level section 'scene'"),
    (lambda t: t.replace("  fx: 50\n", ""), "Missing key 'fx' in section 'intrinsic'"),
    (lambda t: t.replace("width: 64", "width: 6.4"), "Invalid value for key 'width' in section 'intrinsic': '6.4'"),
    (lambda t: t.replace("  readout_latency: 0\n", "  readout_latency: 0\n  leak_rate_hz: 1\n"),
     "removed physic key 'leak_rate_hz'"),
    (lambda t: t.replace("threshold_pos: 0.2", "threshold_pos: 0"), "invalid optical/circuit model parameter range"),
    (lambda t: t.replace("threshold_pos: 0.2", "threshold_pos: -1"), "physic values must be finite and nonnegative"),
    (lambda t: t.replace("frame_count: 2", "frame_count: 1"), "invalid scene or camera range"),
    (lambda t: t.replace("translation: [1, 2.5, -3]", "translation: [1, 2]"), "scene.translation must have three"),
    (lambda t: t.replace("b: 0.3", "b: 1.0"), "invalid Hapke parameter range"),
    (lambda t: t.replace("phi: 0.3", "phi: 0.9"), "invalid Hapke parameter range"),
    (lambda t: t.replace("  width: 64", "width: 64"), "top-level key 'width' has a value"),
    (lambda t: t.replace("  fx: 50", "  fx 50"), "missing colon"),
    (lambda t: "  orphan: 1\n" + t, "without a parent section"),
])
def test_config_errors(tmp_path, edit, message):
    base = (tmp_path / "ok.yaml")
    inputs.write_config(base, dict(width=64, height=48, fx=50, fy=50, cx=32, cy=24),
                        dict(threshold_pos=0.2, threshold_neg=0.3, refractory_time=0, readout_bandwidth=0,
                             readout_latency=0),
                        dict(frame_count=2, fps=10, imu_fps=100, cam_fps=10, time_resolution=1e-4,
                             supersample_factor=1, blur_resolution=1e-3, translation=[1, 2.5, -3]),
                        dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0, phi=0.3))
    text = base.read_text().replace("  width: 64", "  width: 64").replace("fx: 50.0", "fx: 50")
    text = text.replace("threshold_pos: 0.2", "threshold_pos: 0.2").replace("frame_count: 2", "frame_count: 2")
    text = text.replace("translation: [1.0, 2.5, -3.0]", "translation: [1, 2.5, -3]").replace("b: 0.3\n", "b: 0.3\n")
    bad = tmp_path / "bad.yaml"
    bad.write_text(edit(text))
    with pytest.raises(ValueError) as e:
        inputs.load_config(bad)
    assert message in str(e.value)


# ---- trajectory (tests/test_render.cu:115-131) ---------------------------------------
def rot_z(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], np.float32)


def rot_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]], np.float32)


def test_trajectory_mount_light_and_seconds():
    world = rot_z(math.pi / 2)
    fr = inputs.frames_array([.125, .5], [(10, 20, 30)] * 2, [world, world], [(0, 0, 1)] * 2, [1000, 1000])
    scene = dict(fps=24.0, translation=[1, 0, 0], rotation=[math.pi / 2, 0, 0])
    traj = inputs.Trajectory(fr, scene)
    st, R = traj.evaluate(.125)
    assert np.linalg.norm(st["position"] - np.array([10, 21, 30])) < 1e-5  # local mount translation
    assert np.linalg.norm(R - world @ rot_x(math.pi / 2)) < 1e-5           # local mount rotation
    assert tuple(st["light"]) == (0.0, 0.0, 1.0)                          # world light unchanged
    assert traj.range() == (0.125, 0.5)                                   # explicit seconds
    with pytest.raises(ValueError, match="strictly increasing"):
        inputs.Trajectory(inputs.frames_array([.125, .125], [(10, 20, 30)] * 2, [world, world], [(0, 0, 1)] * 2,
                                              [1000, 1000]), scene)
    with pytest.raises(ValueError, match="non-finite"):
        inputs.Trajectory(inputs.frames_array([.125, np.inf], [(10, 20, 30)] * 2, [world, world], [(0, 0, 1)] * 2,
                                              [1000, 1000]), scene)
    with pytest.raises(ValueError, match="rigid poses"):
        inputs.Trajectory(inputs.frames_array([.1, .2], [(0, 0, 0)] * 2, [world, 2 * world], [(0, 0, 1)] * 2,
                                              [1, 1]), scene)
    with pytest.raises(ValueError, match="mount"):
        inputs.Trajectory(fr, dict(fps=0.0))


def test_trajectory_curves():
    eye = np.eye(3, dtype=np.float32)
    # constant keys stay exactly constant, with zero rates
    fr = inputs.frames_array([0, .1, .2, .3], [(5, -7, 900)] * 4, [eye] * 4, [(0.6, 0, 0.8)] * 4, [3] * 4)
    traj = inputs.Trajectory(fr, dict(fps=10.0))
    for t in (0, .03, .1, .17, .3):
        st, R = traj.evaluate(t)
        assert tuple(st["position"]) == (5.0, -7.0, 900.0) and tuple(st["velocity"]) == (0, 0, 0)
        assert st["intensity"] == 3.0 and st["intensity_rate"] == 0.0
        assert np.allclose(R, eye, atol=1e-6)
    # evenly spaced collinear keys: constant velocity, linear position
    fr = inputs.frames_array([0, .1, .2, .3], [(x, 0, 500) for x in (0, 10, 20, 30)], [eye] * 4, [(0, 0, 1)] * 4,
                             [1] * 4)
    traj = inputs.Trajectory(fr, dict(fps=10.0))
    for t in (0.01, .05, .15, .29):
        st, _ = traj.evaluate(t)
        assert abs(st["position"][0] - 100 * t) < 1e-3 and abs(st["velocity"][0] - 100) < 1e-2
    # outside the keys: clamped to the end poses
    assert traj.evaluate(-1)[0]["position"][0] == 0.0 and traj.evaluate(5)[0]["position"][0] == 30.0
    # monotone keys give a monotone curve (auto-clamped handles: no overshoot)
    fr = inputs.frames_array([0, .1, .2, .3, .4], [(x, 0, 0) for x in (0, 0, 10, 10, 11)], [eye] * 5,
                             [(0, 0, 1)] * 5, [1] * 5)
    traj = inputs.Trajectory(fr, dict(fps=10.0))
    xs = [traj.evaluate(t)[0]["position"][0] for t in np.linspace(0, .4, 161)]
    assert all(b >= a for a, b in zip(xs, xs[1:])) and max(xs) <= 11.0
    # rotation about one axis: angle follows the phase curve, rate about that axis
    keys = [rot_z(a) for a in (0.0, 0.2, 0.4)]
    fr = inputs.frames_array([0, 1, 2], [(0, 0, 0)] * 3, keys, [(0, 0, 1)] * 3, [1] * 3)
    traj = inputs.Trajectory(fr, dict(fps=1.0))
    for t in (0.0, 0.5, 1.0, 1.5, 2.0):
        st, R = traj.evaluate(t)
        assert abs(math.atan2(R[1, 0], R[0, 0]) - 0.2 * t) < 1e-5
        q = st["rotation"]
        assert abs(q[0]) < 1e-6 and abs(q[1]) < 1e-6 and abs(np.dot(q, q) - 1) < 1e-6


def test_bundle_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    V = rng.normal(size=(10, 3)).astype(np.float32)
    N = rng.normal(size=(10, 3)).astype(np.float32)
    I = rng.integers(0, 10, (7, 3)).astype(np.uint32)
    worlds = [rot_z(a) @ rot_x(0.3) for a in (0.1, 0.2, 0.3)]
    fr = inputs.frames_array([0.0, 0.04, 0.08], rng.normal(size=(3, 3)), worlds, [(0, 0.5, 1)] * 3, [2, 3, 4])
    inputs.write_bundle(tmp_path, V, N, I, fr)
    back = inputs.load_frames(tmp_path)
    assert len(back) == 3
    for k in ("camera_origin", "camera_world", "light_dir", "light_intensity"):
        assert np.array_equal(back[k], fr[k]), k
    assert np.array_equal(back["timestamp_seconds"], fr["timestamp_seconds"].astype(np.float32))
    v2, n2, i2 = inputs.load_mesh(tmp_path)
    assert np.array_equal(v2, V) and np.array_equal(n2, N) and np.array_equal(i2, I)
    (tmp_path / "frames.bin").write_bytes(b"\0" * 20)
    with pytest.raises(ValueError, match="invalid stride|invalid f32 binary size"):
        inputs.load_frames(tmp_path)


# ---- writers --------------------------------------------------------------------------
def read_hdf5(path):
    """Datasets of an HDF5 file with a version-0 superblock, one root group
    (symbol-table B-tree) and contiguous 1-D integer datasets, read by the
    file format specification."""
    b = open(path, "rb").read()
    u = lambda fmt, off: struct.unpack_from("<" + fmt, b, off)[0]  # noqa: E731
    assert b[:8] == b"\x89HDF\r\n\x1a\n" and b[8] == 0 and b[13] == 8 and b[14] == 8
    assert u("Q", 40) == len(b)  # end-of-file address
    leaf_k, internal_k = u("H", 16), u("H", 18)
    root_oh, cache, btree, heap = u("Q", 64), u("I", 72), u("Q", 80), u("Q", 88)
    assert cache == 1

    def messages(addr):
        assert b[addr] == 1
        n, size = u("H", addr + 2), u("I", addr + 8)
        p, out = addr + 16, []
        for _ in range(n):
            t, s = u("H", p), u("H", p + 2)
            assert s % 8 == 0
            out.append((t, b[p + 8:p + 8 + s]))
            p += 8 + s
        assert p == addr + 16 + size
        return dict(out)

    st = messages(root_oh)[0x11]
    assert struct.unpack("<QQ", st) == (btree, heap)
    assert b[heap:heap + 4] == b"HEAP" and b[heap + 4] == 0
    heap_size, free_head, heap_data = u("Q", heap + 8), u("Q", heap + 16), u("Q", heap + 24)
    assert free_head == 1 or free_head < heap_size
    name = lambda off: b[heap_data + off:b.index(b"\0", heap_data + off)].decode()  # noqa: E731
    assert b[btree:btree + 4] == b"TREE" and b[btree + 4] == 0 and b[btree + 5] == 0
    used = u("H", btree + 6)
    out, names = {}, []
    for i in range(used):
        lo_key, child, hi_key = u("Q", btree + 24 + 16 * i), u("Q", btree + 32 + 16 * i), u("Q", btree + 40 + 16 * i)
        assert b[child:child + 4] == b"SNOD" and b[child + 4] == 1
        n = u("H", child + 6)
        assert n <= 2 * leaf_k
        for j in range(n):
            e = child + 8 + 40 * j
            nm = name(u("Q", e))
            names.append(nm)
            msgs = messages(u("Q", e + 8))
            space, dtype, layout = msgs[0x0001], msgs[0x0003], msgs[0x0008]
            assert space[0] == 1 and space[1] == 1
            count = struct.unpack_from("<Q", space, 8)[0]
            assert dtype[0] == 0x10 and dtype[1] & 0x08  # version 1 fixed-point, signed
            size = struct.unpack_from("<I", dtype, 4)[0]
            assert layout[0] == 3 and layout[1] == 1
            addr, nbytes = struct.unpack_from("<QQ", layout, 2)
            assert nbytes == count * size
            out[nm] = np.frombuffer(b[addr:addr + nbytes], "<i%d" % size) if count else np.zeros(0, "<i%d" % size)
        assert name(hi_key) == names[-1] and name(lo_key) == ""
    assert names == sorted(names)
    assert internal_k == 16
    return out


def read_png(path):
    b = open(path, "rb").read()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    p, chunks = 8, []
    while p < len(b):
        n = struct.unpack_from(">I", b, p)[0]
        kind, data = b[p + 4:p + 8], b[p + 8:p + 8 + n]
        assert struct.unpack_from(">I", b, p + 8 + n)[0] == zlib.crc32(kind + data)
        chunks.append((kind, data))
        p += 12 + n
    assert chunks[0][0] == b"IHDR" and chunks[-1][0] == b"IEND"
    w, h, depth, ctype = struct.unpack_from(">IIBB", chunks[0][1])
    assert depth == 8 and ctype == 0
    raw = zlib.decompress(b"".join(d for k, d in chunks if k == b"IDAT"))
    rows = np.frombuffer(raw, np.uint8).reshape(h, w + 1)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:]


def read_tiff_float(path):
    b = open(path, "rb").read()
    assert b[:4] == b"II*\0"
    ifd = struct.unpack_from("<I", b, 4)[0]
    n = struct.unpack_from("<H", b, ifd)[0]
    tags = {}
    for i in range(n):
        tag, typ, cnt, val = struct.unpack_from("<HHII", b, ifd + 2 + 12 * i)
        tags[tag] = val & 0xffff if typ == 3 else val
    assert tags[258] == 32 and tags[259] == 1 and tags[277] == 1 and tags[339] == 3
    w, h = tags[256], tags[257]
    return np.frombuffer(b[tags[273]:tags[273] + tags[279]], "<f4").reshape(h, w)


@pytest.fixture(scope="module")
def selftest(built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("selftest") / "apps_selftest")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", B.APPS, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "apps_selftest.cpp"), "-o", exe, "-L", B.PKG, "-ldvs_gb300",
                    "-Wl,-rpath," + B.PKG], check=True)
    return exe


def test_event_writers(selftest, tmp_path):
    out = subprocess.run([selftest, "events", str(tmp_path)], capture_output=True, text=True, check=True).stdout
    raw = (tmp_path / "events.bin").read_bytes()
    assert len(raw) == 26  # two legacy 13-byte records
    rec = np.frombuffer(raw, np.dtype([("t", "<f4"), ("x", "<i2"), ("y", "<i2"), ("p", "i1"), ("d", "<f4")]))
    assert rec["t"][0] == np.float32(.001234) and list(rec["x"]) == [2, 4] and list(rec["d"]) == [10, 20]
    h5 = read_hdf5(tmp_path / "events.h5")
    assert set(h5) == {"x", "y", "t", "p", "ms_to_idx"}
    assert list(h5["t"]) == [1234, 2100, 50000001, 50000002]  # microseconds, time-sorted
    assert list(h5["x"]) == [2, 4, 2, 2] and list(h5["p"]) == [1, 0, 1, 1]
    idx = h5["ms_to_idx"]
    assert (idx[0], idx[1], idx[2], idx[3], idx[50000], idx[50001]) == (0, 0, 1, 2, 2, 4) and len(idx) == 50002
    assert "h5 events 4" in out
    empty = read_hdf5(tmp_path / "empty.h5")
    assert all(len(v) == 0 for v in empty.values()) and set(empty) == set(h5)
    for what in ("unordered batches", "negative timestamp", "append after close", "nonfinite end"):
        assert "refused " + what in out, out
    assert not list(tmp_path.glob("*.spool"))


def test_image_writers(selftest, tmp_path):
    out = subprocess.run([selftest, "images", str(tmp_path)], capture_output=True, text=True, check=True).stdout
    encoded = [int(v) for v in out.split("encoded")[1].split()]
    img = read_png(tmp_path / "image.png")
    assert img.shape == (5, 37) and list(img.ravel()) == encoded
    # preview encoding: exposure x/100 clamped, sRGB, rounding to bytes
    x = np.clip(np.arange(37 * 5, dtype=np.float32) * np.float32(0.7) / np.float32(100), 0, 1)
    srgb = np.where(x < 0.0031308, 12.92 * x, 1.055 * np.power(x, 1 / 2.4) - 0.055)
    expect = np.where(srgb <= 0, 0, np.where(srgb >= 1, 255, np.floor(srgb * 255 + 0.5)))
    assert np.abs(expect - np.array(encoded)).max() <= 1
    depth = read_tiff_float(tmp_path / "depth.tif")
    i = np.arange(37 * 5)
    assert np.array_equal(depth.ravel(), np.where(i % 7 == 0, -1.0, 100.0 + 0.25 * i).astype(np.float32))
    big = read_png(tmp_path / "big.png")
    assert big.shape == (260, 300) and np.array_equal(big.ravel(), (np.arange(300 * 260) * 7 & 0xff).astype(np.uint8))


# ---- command line ---------------------------------------------------------------------
def run_app(name, *args, cwd=None):
    return subprocess.run([os.path.join(B.BIN, name), *args], capture_output=True, text=True, cwd=cwd, timeout=120)


def test_cli_errors(built, tmp_path):
    r = run_app("dvs")
    assert r.returncode == 1 and "--scene_dir <path>" in r.stdout
    cfg = tmp_path / "c.yaml"
    inputs.write_config(cfg, DAVIS_CAMERA, PHYSIC, SCENE, HAPKE)
    cases = [
        (("--scene_dir", "x", "--config", str(cfg), "--bogus"), "unknown argument: --bogus"),
        (("--config", str(cfg)), "either --scene_dir or --dem and --traj are required"),
        (("--scene_dir", "x", "--config", str(tmp_path / "none.yaml")), "failed to open config file"),
        (("--scene_dir", "x", "--config", str(cfg), "--event_format", "csv"), "invalid event format"),
        (("--scene_dir", "x", "--config", str(cfg), "--solver", "fast"), "solver must be auto"),
        (("--scene_dir", str(tmp_path / "missing"), "--config", str(cfg)), "failed to load scene: failed to open"),
        (("--dem", "a.tif", "--traj", "t.txt", "--config", str(cfg)), "needs GDAL"),
        (("--scene_dir", "x", "--config", str(cfg), "--solver", "adaptive-optics"), "adaptive optics exports HDF5"),
        (("--scene_dir", "x", "--config", str(cfg), "--output"), "missing value for --output"),
        (("--scene_dir", "x", "--config", str(cfg), "--bvh", "fp16"), "bvh must be fp32, half"),
        (("--scene_dir", "x", "--config", str(cfg), "--circuit", "fp16"), "circuit must be fp64, fp32"),
        (("--scene_dir", "x", "--config", str(cfg), "--event_format", "hdf5", "--circuit", "fp32-philox"),
         "adaptive solver keeps the XORWOW"),
    ]
    for args, msg in cases:
        r = run_app("dvs", *args)
        assert r.returncode == 1 and msg in r.stderr, (args, r.stderr)
    r = run_app("cam", "--scene_dir", str(tmp_path / "missing"), "--config", str(cfg))
    assert r.returncode == 1 and "failed to load scene" in r.stderr
