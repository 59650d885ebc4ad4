"""C-ABI library checks that need no GPU: it loads, exports every symbol the
header declares, keeps the reference's struct layouts, derives the pixel
parameters exactly as the oracle does, and rejects invalid arguments before
touching the device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import _capi
from dvsrender4deepspace_gb300 import build as dvs_build
from dvsrender4deepspace_gb300.raycast import camera_struct, hapke_struct, physic_struct

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    dvs_build.build()
    return _capi.load()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "dvs_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dvs_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 19
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_capi.EXPORTS)


def test_struct_layouts_match_reference():
    assert _capi.STATE_DTYPE.itemsize == 80      # OpticalState with float4 alignment
    assert _capi.INTERVAL_DTYPE.itemsize == 176  # OpticalInterval
    assert _capi.EVENT_DTYPE.itemsize == 17      # packed Event
    assert C.sizeof(_capi.Physic) == 26 * 4


def test_version(lib):
    assert b"sm_103a" in lib.dvs_version()


def test_derive_parameters_matches_oracle(lib):
    from oracle import oracle as O
    from tests.test_oracle_golden import davis_physic
    ol = O.load()
    for effects in (0, 1):
        for over in ({}, dict(reset_leakage_a=1e-16, reset_thermal_noise=1), dict(f_number=1.4, circuit_step=0.5e-6)):
            phys = davis_physic(**over)
            out = (C.c_double * 9)()
            assert lib.dvs_derive_parameters(C.byref(physic_struct(phys)), effects, out) == 0
            p, ph = O.opixel_params(), O.ophoto()
            ol.oracle_derive_parameters(C.byref(O.physic_struct(phys)), effects, C.byref(p), C.byref(ph))
            want = [p.threshold_pos, p.threshold_neg, p.charge_scale, p.refractory_time, p.reference_leak,
                    p.reset_noise_std, ph.electrons_per_radiance, ph.dark_electrons, ph.integration_step]
            assert list(out) == want


def test_scene_create_rejects_invalid_arguments_on_host(lib):
    V = np.zeros((3, 3), np.float32)
    I = np.array([[0, 1, 5]], np.uint32)  # index outside the vertex array
    cam = camera_struct(dict(width=4, height=4, fx=1, fy=1, cx=2, cy=2))
    h = C.c_void_p()
    fp = C.POINTER(C.c_float)
    hap = hapke_struct(dict(b=.24, c=.3, hS=.08, hC=1, thetap=.4, w=.3, B_S0=2, B_C0=0, phi=.3))
    r = lib.dvs_scene_create(V.ctypes.data_as(fp), V.ctypes.data_as(fp), I.ctypes.data_as(C.POINTER(C.c_uint32)),
                             None, 3, 1, C.byref(cam), 1, C.byref(hap), None, C.byref(h))
    assert r == _capi.DVS_ERR_INVALID and b"index" in lib.dvs_last_error()
    bad = camera_struct(dict(width=0, height=4, fx=1, fy=1, cx=2, cy=2))
    I = np.array([[0, 1, 2]], np.uint32)
    r = lib.dvs_scene_create(V.ctypes.data_as(fp), V.ctypes.data_as(fp), I.ctypes.data_as(C.POINTER(C.c_uint32)),
                             None, 3, 1, C.byref(bad), 1, C.byref(hap), None, C.byref(h))
    assert r == _capi.DVS_ERR_INVALID
    V[1, 0] = np.nan
    r = lib.dvs_scene_create(V.ctypes.data_as(fp), V.ctypes.data_as(fp), I.ctypes.data_as(C.POINTER(C.c_uint32)),
                             None, 3, 1, C.byref(cam), 1, C.byref(hap), None, C.byref(h))
    assert r == _capi.DVS_ERR_INVALID and b"nonfinite" in lib.dvs_last_error()
    V[1, 0] = 1.0
    for params in (_capi.BvhParams(0, 0, 7), _capi.BvhParams(0, 9, 0)):  # unknown builder, unknown flags
        r = lib.dvs_scene_create(V.ctypes.data_as(fp), V.ctypes.data_as(fp),
                                 I.ctypes.data_as(C.POINTER(C.c_uint32)), None, 3, 1, C.byref(cam), 1,
                                 C.byref(hap), C.byref(params), C.byref(h))
        assert r == _capi.DVS_ERR_INVALID and b"BVH" in lib.dvs_last_error()


def test_cpp_facade_compiles_links_and_throws(lib, tmp_path):
    """The C++17 facade (include/dvs_gb300.hpp) builds against the library and
    maps an invalid argument to std::invalid_argument, as the reference does."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    src = tmp_path / "facade.cpp"
    src.write_text(r'''
#include "dvs_gb300.hpp"
#include <cstdio>
// compiled and linked, not called (it needs a GPU): the batch facade's API
void batch_api(std::vector<dvs_gb300::DvsRayCaster *> members,
               const std::vector<std::vector<dvs_optical_interval>> &ivs) {
  dvs_gb300::SensorBatch batch(members);
  std::vector<std::vector<dvs_event>> events;
  batch.advance_many(ivs, events);
  std::printf("%llu\n", (unsigned long long)batch.stats().graph_launches);
}
int main() {
  dvs_camera cam{4, 4, 1.f, 1.f, 2.f, 2.f};
  dvs_hapke hap{.24f, .3f, .08f, 1.f, .4f, .3f, 2.f, 0.f, .3f};
  std::vector<float> v(9, 0.f), n(9, 0.f);
  std::vector<uint32_t> i{0, 1, 7};
  try { dvs_gb300::DeviceScene s(v, n, i, cam, 1, hap); }
  catch (const std::invalid_argument &e) { std::printf("invalid_argument: %s\n", e.what()); return 0; }
  return 1;
}
''')
    exe = tmp_path / "facade"
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        _capi.library_path(), "-Wl,-rpath," + os.path.dirname(_capi.library_path())],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "index" in r.stdout, r.stdout + r.stderr


def test_library_readout_matches_reference_fixtures(lib, golden):
    """The library's FIFO (readout.cpp) against the reference EventReadout's
    outputs on the same batches (tests/golden/readout.npz)."""
    from dvsrender4deepspace_gb300.raycast import EventReadout
    g = golden("readout")
    for k in range(4):
        bw, lat, cap = g["s%d_cfg" % k]
        r = EventReadout(bw, lat, int(cap))
        for b in range(3):
            out = r.submit(g["s%d_in%d" % (k, b)], float(g["s%d_now%d" % (k, b)]))
            exp = g["s%d_out%d" % (k, b)]
            assert len(out) == len(exp)
            for f in exp.dtype.names:
                np.testing.assert_array_equal(out[f], exp[f])
        out = r.drain()
        np.testing.assert_array_equal(out["timestamp"], g["s%d_drain" % k]["timestamp"])
        assert r.dropped() == int(g["s%d_dropped" % k]) and r.peak_queue() == int(g["s%d_peak" % k])


def test_library_fifo_known_answer(lib):
    # tests/test_sensor.cu:176-177
    from dvsrender4deepspace_gb300.raycast import EventReadout
    r = EventReadout(100, .001, 2)
    ev = np.zeros(3, _capi.EVENT_DTYPE)
    ev["x"] = [0, 1, 2]
    ev["polarity"] = 1
    ev["depth"] = 1
    assert len(r.submit(ev, .005)) == 0 and r.dropped() == 1
    out = r.submit(np.zeros(0, _capi.EVENT_DTYPE), .012)
    assert len(out) == 1 and abs(out[0]["timestamp"] - .011) < 1e-12
    assert len(r.drain()) == 1


def test_sensor_calls_reject_null_handles(lib):
    h = C.c_void_p()
    assert lib.dvs_sensor_create(None, None, None, C.byref(h)) == _capi.DVS_ERR_INVALID
    n = C.c_size_t()
    assert lib.dvs_sensor_process(None, None, 0, C.byref(n)) == _capi.DVS_ERR_INVALID
    assert lib.dvs_sensor_initialize(None, None, 0.0) == _capi.DVS_ERR_INVALID
    assert lib.dvs_cam_render(None, None, None, None) == _capi.DVS_ERR_INVALID
