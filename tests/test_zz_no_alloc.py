"""The camera render that allocates nothing (dvs_cam_render_noalloc).

It exists for callers that cannot allocate device memory while they render
(a frame loop under a fixed memory budget, a framework that owns all device
memory through its own pool, a latency-critical path).  Through the C-ABI,
two calls in a row must give the same image and depth as dvs_cam_render,
within the tolerance of the other GPU tests (1e-5 relative), and images above
the 1280x720 scratch limit must be rejected.  The output buffers are
allocated here by the test (torch), never by the entry point.  This file is
named to be collected last.
"""
import ctypes as C
import math

import numpy as np
import pytest

from dvsrender4deepspace_gb300 import CamRayCaster, DeviceScene, _capi, terrain, trajectory
from dvsrender4deepspace_gb300.raycast import state_array

pytestmark = pytest.mark.gpu

RTOL = 1e-5
HAPKE = dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3)


def test_noalloc_render_matches_allocating_render_twice():
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    V, N, I = terrain.terrain_mesh(96, seed=5)
    cam = dict(width=160, height=120, fx=120.0, fy=120.0, cx=80.0, cy=60.0)
    scene = DeviceScene(V, N, I, cam, 2, HAPKE)
    pose = dict(position=(13.0, -7.0, 700.0), rotation=(0.02, -0.01, 0.3, math.sqrt(1 - 0.02**2 - 0.01**2 - 0.09)),
                light=trajectory.sun_direction(30, 40), intensity=1000)
    want_img, want_dep = CamRayCaster(scene).render_state(pose)
    n = cam["width"] * cam["height"]
    st = state_array(pose)
    stream = torch.cuda.current_stream().cuda_stream
    # every output buffer exists before the first call, so the device's free
    # memory may only change if the entry point itself allocated
    outs = [(torch.full((n,), -7.0, dtype=torch.float32, device="cuda"),
             torch.full((n,), -7.0, dtype=torch.float32, device="cuda")) for _ in range(2)]
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for img, dep in outs:
        r = lib.dvs_cam_render_noalloc(scene.handle, st.ctypes.data, C.c_void_p(img.data_ptr()),
                                       C.c_void_p(dep.data_ptr()), C.c_void_p(stream))
        assert r == _capi.DVS_OK, lib.dvs_last_error()
        torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after >= free_before, "the first calls reserved %d bytes" % (free_before - free_after)
    for img, dep in outs:
        got_img, got_dep = img.cpu().numpy(), dep.cpu().numpy()
        assert np.all(np.isfinite(got_img))
        np.testing.assert_allclose(got_img, want_img, rtol=RTOL, atol=0)
        np.testing.assert_allclose(got_dep, want_dep, rtol=RTOL, atol=0)
    assert (want_img > 0).mean() > 0.5


def test_noalloc_render_without_depth_on_its_own_stream():
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    V, N, I = terrain.terrain_mesh(64, seed=9)
    cam = dict(width=96, height=72, fx=80.0, fy=80.0, cx=48.0, cy=36.0)
    scene = DeviceScene(V, N, I, cam, 1, HAPKE)
    pose = dict(position=(-20.0, 11.0, 500.0), rotation=(0.0, 0.0, 0.0, 1.0),
                light=trajectory.sun_direction(40, 10), intensity=1000)
    want_img, _ = CamRayCaster(scene).render_state(pose)
    st = state_array(pose)
    side = torch.cuda.Stream()
    for call in range(2):
        img = torch.full((cam["width"] * cam["height"],), -7.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        r = lib.dvs_cam_render_noalloc(scene.handle, st.ctypes.data, C.c_void_p(img.data_ptr()), None,
                                       C.c_void_p(side.cuda_stream))
        assert r == _capi.DVS_OK, lib.dvs_last_error()
        side.synchronize()
        np.testing.assert_allclose(img.cpu().numpy(), want_img, rtol=RTOL, atol=0)


def test_noalloc_render_rejects_images_above_the_limit():
    lib = _capi.load()
    V, N, I = terrain.terrain_mesh(16, seed=1)
    cam = dict(width=1281, height=720, fx=1000.0, fy=1000.0, cx=640.0, cy=360.0)
    scene = DeviceScene(V, N, I, cam, 1, HAPKE)
    st = state_array(dict(position=(0, 0, 500), rotation=(0, 0, 0, 1), light=(0, 0, 1), intensity=1000))
    r = lib.dvs_cam_render_noalloc(scene.handle, st.ctypes.data, C.c_void_p(16), None, None)
    assert r == _capi.DVS_ERR_INVALID
    assert b"exceeds the no-allocation scratch limit" in lib.dvs_last_error()
