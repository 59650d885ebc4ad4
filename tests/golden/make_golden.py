"""Generate the golden fixtures that pin the oracle to the reference.

Runs the REFERENCE's own host-compilable code (oracle/_ref/libdvsref.so, built
from the reference sources by ``make -C oracle ref``) on seeded inputs and
stores inputs and outputs as small .npz files next to this script:

  hapke.npz    hapke_reflectance / hapke_directional_reflectance
               (include/dvs/hapke.hpp:131-157) on random geometry and three
               parameter sets, plus invert_hapke_if round trips (:160-172)
  circuit.npz  advance_pixel (include/dvs/pixel_model.hpp:34-102) on random
               states, rates and windows, with the reference test's zero
               normal() generator
  bvh.npz      BVHBuilder::build (src/bvh/build.cpp:27-76) node arrays and
               reordered indices for a seeded heightfield at leaf sizes 4, 64
  readout.npz  EventReadout::submit/drain (src/event_readout.cpp:6-34) on
               random event batches with and without a finite FIFO

Usage:  python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
HAPKE_SETS = [
    # the small plain-method workload's parameters (theta-bar 20 deg, CBOE off)
    dict(b=0.3, c=0.4, hS=0.06, hC=1.0, thetap=0.349066, w=0.25, B_S0=1.0, B_C0=0.0, phi=0.3),
    # config/davis346.yaml hapke block
    dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=0.453786, w=0.324, B_S0=2.42, B_C0=0.0, phi=0.3),
    # limits exercised by tests/test_sensor.cu:179-180 plus a CBOE-on set
    dict(b=0.24, c=0.305, hS=0.08, hC=0.0, thetap=0.0, w=0.324, B_S0=2.42, B_C0=0.0, phi=0.0),
    dict(b=0.1, c=-0.2, hS=0.02, hC=0.05, thetap=0.6, w=0.9, B_S0=0.5, B_C0=0.8, phi=0.1),
]
KEYS = ("b", "c", "hS", "hC", "thetap", "w", "B_S0", "B_C0", "phi")


def heightfield_mesh(n, seed):
    rng = np.random.default_rng(seed)
    xs, ys = np.meshgrid(np.arange(n) * 10.0, np.arange(n) * 10.0)
    zs = rng.normal(0, 20, xs.shape)
    V = np.stack([xs - 5 * (n - 1), 5 * (n - 1) - ys, zs], -1).reshape(-1, 3).astype(np.float32)
    tris = []
    for y in range(n - 1):
        for x in range(n - 1):
            v1, v2, v3, v4 = y * n + x, y * n + x + 1, (y + 1) * n + x, (y + 1) * n + x + 1
            tris += [(v1, v3, v2), (v2, v3, v4)]
    return V, np.array(tris, np.uint32)


def main():
    ref = O.load_reference()
    if ref is None:
        raise SystemExit("build the reference harness first: make -C oracle ref")
    lib = O.load()
    rng = np.random.default_rng(20261203)

    # ---- Hapke
    geo = np.stack([rng.uniform(-0.05, 1, 3000), rng.uniform(-0.05, 1, 3000), rng.uniform(-1, 1, 3000),
                    rng.uniform(0, 1, 3000)], 1).astype(np.float32)
    params = np.array([[h[k] for k in KEYS] for h in HAPKE_SETS], np.float32)
    refl = np.zeros((len(HAPKE_SETS), len(geo)), np.float32)
    for s, h in enumerate(params):
        for i, (ci, ce, cg, a) in enumerate(geo):
            refl[s, i] = ref.ref_hapke_reflectance(ci, ce, cg, a, O.fptr(h))
    vecs = rng.normal(size=(500, 3, 3)).astype(np.float32)
    vecs[:, 0, 2] = np.abs(vecs[:, 0, 2]) + 0.1
    dirs = np.zeros((len(HAPKE_SETS), len(vecs)), np.float32)
    for s, h in enumerate(params):
        for i, (n, l, v) in enumerate(vecs):
            n, l, v = (np.ascontiguousarray(a) for a in (n, l, v))
            dirs[s, i] = ref.ref_hapke_directional(O.fptr(n), O.fptr(l), O.fptr(v), 0.3, O.fptr(h))
    np.savez_compressed(os.path.join(OUT, "hapke.npz"), geometry=geo, params=params, reflectance=refl,
                        vectors=vecs, directional=dirs)

    # ---- circuit
    cases = []
    for i in range(1500):
        leak = 0.0 if i % 5 else 0.4
        p = np.array([0.2, 0.25, rng.uniform(1, 300), [0.0, 2e-4, 1e-3][i % 3], leak, 0.0])
        rate = 0.0 if i % 11 == 0 else rng.uniform(1, 1e5)
        st = np.array([np.log(rng.uniform(10, 1e5)), 0, -1, 0.2, 0.25])
        st[1] = st[0] + rng.uniform(-0.3, 0.3)
        if i % 7 == 0:
            st[2] = rng.uniform(0, 1)
        rp = int(rng.integers(0, 2))
        t0 = rng.uniform(0, 1)
        t1 = t0 + rng.uniform(1e-7, 1e-2)
        cap = 64 if i % 13 else 2
        # skip the cases the oracle flags as a reference stall (reference_leak > 0)
        ost = O.opixel_state(*st, rp)
        ot = np.zeros(64)
        op = np.zeros(64, np.int32)
        if lib.oracle_advance_pixel(C.byref(ost), C.byref(O.opixel_params(*p)), rate, t0, t1, O.dptr(ot),
                                    op.ctypes.data_as(C.POINTER(C.c_int32)), cap) == -2:
            continue
        st2 = st.copy()
        rp2 = C.c_int(rp)
        et = np.zeros(64)
        ep = np.zeros(64, np.int32)
        n = ref.ref_advance_pixel(O.dptr(st2), C.byref(rp2), O.dptr(p), rate, t0, t1, O.dptr(et),
                                  ep.ctypes.data_as(O.c_i_p), cap)
        cases.append((p, rate, st, rp, t0, t1, cap, n, et, ep, st2, rp2.value))
    np.savez_compressed(
        os.path.join(OUT, "circuit.npz"),
        params=np.array([c[0] for c in cases]), rate=np.array([c[1] for c in cases]),
        state=np.array([c[2] for c in cases]), pending=np.array([c[3] for c in cases], np.int32),
        t0=np.array([c[4] for c in cases]), t1=np.array([c[5] for c in cases]),
        capacity=np.array([c[6] for c in cases], np.int32), count=np.array([c[7] for c in cases], np.int32),
        event_t=np.array([c[8] for c in cases]), event_p=np.array([c[9] for c in cases], np.int32),
        state_out=np.array([c[10] for c in cases]), pending_out=np.array([c[11] for c in cases], np.int32))

    # ---- BVH build
    V, I = heightfield_mesh(40, 7)
    out = {"vertices": V, "indices": I}
    for leaf in (4, 64):
        idx = I.copy()
        nodes = np.zeros(2 * len(I), O.NODE_DTYPE)
        cnt = C.c_int()
        root = ref.ref_bvh_build(leaf, O.fptr(V), len(V), idx.ctypes.data_as(C.POINTER(C.c_uint32)), len(I),
                                 nodes.ctypes.data, C.byref(cnt))
        out["nodes%d" % leaf] = nodes[: cnt.value].view(np.uint8).reshape(cnt.value, 40)
        out["indices%d" % leaf] = idx
        out["root%d" % leaf] = np.int32(root)
    np.savez_compressed(os.path.join(OUT, "bvh.npz"), **out)

    # ---- readout
    streams = {}
    for k, (bw, lat, cap, n) in enumerate([(0.0, 0.0, 10, 300), (5e6, 18e-9, 1000000, 400),
                                           (100.0, 1e-3, 2, 50), (2e4, 5e-5, 8, 600)]):
        r = ref.ref_readout_create(bw, lat, cap)
        outs = []
        now = 0.0
        for b in range(3):
            ev = np.zeros(n, O.PACKED_EVENT_DTYPE)
            ev["timestamp"] = now + np.round(rng.uniform(0, 1e-3, n), 7)
            ev["x"] = rng.integers(0, 16, n)
            ev["y"] = rng.integers(0, 16, n)
            ev["polarity"] = rng.integers(0, 2, n)
            ev["depth"] = rng.uniform(1, 100, n)
            now += 1e-3
            ready = np.zeros(n + 200000, O.PACKED_EVENT_DTYPE)
            m = ref.ref_readout_submit(r, ev.ctypes.data, n, now, ready.ctypes.data, len(ready))
            streams["s%d_in%d" % (k, b)] = ev
            streams["s%d_now%d" % (k, b)] = np.float64(now)
            streams["s%d_out%d" % (k, b)] = ready[:m]
        ready = np.zeros(200000, O.PACKED_EVENT_DTYPE)
        m = ref.ref_readout_drain(r, ready.ctypes.data, len(ready))
        streams["s%d_drain" % k] = ready[:m]
        streams["s%d_cfg" % k] = np.array([bw, lat, cap])
        streams["s%d_dropped" % k] = np.int64(ref.ref_readout_dropped(r))
        streams["s%d_peak" % k] = np.int64(ref.ref_readout_peak(r))
        ref.ref_readout_destroy(r)
    np.savez_compressed(os.path.join(OUT, "readout.npz"), **streams)
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    main()
