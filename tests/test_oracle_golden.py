"""Pin the CPU oracle: against fixtures produced by the reference's own compiled
host code (tests/golden/make_golden.py) and against the known answers of the
reference's tests (tests/test_sensor.cu, tests/test_render.cu).  CPU only."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle as O


def test_hapke_matches_reference_bit_exact(oracle32, golden):
    g = golden("hapke")
    for s, h in enumerate(g["params"]):
        hs = O.ohapke(*[float(v) for v in h])
        out = np.array([oracle32.oracle_hapke_reflectance(*map(float, row), C.byref(hs)) for row in g["geometry"]],
                       np.float32)
        np.testing.assert_array_equal(out.view(np.uint32), g["reflectance"][s].view(np.uint32))
        d = []
        for n, l, v in g["vectors"]:
            n, l, v = (np.ascontiguousarray(a, dtype=np.float32) for a in (n, l, v))
            d.append(oracle32.oracle_hapke_directional(O.fptr(n), O.fptr(l), O.fptr(v), 0.3, C.byref(hs)))
        np.testing.assert_array_equal(np.array(d, np.float32).view(np.uint32), g["directional"][s].view(np.uint32))


def test_circuit_matches_reference_bit_exact(oracle32, golden):
    g = golden("circuit")
    for i in range(len(g["rate"])):
        st = g["state"][i]
        s = O.opixel_state(*st, int(g["pending"][i]))
        p = O.opixel_params(*g["params"][i])
        et = np.zeros(64)
        ep = np.zeros(64, np.int32)
        n = oracle32.oracle_advance_pixel(C.byref(s), C.byref(p), float(g["rate"][i]), float(g["t0"][i]),
                                          float(g["t1"][i]), O.dptr(et), ep.ctypes.data_as(C.POINTER(C.c_int32)),
                                          int(g["capacity"][i]))
        assert n == g["count"][i]
        if n > 0:
            np.testing.assert_array_equal(et[:n], g["event_t"][i][:n])
            np.testing.assert_array_equal(ep[:n], g["event_p"][i][:n])
        if n >= 0:
            assert [s.receptor_log, s.reference_log, s.refractory_until] == list(g["state_out"][i][:3])
            assert s.reset_pending == g["pending_out"][i]


def test_bvh_build_matches_reference(oracle32, golden):
    g = golden("bvh")
    V = np.ascontiguousarray(g["vertices"])
    for leaf in (4, 64):
        idx = np.ascontiguousarray(g["indices"]).copy()
        nodes = np.zeros(2 * len(idx), O.NODE_DTYPE)
        cnt = C.c_int()
        root = oracle32.oracle_bvh_build(leaf, O.fptr(V), len(V), idx.ctypes.data_as(C.POINTER(C.c_uint32)),
                                         len(idx), nodes.ctypes.data, C.byref(cnt))
        assert root == int(g["root%d" % leaf])
        np.testing.assert_array_equal(nodes[: cnt.value].view(np.uint8).reshape(-1, 40), g["nodes%d" % leaf])
        np.testing.assert_array_equal(idx, g["indices%d" % leaf])
        assert oracle32.oracle_bvh_validate(nodes.ctypes.data, cnt.value, root) == 0


def _to_oevents(packed):
    out = np.zeros(len(packed), O.EVENT_DTYPE)
    for k in O.PACKED_EVENT_DTYPE.names:
        out[k] = packed[k]
    return out


def test_readout_matches_reference(oracle32, golden):
    g = golden("readout")
    for k in range(4):
        bw, lat, cap = g["s%d_cfg" % k]
        r = oracle32.oracle_readout_create(bw, lat, int(cap))
        for b in range(3):
            ev = _to_oevents(g["s%d_in%d" % (k, b)])
            out = np.zeros(len(ev) + 200000, O.EVENT_DTYPE)
            n = C.c_size_t()
            oracle32.oracle_readout_submit(r, ev.ctypes.data, len(ev), float(g["s%d_now%d" % (k, b)]),
                                           out.ctypes.data, len(out), C.byref(n))
            exp = g["s%d_out%d" % (k, b)]
            assert n.value == len(exp)
            for f in O.PACKED_EVENT_DTYPE.names:
                np.testing.assert_array_equal(out[: n.value][f], exp[f])
        out = np.zeros(200000, O.EVENT_DTYPE)
        n = C.c_size_t()
        oracle32.oracle_readout_drain(r, out.ctypes.data, len(out), C.byref(n))
        exp = g["s%d_drain" % k]
        assert n.value == len(exp)
        np.testing.assert_array_equal(out[: n.value]["timestamp"], exp["timestamp"])
        assert oracle32.oracle_readout_dropped(r) == int(g["s%d_dropped" % k])
        assert oracle32.oracle_readout_peak(r) == int(g["s%d_peak" % k])
        oracle32.oracle_readout_destroy(r)


# ---- known answers of tests/test_sensor.cu:37-55 -------------------------------------------

def _advance(lib, s, p, rate, t0, t1, cap=64):
    et = np.zeros(64)
    ep = np.zeros(64, np.int32)
    n = lib.oracle_advance_pixel(C.byref(s), C.byref(p), rate, t0, t1, O.dptr(et),
                                 ep.ctypes.data_as(C.POINTER(C.c_int32)), cap)
    return n, et[: max(n, 0)], ep[: max(n, 0)]


def _initial(rate, p):
    return O.opixel_state(math.log(rate), math.log(rate), -1.0, p.threshold_pos, p.threshold_neg, 0)


def test_circuit_known_answers(oracle32):
    lib = oracle32
    p = O.opixel_params(0.2, 0.2, 10.0, 0.0, 0.0, 0.0)
    s = _initial(1000, p)
    assert _advance(lib, s, p, 1000, 0, 1)[0] == 0                        # static circuit
    n, et, ep = _advance(lib, s, p, 2000, 0, 0.1)
    assert n == 3                                                          # ON step count
    target = 1000 * math.exp(0.2)
    expected = -p.charge_scale / 2000 * math.log((1 / target - 1 / 2000.0) / (1 / 1000.0 - 1 / 2000.0))
    assert abs(et[0] - expected) < 1e-12                                   # analytic root
    assert et[2] - et[1] > et[1] - et[0]                                   # nonlinear spacing
    bright = et[0]
    s = _initial(100, p)
    n, et, _ = _advance(lib, s, p, 200, 0, 1)
    assert abs(et[0] - 10 * bright) < 1e-12                                # latency x10 at 1/10 light
    s = _initial(2000, p)
    n, et, ep = _advance(lib, s, p, 1000, 0, 0.1)
    assert n == 3 and ep[0] == 0                                           # OFF polarity
    a = _initial(1000, p)
    b = _initial(1000, p)
    _advance(lib, a, p, 2000, 0, 0.1)
    fine = sum(_advance(lib, b, p, 2000, i * 0.001, (i + 1) * 0.001)[0] for i in range(100))
    assert fine == 3 and abs(a.receptor_log - b.receptor_log) < 1e-12 and abs(a.reference_log - b.reference_log) < 1e-12
    s = _initial(1000, p)
    assert _advance(lib, s, p, 2000, 0, 0.1, cap=2)[0] == -1              # overflow
    p.refractory_time = 0.002
    s = _initial(1000, p)
    n, et, _ = _advance(lib, s, p, 100000, 0, 0.01)
    assert n >= 1 and np.all(np.diff(et) >= p.refractory_time - 1e-12)    # refractory spacing
    p.refractory_time = 0.0
    p.reference_leak = 0.4
    s = _initial(1000, p)
    n, et, _ = _advance(lib, s, p, 1000, 0, 1.1)
    assert n == 2 and abs(et[0] - 0.5) < 1e-12                             # leakage
    assert math.isfinite(lib.oracle_receptor_log_at(math.log(1000.0), 0, 10, 10))


def test_fifo_known_answer(oracle32):
    # tests/test_sensor.cu:176-177
    r = oracle32.oracle_readout_create(100, 0.001, 2)
    ev = np.zeros(3, O.EVENT_DTYPE)
    ev["x"] = [0, 1, 2]
    ev["polarity"] = 1
    ev["depth"] = 1
    out = np.zeros(8, O.EVENT_DTYPE)
    n = C.c_size_t()
    oracle32.oracle_readout_submit(r, ev.ctypes.data, 3, 0.005, out.ctypes.data, 8, C.byref(n))
    assert n.value == 0 and oracle32.oracle_readout_dropped(r) == 1
    oracle32.oracle_readout_submit(r, None, 0, 0.012, out.ctypes.data, 8, C.byref(n))
    assert n.value == 1 and abs(out[0]["timestamp"] - 0.011) < 1e-12
    oracle32.oracle_readout_drain(r, out.ctypes.data, 8, C.byref(n))
    assert n.value == 1
    oracle32.oracle_readout_destroy(r)


def test_hapke_known_answers(oracle32):
    # tests/test_sensor.cu:178-180 with the HapkeConfig defaults (scene_types.hpp:204-214)
    hp = dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=26.0 * float(np.float32(math.pi)) / 180.0, w=0.324,
              B_S0=2.42, B_C0=0.0, phi=0.3)
    hs = O.hapke_struct(hp)
    n = np.array([0, 0, 1], np.float32)
    l = np.array([0.8660254, 0, 0.5], np.float32)
    opp = oracle32.oracle_hapke_directional(O.fptr(n), O.fptr(n), O.fptr(n), hp["w"], C.byref(hs))
    ang = oracle32.oracle_hapke_directional(O.fptr(n), O.fptr(l), O.fptr(n), hp["w"], C.byref(hs))
    assert math.isfinite(opp) and opp > ang > 0
    hp.update(phi=0, thetap=0, hC=0, B_C0=0)
    hs = O.hapke_struct(hp)
    assert math.isfinite(oracle32.oracle_hapke_directional(O.fptr(n), O.fptr(n), O.fptr(n), hp["w"], C.byref(hs)))


def test_hapke_identity_form_against_the_fp64_reference_form(oracle32):
    """The CUDA kernels evaluate hapke.hpp:131-151 through exact identities
    (tan(acos(c)/2) = sqrt((1-c)/(1+c)), sin^2(psi/2) = (1-cos psi)/2,
    y^1.5 = y sqrt(y), one quotient for e1/e2).  In FP64 the two forms agree to
    rounding; in FP32 the identity form is as close to the FP64 reference as the
    reference's own FP32 order is, and within 1e-5 of it except where both are."""
    o64 = O.load(True)
    rng = np.random.default_rng(7)

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)
    k = 4000
    l, v = unit(k), unit(k)
    l[:, 2], v[:, 2] = np.abs(l[:, 2]), np.abs(v[:, 2])
    l[:400, 2] *= 1e-3          # grazing light
    v[400:800, 2] *= 1e-3       # grazing view
    l /= np.linalg.norm(l, axis=1, keepdims=True)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    geo = np.stack([l[:, 2], v[:, 2], (l * v).sum(1)], 1).astype(np.float32)
    mats = [dict(b=.3, c=.4, hS=.06, hC=1.0, thetap=0.349066, w=.25, B_S0=1.0, B_C0=0.0, phi=0.3),
            dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=26.0 * float(np.float32(math.pi)) / 180.0, w=0.324,
                 B_S0=2.42, B_C0=0.0, phi=0.3),
            dict(b=.2, c=.5, hS=.05, hC=.05, thetap=0.0, w=.5, B_S0=1.5, B_C0=1.0, phi=0.0),
            # extremes: strong forward lobe, 40 degree roughness, w near 1, porous; near-smooth, dark
            dict(b=.9, c=.1, hS=.01, hC=.02, thetap=0.7, w=0.99, B_S0=3.0, B_C0=1.0, phi=0.6),
            dict(b=.05, c=.9, hS=.5, hC=.5, thetap=1e-9, w=0.01, B_S0=0.0, B_C0=0.5, phi=1e-9)]
    for m in mats:
        hs = O.hapke_struct(m)

        def ev(lib, form, rows=geo):
            return np.array([lib.oracle_hapke_reflectance_form(form, *map(float, g), m["w"], C.byref(hs))
                             for g in rows])
        r32, i32, r64, i64 = ev(oracle32, 0), ev(oracle32, 1), ev(o64, 0), ev(o64, 1)
        ok = np.isfinite(r64) & (np.abs(r64) > 1e-30)
        assert ok.mean() > 0.2
        assert np.array_equal(np.isnan(r32), np.isnan(i32))
        err = lambda a: np.abs(a[ok] - r64[ok]) / np.abs(r64[ok])
        assert err(i64).max() < 1e-13                                   # the identities are exact
        e_ref, e_id = err(r32), err(i32)
        assert np.quantile(e_id, 0.999) <= 1.1 * np.quantile(e_ref, 0.999) + 1e-7
        assert e_id.max() <= 1.1 * e_ref.max() + 1e-7
        assert np.mean(e_id > 1e-5) <= np.mean(e_ref > 1e-5) + 1e-3
        # cos psi clamped to -1: the FP32 reference's tan(pi_f / 2) < 0 overflows exp and
        # makes the sample NaN (dropped by the sampler); FP64 gives a finite value.
        if m["thetap"] > 1e-8:  # the rough branch (hapke.hpp:89 treats thetap <= 1e-8 as smooth)
            corner = np.float32([[0.5, 0.5, -0.51]])
            assert math.isnan(ev(oracle32, 0, corner)[0]) and math.isnan(ev(oracle32, 1, corner)[0])
            a, b = ev(o64, 0, corner)[0], ev(o64, 1, corner)[0]
            assert math.isfinite(a) and abs(a - b) <= 1e-13 * abs(a)


def test_shadow_origins_above_tilted_plane(oracle32):
    # tests/test_render.cu:18-30,95-106: 10000 origins at km coordinates lie outside the plane
    V = np.array([[13000, -13000, 4000], [13005, -13000, 4001.5], [13000, -12995, 4000.75]], np.float32)
    N = np.tile(np.cross(V[1] - V[0], V[2] - V[0]) / np.linalg.norm(np.cross(V[1] - V[0], V[2] - V[0])),
                (3, 1)).astype(np.float32)
    cam = dict(width=4, height=4, fx=1, fy=1, cx=2, cy=2)
    hap = dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=0.45, w=0.324, B_S0=2.42, B_C0=0.0, phi=0.3)
    sc = O.OracleScene(V, N, np.array([[0, 1, 2]]), cam, 1, hap)
    a, b, c = (V[i].astype(np.float64) for i in sc.indices[0])
    nrm = np.cross(b - a, c - a)
    light = np.array([0, 0, 1], np.float32)
    out = np.zeros(3, np.float32)
    failures = 0
    for i in range(10000):
        u = np.float32((i % 100 + 0.5) / 101)
        v = np.float32((i // 100 + 0.5) / 101 * (1 - u))
        oracle32.oracle_shadow_origin(C.byref(sc.s), 0, u, v, O.fptr(light), O.fptr(out))
        if not (np.dot(nrm, out.astype(np.float64) - a) > 0):
            failures += 1
    assert failures == 0


def test_watertight_known_answers(oracle32):
    """Hit distance and barycentrics of the watertight test on a unit right
    triangle: interior, on the hypotenuse, on a vertex, behind the origin,
    and parallel to the plane."""
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    N = np.tile(np.float32([0, 0, 1]), (3, 1))
    cam = dict(width=4, height=4, fx=1, fy=1, cx=2, cy=2)
    hap = dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=0.45, w=0.324, B_S0=2.42, B_C0=0.0, phi=0.3)
    sc = O.OracleScene(V, N, np.array([[0, 1, 2]]), cam, 1, hap, watertight=True)
    tri, t, u, v = C.c_int(), C.c_float(), C.c_float(), C.c_float()

    def hit(o, d):
        o, d = np.float32(o), np.float32(d)
        h = oracle32.oracle_trace_nearest(C.byref(sc.s), O.fptr(o), O.fptr(d), C.byref(tri), C.byref(t),
                                          C.byref(u), C.byref(v))
        return h, t.value, u.value, v.value
    assert hit([0.25, 0.25, 2.0], [0, 0, -1]) == (1, 2.0, 0.25, 0.25)       # u on v1, v on v2
    h, tt, uu, vv = hit([0.5, 0.5, 1.0], [0, 0, -1])                        # the hypotenuse
    assert h == 1 and tt == 1.0 and uu + vv == 1.0
    assert hit([0.0, 0.0, 3.0], [0, 0, -1])[:2] == (1, 3.0)                 # a vertex
    assert hit([0.25, 0.25, -1.0], [0, 0, -1])[0] == 0                      # behind the origin
    assert hit([0.25, 0.25, 1.0], [1, 0, 0])[0] == 0                        # parallel
    assert hit([0.75, 0.75, 1.0], [0, 0, -1])[0] == 0                       # outside


def test_watertight_test_closes_shared_edges(oracle32):
    """The precision geometry's watertight test (Woop et al. 2013): rays aimed at
    the shared diagonal of a two-triangle quad, at km coordinates, always hit
    one of the two triangles (the reference's Moller-Trumbore test may leak
    through the crack); away from the edges both tests give the same hit and t."""
    V = np.array([[12000.25, -7000.5, 350.0], [12010.25, -7000.5, 351.5], [12010.25, -6990.5, 352.25],
                  [12000.25, -6990.5, 350.75]], np.float32)
    N = np.tile(np.float32([0, 0, 1]), (4, 1))
    I = np.array([[0, 1, 2], [0, 2, 3]])
    cam = dict(width=4, height=4, fx=1, fy=1, cx=2, cy=2)
    hap = dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=0.45, w=0.324, B_S0=2.42, B_C0=0.0, phi=0.3)
    wt = O.OracleScene(V, N, I, cam, 1, hap, watertight=True)
    mt = O.OracleScene(V, N, I, cam, 1, hap)
    rng = np.random.default_rng(11)
    tri, t, u, v = C.c_int(), C.c_float(), C.c_float(), C.c_float()

    def trace(sc, o, d):
        h = oracle32.oracle_trace_nearest(C.byref(sc.s), O.fptr(o), O.fptr(d), C.byref(tri), C.byref(t),
                                          C.byref(u), C.byref(v))
        return h, t.value
    a, c = V[0].astype(np.float64), V[2].astype(np.float64)
    wt_miss = mt_miss = 0
    for i in range(4000):
        target = (a + rng.uniform(0.01, 0.99) * (c - a)).astype(np.float32)
        o = (target + np.array([rng.uniform(-300, 300), rng.uniform(-300, 300), rng.uniform(200, 900)])).astype(
            np.float32)
        d = (target.astype(np.float64) - o).astype(np.float64)
        d = (d / np.linalg.norm(d)).astype(np.float32)
        wt_miss += trace(wt, o, d)[0] != 1
        mt_miss += trace(mt, o, d)[0] != 1
    assert wt_miss == 0 and mt_miss > 0, (wt_miss, mt_miss)   # Moller-Trumbore: ~3 % leak through
    # elsewhere: the same hit and distance (a disagreement needs a ray within rounding of an edge)
    disagree = hits = 0
    for i in range(2000):
        target = (V[0] + np.array([rng.uniform(0.5, 9.5), rng.uniform(0.5, 9.5), 0.0])).astype(np.float64)
        o = (target + np.array([rng.uniform(-200, 200), rng.uniform(-200, 200), 600.0])).astype(np.float32)
        d = target - o
        d = (d / np.linalg.norm(d)).astype(np.float32)
        hw, tw = trace(wt, o, d)
        hm, tm = trace(mt, o, d)
        if hw == hm == 1:
            hits += 1
            assert abs(tw - tm) <= 1e-5 * tm
        disagree += hw != hm
    assert hits > 1000 and disagree <= 2


# ---- tests/test_render.cu:37-79 on a cropped DAVIS346 camera ----------------------------------
DAVIS = dict(width=346, height=260, fx=226.3802, fy=226.1500, cx=173.6471, cy=133.7327)
DAVIS_HAPKE = dict(b=0.24, c=0.305, hS=0.08, hC=1.0, thetap=0.453786, w=0.324, B_S0=2.42, B_C0=0.0, phi=0.3)


def half_plane(fp64=False, samples=4, camera=None):
    V = np.array([[-100, 0, 0], [100, 0, 0], [100, 100, 0], [-100, 100, 0]], np.float32)
    N = np.tile([0, 0, 1], (4, 1)).astype(np.float32)
    return O.OracleScene(V, N, np.array([[0, 1, 2], [0, 2, 3]]), camera or DAVIS, samples, DAVIS_HAPKE, fp64=fp64)


def test_render_orientation_misses_and_partial_depth():
    sc = half_plane(samples=4)
    pose = dict(position=(0, 0, 10), rotation=(0, 0, 0, 1), light=(0, 0, 1), intensity=1000)
    rad, dep, val = sc.render(pose)
    assert val.all()
    W, H = DAVIS["width"], DAVIS["height"]
    col = int(DAVIS["cx"])
    assert rad[col] > 0 and dep[col] > 0                                    # +Y appears in upper image
    assert rad[(H - 1) * W + col] == 0 and dep[(H - 1) * W + col] == -1     # miss -> 0 / -1
    row = round(DAVIS["cy"])
    ss = 4
    rng_, hits = 0.0, 0
    for sy in range(ss):
        for sx in range(ss):
            px = (col + (sx + .5) / ss - .5 - DAVIS["cx"]) / DAVIS["fx"]
            py = (row + (sy + .5) / ss - .5 - DAVIS["cy"]) / DAVIS["fy"]
            if py <= 0:
                rng_ += 10 * math.sqrt(1 + px * px + py * py)
                hits += 1
    assert 0 < hits < ss * ss
    assert abs(dep[row * W + col] - rng_ / hits) < 1e-5                    # depth averages hits only
    rad2, dep2, _ = sc.render(pose)
    assert np.array_equal(rad, rad2) and np.array_equal(dep, dep2)         # repeatable


def _plane_sensor(crop=(48, 32), shot=0, circuit_step=1e-6):
    W, H = crop
    cam = dict(width=W, height=H, fx=DAVIS["fx"], fy=DAVIS["fy"], cx=DAVIS["cx"] - (346 - W) / 2,
               cy=DAVIS["cy"] - (260 - H) / 2)
    V = np.array([[-100, -100, 0], [100, -100, 0], [100, 100, 0], [-100, 100, 0]], np.float32)
    N = np.tile([0, 0, 1], (4, 1)).astype(np.float32)
    sc = O.OracleScene(V, N, np.array([[0, 1, 2], [0, 2, 3]]), cam, 1, DAVIS_HAPKE)
    phys = davis_physic(threshold_std=0, photon_shot_noise=shot, max_events_per_step=64, readout_bandwidth=0,
                        readout_latency=0, random_seed=42, circuit_step=circuit_step)
    return sc, phys


def davis_physic(**over):
    p = dict(threshold_pos=0.28, threshold_neg=0.28, threshold_std=0.03, threshold_min=0.01,
             refractory_time=200e-6, wavelength_nm=550, quantum_efficiency=0.3, pixel_pitch_um=15,
             fill_factor=0.2, f_number=2.0, lens_transmission=0.8, radiance_scale=0.001, temperature_k=300,
             subthreshold_kappa=0.8, receptor_capacitance_f=1e-15, reset_capacitance_f=20e-15,
             dark_current_a=1e-18, reset_leakage_a=0, photon_shot_noise=1, reset_thermal_noise=0,
             circuit_step=1e-6, readout_bandwidth=5e6, readout_latency=18e-9, readout_queue_capacity=1000000,
             max_events_per_step=16, random_seed=114514)
    p.update(over)
    return p


POSE = dict(position=(0, 0, 10), rotation=(0, 0, 0, 1), light=(0, 0, 1), intensity=1000)


def test_sensor_static_and_pulse_known_answers():
    # tests/test_sensor.cu:66-80: static -> no events; Hermite pulse -> ON and OFF with depth >= 10
    sc, phys = _plane_sensor()
    s = O.OracleSensor(sc, phys)
    s.initialize(POSE, 0)
    assert len(s.process([(POSE, POSE, 0, 0.002)])) == 0
    start = dict(POSE, intensity_rate=8e6)
    end = dict(POSE, intensity_rate=-8e6)
    ev = s.process([(start, end, 0.002, 0.004)])
    on = int((ev["polarity"] == 1).sum())
    off = int((ev["polarity"] == 0).sum())
    assert on > 0 and off > 0
    assert np.all(ev["depth"] >= 10) and np.all(ev["timestamp"] > 0.002) and np.all(ev["timestamp"] <= 0.004)
    # tests/test_sensor.cu:160-166: halving circuit_step keeps the count, timestamps within 2 us
    sc2, phys2 = _plane_sensor(circuit_step=0.5e-6)
    r = O.OracleSensor(sc2, phys2)
    r.initialize(POSE, 0)
    r.process([(POSE, POSE, 0, 0.002)])
    ev2 = r.process([(start, end, 0.002, 0.004)])
    assert len(ev2) == len(ev)
    assert np.max(np.abs(ev2["timestamp"] - ev["timestamp"])) < 2e-6


def test_sensor_batch_invariance():
    # tests/test_sensor.cu:81-93 with shot noise off
    sc, phys = _plane_sensor()
    bright = dict(POSE, intensity=2000)
    ivs = [(POSE, POSE, 0, 0.001), (bright, bright, 0.001, 0.002), (POSE, POSE, 0.002, 0.003)]
    grouped = O.OracleSensor(sc, phys)
    separate = O.OracleSensor(sc, phys)
    grouped.initialize(POSE, 0)
    separate.initialize(POSE, 0)
    individual = np.concatenate([separate.process([iv]) for iv in ivs])
    allev = grouped.process(ivs)
    assert len(allev) == len(individual) > 0
    for f in ("timestamp", "x", "y", "polarity"):
        np.testing.assert_array_equal(allev[f], individual[f])


def test_sensor_rejects_noncontiguous_intervals():
    sc, phys = _plane_sensor()
    s = O.OracleSensor(sc, phys)
    s.initialize(POSE, 0)
    with pytest.raises(RuntimeError):
        s.process([(POSE, POSE, 0.001, 0.002)])
