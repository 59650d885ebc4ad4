"""The packet slab test's sign-specialised bounds (axis_bounds_fixed in
csrc/device_optics.cuh) equal the general four-corner interval bounds of
the packet's slab distances (axis_bounds below) in float32 whenever the
inverse direction keeps one sign -- the only packets the device takes the
interval path for -- so the fast form never culls a node that a ray of the
packet enters.  Both are restated here in numpy float32 (IEEE single
rounding per operation, as the device code is built without contraction)."""
import numpy as np

f32 = np.float32


def axis_bounds(lo, hi, olo, ohi, ilo, ihi):
    def imul(a0, a1, b0, b1):
        p = np.stack([a0 * b0, a0 * b1, a1 * b0, a1 * b1])
        return p.min(0), p.max(0)
    a0, a1 = imul(lo - ohi, lo - olo, ilo, ihi)
    b0, b1 = imul(hi - ohi, hi - olo, ilo, ihi)
    return np.minimum(a0, b0), np.maximum(a1, b1)


def axis_bounds_fixed(lo, hi, olo, ohi, ilo, ihi):
    neg = ihi < 0
    on = np.where(neg, olo, ohi)
    of = np.where(neg, ohi, olo)
    aN = np.where(neg, hi, lo) - on
    aF = np.where(neg, lo, hi) - of
    return aN * np.where(aN >= 0, ilo, ihi), aF * np.where(aF >= 0, ihi, ilo)


def random_case(rng, n):
    c = rng.uniform(-1e4, 1e4, n).astype(f32)
    ext = (10.0 ** rng.uniform(-3, 4, n)).astype(f32)
    lo, hi = c, (c + ext).astype(f32)
    # origins around, inside and on the slab planes
    oc = np.where(rng.random(n) < 0.3, lo, c + rng.uniform(-2e4, 2e4, n).astype(f32)).astype(f32)
    ospan = (10.0 ** rng.uniform(-6, 2, n)).astype(f32) * (rng.random(n) < 0.9)
    olo, ohi = oc, (oc + ospan).astype(f32)
    sign = np.where(rng.random(n) < 0.5, -1, 1).astype(f32)
    mag = (10.0 ** rng.uniform(-4, 20, n)).astype(f32)
    spread = (1 + rng.uniform(0, 0.05, n)).astype(f32)
    a, b = (sign * mag).astype(f32), (sign * mag * spread).astype(f32)
    ilo, ihi = np.minimum(a, b), np.maximum(a, b)
    return lo, hi, olo, ohi, ilo, ihi


def test_fixed_sign_bounds_equal_general_bounds():
    rng = np.random.default_rng(7)
    for _ in range(20):
        args = random_case(rng, 200_000)
        with np.errstate(over="ignore", invalid="ignore"):
            L, U = axis_bounds(*args)
            Lf, Uf = axis_bounds_fixed(*args)
        assert np.array_equal(L, Lf) and np.array_equal(U, Uf)  # == treats -0 and +0 alike


def test_plane_offsets_of_zero():
    lo, hi = f32([1.0, 1.0]), f32([2.0, 2.0])
    olo, ohi = f32([1.0, 2.0]), f32([1.0, 2.0])
    for ilo, ihi in ((f32([0.5, 0.5]), f32([3.0, 3.0])), (f32([-3.0, -3.0]), f32([-0.5, -0.5]))):
        L, U = axis_bounds(lo, hi, olo, ohi, ilo, ihi)
        Lf, Uf = axis_bounds_fixed(lo, hi, olo, ohi, ilo, ihi)
        assert np.array_equal(L, Lf) and np.array_equal(U, Uf)
