"""Host-side wide-BVH checks (CPU): the builder's leaves cover every triangle
once inside their boxes, and the FP16 child bounds of the precision geometry
decode -- origin + offset with the device's directed rounding, re-done here
through the floating-point environment -- to boxes that enclose the FP32 ones,
including beyond the FP16 range (saturated lower bounds, infinite upper ones).
Drives tests/bvh_selftest.cpp linked against libdvs_gb300.so."""
import os
import subprocess

import pytest

from dvsrender4deepspace_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def selftest(tmp_path_factory):
    B.build()
    exe = str(tmp_path_factory.mktemp("bvh") / "bvh_selftest")
    subprocess.run(["g++", "-std=c++17", "-O1", "-frounding-math", "-I", os.path.join(B.PKG, "csrc"),
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "bvh_selftest.cpp"), "-o", exe,
                    "-L", B.PKG, "-ldvs_gb300", "-Wl,-rpath," + B.PKG], check=True)
    return exe


@pytest.mark.parametrize("collapse", [1, 0])  # slot budgets (default), greedy largest-area
@pytest.mark.parametrize("builder", [0, 1])  # binned SAH splits, Morton radix splits
@pytest.mark.parametrize("seed,n,scale,slack", [(1, 64, 1000.0, 2e-3),       # a 1 km tile
                                                (2, 160, 40960.0, 2e-3),     # the 4096^2 terrain's extent
                                                (3, 40, 300000.0, None)])    # offsets beyond 65504
def test_quantised_bounds_enclose_the_fp32_tree(selftest, seed, n, scale, slack, builder, collapse):
    out = subprocess.run([selftest, str(seed), str(n), str(scale), str(builder), str(collapse)], capture_output=True,
                         text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    fields = out.stdout.split()
    assert fields[0] == "nodes" and int(fields[1]) > 0 and int(fields[5]) > 0
    if slack is not None:
        assert float(fields[7]) < slack, out.stdout   # FP16 offsets widen a box by well under 0.2 % of its node


def test_sah_splits_lower_the_surface_area_cost(selftest):
    """On a jittered terrain grid the binned-SAH tree's surface-area model
    (expected wide nodes plus triangle tests per ray through the root box) is
    below the Morton tree's: the SAH splits minimise that cost level by level."""
    got = {}
    for builder in (0, 1):
        out = subprocess.run([selftest, "5", "200", "10000.0", str(builder)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        f = out.stdout.split()
        got[builder] = float(f[9]) + float(f[11])
    assert got[0] < got[1], got  # builder 0: SAH


def test_slot_budget_collapse_lowers_the_node_cost(selftest):
    """The slot-budget collapse minimises the wide nodes' total area (the
    surface-area model's node visits) over every way of grouping the binary
    tree into nodes of at most 8 children; the greedy largest-area collapse is
    one of those groupings, so it can only cost as much or more.  Leaves, and so
    the triangle tests, are the same."""
    for builder in (0, 1):
        got = {}
        for collapse in (0, 1):
            out = subprocess.run([selftest, "7", "300", "20000.0", str(builder), str(collapse)], capture_output=True,
                                 text=True)
            assert out.returncode == 0, out.stdout + out.stderr
            f = out.stdout.split()
            got[collapse] = (float(f[9]), float(f[11]), int(f[5]))
        assert got[1][0] <= got[0][0] * (1 + 1e-6) and got[1][2] == got[0][2], got
        assert abs(got[1][1] - got[0][1]) <= 1e-9 * got[0][1], got


@pytest.mark.parametrize("builder,collapse", [(0, 1), (0, 0), (1, 1)])
def test_tree_is_the_same_at_every_thread_count(selftest, builder, collapse):
    """The builder runs in parallel (chunked binning, subtree tasks, the slot
    tables as post-order tasks, each level's wide nodes at once); the tree it
    returns -- node bytes, triangle order, depth -- is the same with one thread
    as with several.  2.1 M triangles reach every parallel path."""
    hashes = set()
    for threads in ("1", "3", "8"):
        env = dict(os.environ, OMP_NUM_THREADS=threads)
        out = subprocess.run([selftest, "9", "1024", "10240.0", str(builder), str(collapse)], capture_output=True,
                             text=True, env=env)
        assert out.returncode == 0, out.stdout + out.stderr
        f = out.stdout.split()
        assert f[12] == "hash", out.stdout
        hashes.add(f[13])
    assert len(hashes) == 1, hashes
