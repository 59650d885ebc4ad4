"""Synthetic terrain follows the raster builder's triangulation and normal rules."""
import numpy as np

from dvsrender4deepspace_gb300 import terrain


def test_triangle_count_and_winding():
    V, N, I = terrain.terrain_mesh(64, seed=3)
    assert V.shape == (64 * 64, 3) and N.shape == V.shape
    assert I.shape == (2 * 63 * 63, 3)  # 2(n-1)^2, e.g. 130,050 at n = 256
    a, b, c = V[I[:, 0]], V[I[:, 1]], V[I[:, 2]]
    fn = np.cross(b - a, c - a)
    assert np.all(fn[:, 2] > 0)  # T1=(v1,v3,v2), T2=(v2,v3,v4) wind upward
    assert np.allclose(np.linalg.norm(N, axis=1), 1, atol=1e-5)
    assert np.all(N[:, 2] > 0)


def test_seeded_and_bounded():
    h1 = terrain.heightfield(128, seed=11)
    h2 = terrain.heightfield(128, seed=11)
    assert np.array_equal(h1, h2)
    assert not np.array_equal(h1, terrain.heightfield(128, seed=12))
    assert np.abs(h1).max() < 200 + 0.4 * 300 + 1
    assert terrain.heightfield(256, seed=1, craters=0).std() > 10


def test_flat_plane_normals_exact():
    V, N, I = terrain.mesh_from_heightfield(np.zeros((5, 7), np.float32))
    assert np.array_equal(N, np.tile(np.float32([0, 0, 1]), (35, 1)))
    assert V[0, 0] == -30 and V[0, 1] == 20  # row 0 is north (+y)
