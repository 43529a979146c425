"""GPU mesh voxeliser (bf_voxelize_mesh) against the oracle's ray-parity
restatement: identical masks on closed meshes, including column centres that
fall exactly on shared edges and vertices."""
import numpy as np
import pytest

from boltzmannfluids_gb300.marching_cubes import voxelize_mesh
from oracle.voxelize import icosphere, voxelize

pytestmark = pytest.mark.gpu


def cube_mesh(lo, hi):
    """Axis-aligned box as 12 outward-oriented triangles."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4), (2, 3, 7), (2, 7, 6), (1, 2, 6), (1, 6, 5),
         (0, 4, 7), (0, 7, 3)]
    return v[np.array(f)]


def rotation(ax, ay):
    cx, sx, cy, sy = np.cos(ax), np.sin(ax), np.cos(ay), np.sin(ay)
    rx = np.array([[1, 0, 0, 0], [0, cx, -sx, 0], [0, sx, cx, 0], [0, 0, 0, 1]])
    ry = np.array([[cy, 0, sy, 0], [0, 1, 0, 0], [-sy, 0, cy, 0], [0, 0, 0, 1]])
    return (rx @ ry).T.astype(np.float32).reshape(-1)  # column-major


@pytest.mark.parametrize("mesh,res,samples,model", [
    (icosphere(2, 0.6), (24, 24, 24), 64, None),
    (icosphere(3, 0.8, (0.1, -0.05, 0.0)), (32, 20, 28), 16, None),
    # edges and vertices on column centres: a box with corners at centres of a 16^3 grid
    (cube_mesh((-0.625, -0.625, -0.5), (0.375, 0.625, 0.5)), (16, 16, 16), 64, None),
    (cube_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)), (20, 18, 22), 8, rotation(0.3, 0.7)),
])
def test_gpu_voxeliser_matches_oracle(mesh, res, samples, model, product_lib):
    got = voxelize_mesh(mesh, res, samples, model).reshape(-1)
    ref = voxelize(mesh.reshape(-1), res, samples, model)
    assert got.sum() > 0
    assert np.array_equal(got, ref), int(np.sum(got != ref))
