"""The package's camera matrices (render3d's view/projection inputs) against
the oracle's glm restatement, and the sphere mesh helper."""
import numpy as np

from boltzmannfluids_gb300.camera import look_at, perspective
from boltzmannfluids_gb300.workloads import uv_sphere
from oracle.render3d import look_at as look_at_ref, perspective as perspective_ref


def test_camera_matrices_match_glm_restatement():
    for eye, tgt in (((1.4, 0.9, 1.7), (0, 0, 0)), ((-3.0, 2.0, 0.5), (0.2, -0.1, 0.3))):
        assert np.array_equal(look_at(eye, tgt), look_at_ref(eye, tgt))
    for fov, asp in ((0.9, 1.3), (0.6, 16 / 9)):
        assert np.array_equal(perspective(fov, asp, 0.1, 10.0), perspective_ref(fov, asp, 0.1, 10.0))


def test_uv_sphere_is_a_closed_sphere():
    t = uv_sphere(32, 16, 0.5).astype(np.float64)
    assert t.shape == (2 * 32 * 16, 3, 3)
    np.testing.assert_allclose(np.linalg.norm(t, axis=2), 0.5, rtol=1e-6)
    # every edge of the non-degenerate triangles is shared by two triangles
    edges = {}
    for tri in np.round(t, 6):
        if np.linalg.norm(np.cross(tri[1] - tri[0], tri[2] - tri[0])) < 1e-12:
            continue
        for a, b in ((0, 1), (1, 2), (2, 0)):
            k = tuple(sorted((tuple(tri[a]), tuple(tri[b]))))
            edges[k] = edges.get(k, 0) + 1
    assert set(edges.values()) <= {2}
