"""Headless volume renderer (bf_render3d) against the oracle's restatement of
the five LBM::render3d_* ray-marchers, on the fields of a running 3D solver
with an object, a force field and a temperature field."""
import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from oracle.render3d import look_at, perspective, render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solver(product_lib):
    nx, ny, nz = 16, 14, 12
    n = nx * ny * nz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ids = np.zeros((nz, ny, nx), np.uint32)
    ids[(x - 7) ** 2 + (y - 6) ** 2 + (z - 5) ** 2 < 9] = 1
    rng = np.random.default_rng(9)
    force = np.zeros((n, 3), np.float32)
    force[:, 0] = 1e-4 * rng.uniform(0.5, 1.0, n)
    temp = (1.0 + 0.2 * np.sin(2 * np.pi * z / nz)).astype(np.float32).reshape(-1)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.set_boundry_properties(1, velocity_translational=(0, 0, 0), temperature=1.5)
    s.initialize_fields_from_arrays((nx, ny, nz), 0.6, force=force, temperature=temp, boundry_id=ids.reshape(-1),
                                    velocity_set=bf.VelocitySet.D3Q19)
    s.iterate_time(steps=30, save=True)
    return s


@pytest.mark.parametrize("mode", list(bf.RenderMode))
def test_render_matches_oracle(solver, mode):
    w, h, samples = 36, 28, 24
    view = look_at((1.4, 0.9, 1.7), (0, 0, 0))
    proj = perspective(0.9, w / h, 0.1, 10.0)
    img = bf.render3d(solver, mode, view, proj, w, h, samples)
    res = solver.get_resolution()
    vd = solver.get_velocity_density_texture().reshape(-1, 4)
    ft = solver.get_force_temperature_texture().reshape(-1, 4)
    bd = solver.get_boundry_texture().reshape(-1)
    ref = render(vd, ft, bd, res, int(mode), view, proj, w, h, samples)
    assert img.shape == ref.shape
    covered = ref[..., 3] != 0
    assert covered.sum() > 50 or mode == bf.RenderMode.boundries
    np.testing.assert_array_equal(img, ref)
