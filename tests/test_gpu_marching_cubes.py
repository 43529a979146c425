"""GPU marching cubes (bf_mc_*) against the oracle's restatement: the same
triangles in the same order, bit for bit, on seeded fields and on the density
field of a running solver."""
import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from boltzmannfluids_gb300.marching_cubes import MarchingCubes
from oracle.marching_cubes import extract

pytestmark = pytest.mark.gpu


def smooth_random(res, seed):
    nx, ny, nz = res
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f = np.zeros((nz, ny, nx))
    for _ in range(6):
        k = rng.uniform(0.1, 0.6, 3)
        ph = rng.uniform(0, 2 * np.pi, 3)
        f += np.sin(k[0] * x + ph[0]) * np.cos(k[1] * y + ph[1]) * np.sin(k[2] * z + ph[2])
    return (1.0 + 0.1 * f).astype(np.float32).reshape(-1)


def device_field(arr):
    import torch
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


@pytest.mark.parametrize("res,thr,scale", [((20, 18, 16), 1.0, (1.0, 1.0, 1.0)),
                                           ((33, 17, 9), 1.03, (2.0, 0.5, 1.5))])
def test_gpu_mesh_matches_oracle(res, thr, scale, product_lib):
    field = smooth_random(res, 3)
    d = device_field(field)
    mc = MarchingCubes()
    n = mc.compute_device(d.data_ptr(), res, 1, 0, thr, scale)
    got = mc.vertices()
    ref = extract(field, res, thr, scale)
    assert n == len(ref) > 0
    assert np.array_equal(got, ref)


def test_gpu_mesh_of_solver_density(product_lib):
    res = (24, 20, 16)
    rng = np.random.default_rng(4)
    n = res[0] * res[1] * res[2]
    rho = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.intermolecular_interaction_strength = -5.0
    s.initialize_fields_from_arrays(res, 1.0, density=rho, velocity_set=bf.VelocitySet.D3Q19, is_flow_multiphase=True)
    s.iterate_time(steps=200, save=True)
    dens = s.get_velocity_density_texture().reshape(-1, 4)[:, 3].copy()
    thr = float(np.median(dens))
    tris = MarchingCubes().compute(s, threshold=thr)
    ref = extract(dens, res, thr)
    assert len(tris) == len(ref) > 0
    assert np.array_equal(tris, ref)
