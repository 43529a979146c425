"""The boundary-aware step with the special cells taken out of the lanes
(cells with an empty mask in the periodic kernel's cell update, the listed
special cells in blocks of their own, interleaved in launch order) against
the oracle, bit for bit, and against the single-pass masked kernel."""
import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from boltzmannfluids_gb300.workloads import sphere_channel
from gpu_helpers import make_pair, step_and_compare

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage,collision,forced", [
    (bf.FloatingPointAccuracy.fp32, 1, False),
    (bf.FloatingPointAccuracy.fp32, 0, True),
    (bf.FloatingPointAccuracy.fp16s, 1, True),
    (bf.FloatingPointAccuracy.fp16c, 0, False),
])
def test_sphere_channel_matches_oracle(storage, collision, forced):
    res = (40, 18, 16)
    rho, u, ids, objs = sphere_channel(res, radius=4.0, center=(12.0, 9.0, 8.0))
    n = res[0] * res[1] * res[2]
    force = None
    if forced:
        force = np.zeros((n, 3), np.float32)
        force[:, 1] = 1e-5
    s, o = make_pair(res, 0.55, bf.VelocitySet.D3Q19, density=rho, velocity=u, force=force, ids=ids, objects=objs,
                     periodic=(False, True, True), boundary_mode=1, collision=collision, storage=storage)
    solid = ids != 3
    step_and_compare(s, o, [1, 2, 7, 30], mask=solid)
    assert np.array_equal(s.get_populations(), o.lattice().astype(np.float32))


@pytest.mark.parametrize("q,res,periodic", [
    (bf.VelocitySet.D3Q19, (300, 20, 14), (False, True, True)),   # rows of two blocks
    (bf.VelocitySet.D3Q27, (72, 40, 14), (False, False, True)),   # open y faces too
    (bf.VelocitySet.D2Q9, (64, 40, 1), (False, True, True)),
])
def test_split_equals_single_launch(monkeypatch, q, res, periodic):
    nx, ny, nz = res
    dims = 2 if nz == 1 else 3
    center = (nx / 3, ny / 2, nz / 2 if dims == 3 else 0.0)
    rho, u, ids, objs = sphere_channel(res, radius=4.0, center=center)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("BF_MASKED_SPLIT", flag)
        s = bf.LBM()
        s.is_collide_esoteric = True
        s.collision = bf.Collision.trt
        s.boundary_mode = bf.BoundaryMode.bounce_back
        for k, o in objs.items():
            s.set_boundry_properties(k, velocity_translational=(0, 0, 0), kind=o["kind"])
        s.initialize_fields_from_arrays(res, 0.56, density=rho, velocity=u, boundry_id=ids, periodic=periodic,
                                        velocity_set=q)
        s.iterate_time(steps=41, save=True)
        out.append((s.get_populations(), s.get_velocity_density_texture().copy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
