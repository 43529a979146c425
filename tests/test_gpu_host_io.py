"""Host buffers through the C ABI: page-locked (pinned) arrays are read and
written by kernels in place, pageable ones go through cudaMemcpy.  Both
routes must give the same solver state and the same bytes."""
import ctypes as C

import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from boltzmannfluids_gb300.lbm import Field

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned_copy(a):
    t = torch.from_numpy(np.ascontiguousarray(a).reshape(-1)).pin_memory()
    return t, t.numpy().reshape(a.shape)


def solver(res, rho, u, storage):
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.collision = bf.Collision.trt
    s.initialize_fields_from_arrays(res, 0.56, density=rho, velocity=u, velocity_set=bf.VelocitySet.D3Q19,
                                    fp_accuracy=storage)
    return s


@pytest.mark.parametrize("storage", [bf.FloatingPointAccuracy.fp32, bf.FloatingPointAccuracy.fp16s])
def test_pinned_initial_arrays_equal_pageable(storage):
    res = (40, 24, 18)
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(21)
    rho = (1 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    u = (0.03 * rng.uniform(-1, 1, (n, 3))).astype(np.float32)
    keep_r, rho_p = pinned_copy(rho)
    keep_u, u_p = pinned_copy(u)
    a = solver(res, rho, u, storage)
    b = solver(res, rho_p, u_p, storage)
    assert np.array_equal(a.get_populations(), b.get_populations())
    a.iterate_time(steps=7, save=True)
    b.iterate_time(steps=7, save=True)
    assert np.array_equal(a.get_velocity_density_texture(), b.get_velocity_density_texture())
    del keep_r, keep_u


@pytest.mark.parametrize("offset", [0, 4])
def test_readback_into_pinned_buffer(offset):
    res = (33, 20, 17)  # 11220 cells: the u/rho field is 179,520 bytes
    n = res[0] * res[1] * res[2]
    rng = np.random.default_rng(22)
    u = (0.03 * rng.uniform(-1, 1, (n, 3))).astype(np.float32)
    s = solver(res, None, u, bf.FloatingPointAccuracy.fp32)
    s.iterate_time(steps=5, save=True)
    ref = s.get_velocity_density_texture().reshape(-1)
    lib = bf.load_library()
    # offset 4: a destination that is not 16-byte aligned takes the cudaMemcpy route
    buf = torch.zeros(n * 4 + 8, dtype=torch.float32).pin_memory()
    view = buf.numpy()
    addr = view.ctypes.data + offset
    rc = lib.bf_copy_field_to_host(s._h, int(Field.velocity_density), C.c_void_p(addr), n * 16)
    assert rc == 0, lib.bf_last_error()
    got = np.frombuffer((C.c_char * (n * 16)).from_address(addr), dtype=np.float32)
    assert np.array_equal(got, ref)
