"""LBM::iterate_time's tick cadence and throttle (LBM.cpp:220-240), knobs set
between steps, and the macroscopic save/load pair (LBM.h:123, :125) through
the Python mirror of the C ABI."""
import time

import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from gpu_helpers import seeded_fields

pytestmark = pytest.mark.gpu


def periodic_solver(res, vs, rho, u, storage=bf.FloatingPointAccuracy.fp32, velocity_limit=0.25, trt=False):
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.velocity_limit = velocity_limit
    if trt:
        s.collision = bf.Collision.trt
    s.initialize_fields_from_arrays(res, 0.6, density=rho, velocity=u, velocity_set=vs, fp_accuracy=storage)
    return s


def macro_tick(path):
    """The tick stored in a macroscopic file's header (magic, 3 x int32, int32, int64)."""
    return int(np.frombuffer(open(path, "rb").read(32)[24:32], np.int64)[0])


def test_iterate_time_saves_at_most_sixty_times_a_second(tmp_path):
    res = (64, 48, 1)
    rho, u = seeded_fields(res, 3, dims=2)
    s = periodic_solver(res, bf.VelocitySet.D2Q9, rho, u)
    s.iterate_time()  # the first tick always saves
    s.synchronize()
    s.save_current_tick_macroscopic(tmp_path / "a.bin")
    assert s.get_total_ticks_elapsed() == 1 and macro_tick(tmp_path / "a.bin") == 1
    t0 = time.time()
    k = 0
    while time.time() - t0 < 0.010 and k < 5:  # well inside one 1/60 s frame
        s.iterate_time()
        k += 1
    s.synchronize()
    s.save_current_tick_macroscopic(tmp_path / "b.bin")
    assert s.get_total_ticks_elapsed() == 1 + k
    assert macro_tick(tmp_path / "b.bin") == 1  # no save within the frame
    time.sleep(0.03)
    s.iterate_time()
    s.synchronize()
    s.save_current_tick_macroscopic(tmp_path / "c.bin")
    assert macro_tick(tmp_path / "c.bin") == 2 + k  # a frame later the tick saves
    assert s.get_total_time_elapsed() >= 30.0


def test_iterate_time_throttles_to_the_target_rate():
    res = (32, 32, 1)
    rho, u = seeded_fields(res, 4, dims=2)
    s = periodic_solver(res, bf.VelocitySet.D2Q9, rho, u)
    t0 = time.time()
    while time.time() - t0 < 0.5:
        s.iterate_time(40.0)
        time.sleep(0.001)
    s.synchronize()
    ticks = s.get_total_ticks_elapsed()
    # 40 ticks/s over ~0.5 s (the first call always ticks)
    assert 15 <= ticks <= 23, ticks


def test_velocity_limit_set_between_steps_takes_effect():
    """A limiter changed after initialisation reaches the kernels before the
    next step: the same run as a solver initialised with that limit."""
    res = (40, 24, 1)
    rng = np.random.default_rng(5)
    n = res[0] * res[1]
    rho = np.ones(n, np.float32)
    u = np.zeros((n, 3), np.float32)
    u[:, 0] = 0.2 * rng.uniform(-1, 1, n)  # limited by 0.1, not by 0.25
    a = periodic_solver(res, bf.VelocitySet.D2Q9, rho, u)
    a.velocity_limit = 0.1
    a.iterate_time(steps=10, save=True)
    b = periodic_solver(res, bf.VelocitySet.D2Q9, rho, u, velocity_limit=0.1)
    b.iterate_time(steps=10, save=True)
    c = periodic_solver(res, bf.VelocitySet.D2Q9, rho, u)
    c.iterate_time(steps=10, save=True)
    pa, pb, pc = a.get_populations(), b.get_populations(), c.get_populations()
    assert np.array_equal(pa, pb)
    assert not np.array_equal(pa, pc)


@pytest.mark.parametrize("vs,res,storage,steps", [
    (bf.VelocitySet.D2Q9, (48, 32, 1), bf.FloatingPointAccuracy.fp32, 7),
    (bf.VelocitySet.D2Q9, (48, 32, 1), bf.FloatingPointAccuracy.fp32, 8),
    (bf.VelocitySet.D3Q19, (24, 20, 16), bf.FloatingPointAccuracy.fp32, 5),
    (bf.VelocitySet.D3Q19, (24, 20, 16), bf.FloatingPointAccuracy.fp16s, 9),
])
def test_macroscopic_load_restarts_as_initialisation(tmp_path, vs, res, storage, steps):
    """Loading a macroscopic file (at an odd or even tick) gives the state
    initialize_fields would give from the same fields: the next steps agree
    bit for bit with a fresh solver initialised from the saved arrays."""
    rho, u = seeded_fields(res, 11, dims=2 if vs == bf.VelocitySet.D2Q9 else 3)
    a = periodic_solver(res, vs, rho, u, storage=storage, trt=True)
    a.iterate_time(steps=steps, save=True)
    a.synchronize()
    path = tmp_path / "m.bin"
    a.save_current_tick_macroscopic(path)
    assert macro_tick(path) == steps
    saved = a.get_velocity_density_texture().reshape(-1, 4).copy()
    a.iterate_time(steps=3, save=True)  # move on, then restart from the file
    with pytest.raises(bf.LBMError):
        a.load_tick_macroscopic(path, steps + 1)  # wrong tick
    a.load_tick_macroscopic(path, steps)
    assert a.get_total_ticks_elapsed() == steps
    b = periodic_solver(res, vs, saved[:, 3].copy(), saved[:, :3].copy(), storage=storage, trt=True)
    assert np.array_equal(a.get_velocity_density_texture(), b.get_velocity_density_texture())
    for k in (1, 4):
        a.iterate_time(steps=k, save=True)
        b.iterate_time(steps=k, save=True)
        assert np.array_equal(a.get_velocity_density_texture(), b.get_velocity_density_texture())


def cylinder_solver(nx, ny, ids, rho=None, u=None):
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.boundary_mode = bf.BoundaryMode.bounce_back
    s.set_boundry_properties(1, velocity_translational=(0, 0, 0))
    s.initialize_fields_from_arrays((nx, ny, 1), 0.6, density=rho, velocity=u, boundry_id=ids,
                                    periodic=(True, True, True), velocity_set=bf.VelocitySet.D2Q9)
    return s


def test_macroscopic_load_keeps_geometry_and_rejects_other_files(tmp_path):
    """A restart at an odd tick with a solid cylinder under bounce-back: the
    geometry is kept, and the steps after it agree bit for bit with a fresh
    solver of the same geometry initialised from the saved fields."""
    nx, ny = 40, 24
    y, x = np.mgrid[0:ny, 0:nx]
    ids = np.zeros((ny, nx), np.uint32)
    ids[(x - 12) ** 2 + (y - 12) ** 2 < 20] = 1
    u = np.zeros((nx * ny, 3), np.float32)
    u[:, 0] = 0.04
    s = cylinder_solver(nx, ny, ids, u=u)
    s.iterate_time(steps=51, save=True)
    path = tmp_path / "m.bin"
    s.save_current_tick_macroscopic(path)
    saved = s.get_velocity_density_texture().reshape(-1, 4).copy()
    s.iterate_time(steps=20, save=True)
    s.load_tick_macroscopic(path)
    assert np.array_equal(s.get_boundry_texture()[0], ids.astype(np.uint8))
    fresh = cylinder_solver(nx, ny, ids, rho=saved[:, 3].copy(), u=saved[:, :3].copy())
    assert np.array_equal(s.get_velocity_density_texture(), fresh.get_velocity_density_texture())
    for k in (1, 10):
        s.iterate_time(steps=k, save=True)
        fresh.iterate_time(steps=k, save=True)
        assert np.array_equal(s.get_velocity_density_texture(), fresh.get_velocity_density_texture())
    # a file of another resolution or kind leaves the solver as it was
    other = bf.LBM()
    other.initialize_fields_from_arrays((32, 32, 1), 0.6, velocity_set=bf.VelocitySet.D2Q9)
    with pytest.raises(bf.LBMError):
        other.load_tick_macroscopic(path)
    junk = tmp_path / "junk.bin"
    junk.write_bytes(b"\0" * 100)
    before = s.get_velocity_density_texture().copy()
    with pytest.raises(bf.LBMError):
        s.load_tick_macroscopic(junk)
    s.iterate_time(steps=1, save=True)
    fresh.iterate_time(steps=1, save=True)
    assert np.array_equal(s.get_velocity_density_texture(), fresh.get_velocity_density_texture())
    assert not np.array_equal(before, s.get_velocity_density_texture())
