"""The C++ facade (include/bf/LBM.hpp) compiles against the C ABI, links the
in-tree library and, on a GPU, reproduces the Python API's result bit for bit."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "boltzmannfluids_gb300")


def build_demo(tmp_path, name="lid_cavity_demo"):
    exe = str(tmp_path / name)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-L", LIBDIR,
                           "-lbfgb300", f"-Wl,-rpath,{LIBDIR}", "-o", exe])
    return exe


def test_facade_compiles_and_links(product_lib, tmp_path):
    for name in ("lid_cavity_demo", "adjoint_demo", "facade_knobs_demo"):
        assert os.path.exists(build_demo(tmp_path, name))


def test_facade_reports_missing_device(product_lib, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    exe = build_demo(tmp_path)
    r = subprocess.run([exe, "16", "1", str(tmp_path / "o.bin")], capture_output=True, text=True)
    assert r.returncode == 2 and "[LBM Error]" in r.stderr


@pytest.mark.gpu
def test_facade_matches_python_api(product_lib, tmp_path):
    import boltzmannfluids_gb300 as bf
    exe = build_demo(tmp_path)
    n, steps = 48, 300
    out = tmp_path / "cavity.bin"
    r = subprocess.run([exe, str(n), str(steps), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.float32).reshape(n, n, 4)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.boundary_mode = bf.BoundaryMode.bounce_back
    s.set_boundry_properties(1, (0.0, 0.0, 0.0))
    s.set_boundry_properties(2, (0.1, 0.0, 0.0))
    y, x = np.mgrid[0:n, 0:n]
    ids = np.zeros((n, n), np.uint32)
    ids[(x == 0) | (x == n - 1) | (y == 0)] = 1
    ids[y == n - 1] = 2
    s.initialize_fields_from_arrays((n, n, 1), 0.6, boundry_id=ids, periodic=(False, False, True),
                                    velocity_set=bf.VelocitySet.D2Q9)
    s.iterate_time(steps=steps, save=True)
    ref = s.get_velocity_density_texture().reshape(n, n, 4)
    assert np.array_equal(got, ref)


@pytest.mark.gpu
def test_facade_adjoint_matches_python_api(product_lib, tmp_path):
    """bf::Adjoint's forward/backward pair gives the Python AdjointChannel's
    objective and gradients bit for bit (the same library underneath)."""
    from boltzmannfluids_gb300.adjoint import AdjointChannel, channel_setup
    import boltzmannfluids_gb300 as bf
    res, steps, K = (64, 32, 1), 120, 40
    s, u_in, tgt = channel_setup(res)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        for a in (s, u_in, tgt):
            np.ascontiguousarray(a, np.float32).tofile(f)
    out = tmp_path / "out.bin"
    exe = build_demo(tmp_path, "adjoint_demo")
    r = subprocess.run([exe, *map(str, res), str(steps), str(K), str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.float64)
    n, rows = res[0] * res[1] * res[2], res[1] * res[2]
    g = AdjointChannel(res, 0.6, bf.VelocitySet.D2Q9, steps, K)
    g.set_parameters(s, u_in)
    g.set_target(tgt)
    j = g.forward()
    gs, gu = g.backward()
    assert got[0] == j
    assert np.array_equal(got[1:1 + n], gs) and np.array_equal(got[1 + n:1 + n + rows], gu)


@pytest.mark.gpu
def test_facade_knobs_and_macroscopic_restart_match_python_api(product_lib, tmp_path):
    """The C++ facade's knob changes between steps (velocity limit, thermal
    relaxation time set after initialisation, an invalid value refused), the
    reference-cadence iterate_time and the macroscopic save/load give the
    Python mirror's result bit for bit."""
    import boltzmannfluids_gb300 as bf
    nx, ny = 40, 24
    exe = build_demo(tmp_path, "facade_knobs_demo")
    out, macro = tmp_path / "out.bin", tmp_path / "macro_cpp.bin"
    r = subprocess.run([exe, str(nx), str(ny), str(out), str(macro)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, np.uint8)
    ticks = int(raw[:4].view(np.int32)[0])
    got = raw[4:].view(np.float32).reshape(2, ny, nx, 4)
    s = bf.LBM()
    s.clear_boundry_properties()
    s.set_boundry_properties(1, (0.0, 0.0, 0.0), 1.5)
    s.set_boundry_properties(2, (0.0, 0.0, 0.0), 0.5)
    s.is_collide_esoteric = True
    s.boundary_mode = bf.BoundaryMode.bounce_back
    s.thermal_init_equilibrium = True
    y, x = np.mgrid[0:ny, 0:nx]
    ids = np.zeros((ny, nx), np.uint32)
    ids[y == 0] = 1
    ids[y == ny - 1] = 2
    # the demo's lambda: 1 + 0.01 * ((7x + 3y) % 5 - 2), in FP32
    temp = (np.float32(1.0) + np.float32(0.01) * ((x * 7 + y * 3) % 5 - 2).astype(np.float32)).astype(np.float32)
    force = np.zeros((nx * ny, 3), np.float32)
    force[:, 1] = np.float32(-1e-4)
    s.initialize_fields_from_arrays((nx, ny, 1), 0.6, force=force, temperature=temp, boundry_id=ids,
                                    periodic=(True, False, True), velocity_set=bf.VelocitySet.D2Q9)
    s.thermal_relaxation_time = 0.8
    s.iterate_time(steps=20, save=False)
    s.velocity_limit = 0.001
    s.iterate_time(steps=20, save=False)
    s.thermal_relaxation_time = 0.4
    with pytest.raises(bf.LBMError):
        s.iterate_time(steps=1, save=False)
    s.thermal_relaxation_time = 0.8
    for _ in range(5):
        s.iterate_time()
    s.iterate_time(steps=1, save=True)
    s.save_current_tick_macroscopic(tmp_path / "macro_py.bin")
    s.iterate_time(steps=7, save=False)
    s.load_tick_macroscopic(tmp_path / "macro_py.bin")
    s.iterate_time(steps=3, save=True)
    assert ticks == s.get_total_ticks_elapsed() == 49
    assert open(macro, "rb").read() == open(tmp_path / "macro_py.bin", "rb").read()
    assert np.array_equal(got[0], s.get_velocity_density_texture()[0])
    assert np.array_equal(got[1], s.get_force_temperature_texture()[0])
