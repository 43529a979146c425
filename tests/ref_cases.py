"""Seeded inputs for the configurations the reference-built checker is
compiled for (oracle/build_ref.py CONFIGS).  Each case gives the solver
inputs and the matching oracle / product switches."""
import numpy as np


def smooth_field(res, seed, amp, dims):
    nx, ny, nz = res
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    u = np.zeros((nz, ny, nx, 3))
    for a in range(3 if dims == 3 else 2):
        ph = rng.uniform(0, 2 * np.pi, 3)
        u[..., a] = amp * np.sin(2 * np.pi * x / nx + ph[0]) * np.cos(2 * np.pi * y / ny + ph[1]) * \
            (np.cos(2 * np.pi * z / nz + ph[2]) if dims == 3 else 1.0)
    rho = 1.0 + 0.1 * amp * np.cos(2 * np.pi * (x / nx + y / ny))
    return rho.reshape(-1).astype(np.float32), u.reshape(-1, 3).astype(np.float32)


def ball(res, center, radius):
    nx, ny, nz = res
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cx, cy, cz = center
    return ((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 < radius * radius).reshape(-1)


def case(name):
    """-> dict(res, tau, kwargs for LBM/Oracle/RefShaders, product switches)"""
    d = dict(velocity_set=2, esoteric=True, storage=0, multiphase=False, periodic=(True, True, True),
             objects=None, ids=None, force=None, temperature=None, G=-6.0, tau=0.6, velocity_limit=0.25,
             velocity_limit_extreme=0.30)
    if name == "d2q9_periodic":
        d.update(res=(48, 32, 1))
        d["density"], d["velocity"] = smooth_field(d["res"], 1, 0.05, 2)
    elif name in ("d3q19_periodic", "d3q15_periodic", "d3q27_periodic"):
        d.update(res=(16, 12, 10), velocity_set={"d3q19_periodic": 4, "d3q15_periodic": 3, "d3q27_periodic": 5}[name])
        d["density"], d["velocity"] = smooth_field(d["res"], 2, 0.05, 3)
    elif name == "d2q9_objects_force":
        nx, ny = 48, 24
        d.update(res=(nx, ny, 1), periodic=(False, True, True))
        y, x = np.mgrid[0:ny, 0:nx]
        ids = np.zeros((ny, nx), np.uint32)
        ids[(x - 16) ** 2 + (y - 12) ** 2 < 25] = 1
        ids[-1, :] = 2
        d["ids"] = ids.reshape(-1)
        d["objects"] = {1: dict(velocity=(0, 0, 0)), 2: dict(velocity=(0.05, 0, 0))}
        f = np.zeros((nx * ny, 3), np.float32)
        f[:, 0] = 1e-5
        d["force"] = f
        d["density"], d["velocity"] = smooth_field(d["res"], 3, 0.02, 2)
        d["velocity"][:, 0] += 0.03
    elif name in ("d2q9_thermal", "d3q19_thermal"):
        res = (32, 24, 1) if name == "d2q9_thermal" else (12, 10, 8)
        nx, ny, nz = res
        d.update(res=res, periodic=(True, False, True), velocity_set=2 if nz == 1 else 4)
        ids = np.zeros((nz, ny, nx), np.uint32)
        ids[:, 0, :] = 1
        ids[:, -1, :] = 2
        d["ids"] = ids.reshape(-1)
        d["objects"] = {1: dict(temperature=1.5), 2: dict(temperature=0.5)}
        f = np.zeros((nx * ny * nz, 3), np.float32)
        f[:, 1] = -1e-4
        d["force"] = f
    elif name in ("d2q9_multiphase", "d3q19_multiphase"):
        res = (32, 32, 1) if name == "d2q9_multiphase" else (12, 12, 12)
        rng = np.random.default_rng(4)
        n = res[0] * res[1] * res[2]
        d.update(res=res, velocity_set=2 if res[2] == 1 else 4, multiphase=True, G=-5.0, tau=1.0)
        d["density"] = (0.69 + 0.01 * rng.uniform(-1, 1, n)).astype(np.float32)
    elif name == "d2q9_two_buffer":
        n = 24
        d.update(res=(n, n, 1), periodic=(False, False, True), esoteric=False)
        ids = np.zeros((n, n), np.uint32)
        ids[0, :] = 1
        ids[:, 0] = 1
        ids[:, -1] = 1
        ids[-1, :] = 2
        d["ids"] = ids.reshape(-1)
        d["objects"] = {1: dict(velocity=(0, 0, 0)), 2: dict(velocity=(0.1, 0, 0))}
    elif name == "d2q9_fp16_texture":
        d.update(res=(32, 24, 1), storage=1)
        d["density"], d["velocity"] = smooth_field(d["res"], 5, 0.05, 2)
    elif name == "d2q9_cavity_skip":
        # the 256^2 cavity of the plain-method configuration on the reference's
        # AA path: solid walls and the lid object (u 0.1, which collide.comp
        # never reads) skipped, a seeded flow driven by a constant force
        n = 256
        d.update(res=(n, n, 1), periodic=(False, False, True))
        y, x = np.mgrid[0:n, 0:n]
        ids = np.zeros((n, n), np.uint32)
        ids[(x == 0) | (x == n - 1) | (y == 0)] = 1
        ids[y == n - 1] = 2
        d["ids"] = ids.reshape(-1)
        d["objects"] = {1: dict(velocity=(0, 0, 0)), 2: dict(velocity=(0.1, 0, 0))}
        f = np.zeros((n * n, 3), np.float32)
        f[:, 0] = 2e-7
        d["force"] = f
        d["density"], d["velocity"] = smooth_field(d["res"], 6, 0.05, 2)
    elif name == "d3q19_sphere_skip":
        res = (48, 32, 24)
        d.update(res=res, velocity_set=4)
        d["ids"] = ball(res, (16, 16, 12), 6.0).astype(np.uint32)
        d["objects"] = {1: dict(velocity=(0, 0, 0))}
        d["density"], d["velocity"] = smooth_field(res, 7, 0.03, 3)
        d["velocity"][:, 0] += 0.04
    elif name == "d2q9_von_karman":
        # LBMDemo2D.cpp:65-93 (von_karman_street_periodic) at 256x128: u 1/16,
        # solid cylinder r 8 (the demo's 32 at 1024^2 scaled), tau 0.51
        res = (256, 128, 1)
        d.update(res=res, tau=0.51)
        d["ids"] = ball(res, (64, 64, 0), 8.0).astype(np.uint32)
        d["objects"] = {1: dict(velocity=(0, 0, 0))}
        u = np.zeros((res[0] * res[1], 3), np.float32)
        u[:, 0] = np.float32(1.0 / 16.0)
        d["velocity"] = u
    elif name == "d3q19_droplets_limiter":
        # LBMDemo3D.cpp:95-130 (Shan-Chen droplet collision) at 48x32x32: gas
        # rho 0.056, drops rho 2.659 of radius 6 moving at u = +-1.5 (the
        # demo's 24/16), limits 0.32 / 0.35, tau 0.51: the velocity limiter,
        # its equilibrium-only extreme branch (collide.comp:722-742) and the
        # density floor (:704-705) all act
        res = (48, 32, 32)
        d.update(res=res, velocity_set=4, multiphase=True, tau=0.51, velocity_limit=0.32,
                 velocity_limit_extreme=0.35)
        n = res[0] * res[1] * res[2]
        rho = np.full(n, 0.056, np.float32)
        u = np.zeros((n, 3), np.float32)
        a = ball(res, (48 * 1.2 / 4.0, 16, 16 + 2), 6.0)
        b = ball(res, (48 * 2.8 / 4.0, 16, 16 - 2), 6.0)
        rho[a | b] = 2.659
        u[a, 0] = 24.0 / 16.0
        u[b, 0] = -24.0 / 16.0
        d["density"], d["velocity"] = rho, u
    else:
        raise KeyError(name)
    d.setdefault("density", None)
    d.setdefault("velocity", None)
    return d


NAMES = ["d2q9_periodic", "d3q19_periodic", "d3q15_periodic", "d3q27_periodic", "d2q9_objects_force",
         "d2q9_thermal", "d3q19_thermal", "d2q9_multiphase", "d3q19_multiphase", "d2q9_two_buffer",
         "d2q9_fp16_texture", "d2q9_cavity_skip", "d3q19_sphere_skip", "d2q9_von_karman", "d3q19_droplets_limiter"]
STEPS = [1, 2, 5, 30]
# the stated step counts of the long runs
LONG_STEPS = {"d2q9_cavity_skip": [1, 100, 10000], "d3q19_sphere_skip": [1, 100, 1000],
              "d2q9_von_karman": [1, 100, 1000], "d3q19_droplets_limiter": [1, 100, 1000]}


def steps_of(name):
    return LONG_STEPS.get(name, STEPS)
