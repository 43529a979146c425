"""Seeded synthetic initial conditions of the standard workloads (numpy
arrays in x-fastest cell order, ready for LBM.initialize_fields_from_arrays)."""
import numpy as np


def taylor_green_3d(res, u0=0.05):
    """3D Taylor-Green vortex on a periodic box, lattice units:
    u = u0 sin(kx) cos(ky) cos(kz), v = -u0 cos(kx) sin(ky) cos(kz), w = 0,
    rho = 1 + 3 p' with p' = u0^2/16 (cos 2kx + cos 2ky)(cos 2kz + 2)
    (cs^2 = 1/3), k = 2 pi / edge per axis.  Returns (rho[N], u[N, 3]) float32."""
    nx, ny, nz = (int(v) for v in res)
    x = 2 * np.pi * (np.arange(nx) + 0.5) / nx
    y = 2 * np.pi * (np.arange(ny) + 0.5) / ny
    z = 2 * np.pi * (np.arange(nz) + 0.5) / nz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    u = np.zeros((nz, ny, nx, 3))
    u[..., 0] = u0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    u[..., 1] = -u0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    p = u0 * u0 / 16.0 * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0)
    rho = 1.0 + 3.0 * p
    return rho.reshape(-1).astype(np.float32), u.reshape(-1, 3).astype(np.float32)


def noisy_rest(res, amplitude=1e-4, seed=1):
    """rho = 1 and u uniform in [-amplitude, amplitude] per component (seeded)."""
    n = int(res[0]) * int(res[1]) * int(res[2])
    rng = np.random.default_rng(seed)
    return np.ones(n, np.float32), rng.uniform(-amplitude, amplitude, (n, 3)).astype(np.float32)


def spinodal(res, rho0=0.69, amplitude=0.01, seed=4):
    """Shan-Chen spinodal decomposition start: rho = rho0 + amplitude U(-1, 1), u = 0."""
    n = int(res[0]) * int(res[1]) * int(res[2])
    rng = np.random.default_rng(seed)
    return (rho0 + amplitude * rng.uniform(-1, 1, n)).astype(np.float32)


def rayleigh_benard(res, ra=1e5, pr=0.71, kappa=0.008, beta=0.5, seed=5, storage=None):
    """Hot bottom (T = 1) and cold top (T = 0) walls at z = 0 and z = nz-1,
    periodic x and y; gravity along -z sized for Rayleigh number `ra` with
    H = nz - 2 fluid layers, D3Q7 diffusivity kappa = (tau_T - 1/2)/4 and
    nu = pr kappa; Boussinesq force F (1 - beta (T - 1)) from the solver's
    thermal coupling (the reference's buoyancy form).
    -> (solver, kappa, h)."""
    from . import lbm as bf
    if storage is None:
        storage = bf.FloatingPointAccuracy.fp32
    nx, ny, nz = res
    n = nx * ny * nz
    h = nz - 2
    nu = pr * kappa
    tau, tau_t = 3 * nu + 0.5, 4 * kappa + 0.5
    # buoyancy contrast across the layer: g beta dT with dT = 1
    g = ra * nu * kappa / (beta * h ** 3)
    z = np.repeat(np.arange(nz), nx * ny)
    ids = np.zeros(n, np.uint32)
    ids[z == 0] = 1
    ids[z == nz - 1] = 2
    rng = np.random.default_rng(seed)
    zf = (z - 0.5) / h
    temp = (1.0 - np.clip(zf, 0, 1) + 1e-3 * rng.uniform(-1, 1, n)).astype(np.float32)
    force = np.zeros((n, 3), np.float32)
    force[:, 2] = -g
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.boundary_mode = bf.BoundaryMode.bounce_back
    s.collision = bf.Collision.trt
    s.thermal_expansion_coefficient = beta
    s.thermal_init_equilibrium = True
    s.set_boundry_properties(1, velocity_translational=(0, 0, 0), temperature=1.0)
    s.set_boundry_properties(2, velocity_translational=(0, 0, 0), temperature=0.0)
    s.initialize_fields_from_arrays(res, tau, force=force, temperature=temp, boundry_id=ids,
                                    periodic=(True, True, False), velocity_set=bf.VelocitySet.D3Q19,
                                    fp_accuracy=storage)
    # initialisation resets the thermal relaxation time to 2 (LBM.cpp:461);
    # the flow's value takes effect from the first step
    s.thermal_relaxation_time = tau_t
    return s, kappa, h


def nusselt(s, kappa, h):
    nx, ny, nz = s.get_resolution()
    vd = s.get_velocity_density_texture().reshape(nz, ny, nx, 4)
    ft = s.get_force_temperature_texture().reshape(nz, ny, nx, 4)
    uz, T = vd[1:-1, :, :, 2].astype(np.float64), ft[1:-1, :, :, 3].astype(np.float64)
    # conductive profile dT/dz = -1/h: Nu = 1 + <u_z T> h / kappa
    return 1.0 + (uz * T).mean() * h / kappa


def sphere_channel(res=(256, 128, 128), radius=16.0, center=(64.0, 64.0, 64.0), u_in=0.05, noise=1e-4, seed=2):
    """Flow past a sphere: velocity inlet (equilibrium object, u = (u_in, 0, 0))
    on the x = 0 layer, density outlet (equilibrium object, rho = 1) on the
    x = nx-1 layer, a solid sphere, periodic y and z; equilibrium start at
    u_in plus seeded uniform noise of `noise` on u.  Returns (rho, u, ids,
    objects) for LBM.initialize_fields_from_arrays / set_boundry_properties
    (ids 1 inlet, 2 outlet, 3 sphere)."""
    nx, ny, nz = (int(v) for v in res)
    n = nx * ny * nz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ids = np.zeros((nz, ny, nx), np.uint32)
    ids[:, :, 0] = 1
    ids[:, :, -1] = 2
    cx, cy, cz = center
    ids[(x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 <= radius * radius] = 3
    rng = np.random.default_rng(seed)
    u = rng.uniform(-noise, noise, (n, 3)).astype(np.float32)
    u[:, 0] += np.float32(u_in)
    rho = np.ones(n, np.float32)
    objects = {1: dict(kind=1), 2: dict(kind=2), 3: dict(kind=0)}
    return rho, u, ids.reshape(-1), objects


def uv_sphere(n_lon=256, n_lat=128, radius=0.8):
    """Closed triangle mesh of a sphere centred at the origin (latitude /
    longitude grid, two triangles per quad) as (T, 3, 3)
    float32, for voxelize_mesh."""
    th = np.linspace(0.0, np.pi, n_lat + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, n_lon + 1)
    pts = np.stack([np.sin(th)[:, None] * np.cos(ph)[None, :],
                    np.sin(th)[:, None] * np.sin(ph)[None, :],
                    np.cos(th)[:, None] * np.ones_like(ph)[None, :]], -1) * radius
    a, b, c, d = pts[:-1, :-1], pts[1:, :-1], pts[1:, 1:], pts[:-1, 1:]
    tris = np.concatenate([np.stack([a, b, c], 2).reshape(-1, 3, 3), np.stack([a, c, d], 2).reshape(-1, 3, 3)])
    return tris.astype(np.float32)
