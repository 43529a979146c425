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
