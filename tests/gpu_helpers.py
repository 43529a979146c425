"""Shared set-up for the GPU parity tests: one configuration is run through
the product (C ABI, sm_103a kernels) and through the CPU oracle on the same
seeded inputs, and the macroscopic fields are compared."""
import numpy as np

import boltzmannfluids_gb300 as bf
from oracle.oracle import Oracle

# Parity bar for the plain FP32 path: max relative difference in rho and u.
# u is compared relative to max(|u_ref|, U_FLOOR) so that a fluid at rest is
# held to an absolute 1e-8.
RTOL = 1e-5
U_FLOOR = 1e-3


def seeded_fields(res, seed, rho_amp=0.01, u_amp=0.02, dims=3):
    rng = np.random.default_rng(seed)
    n = res[0] * res[1] * res[2]
    rho = (1.0 + rho_amp * rng.uniform(-1, 1, n)).astype(np.float32)
    u = (u_amp * rng.uniform(-1, 1, (n, 3))).astype(np.float32)
    if dims == 2:
        u[:, 2] = 0
    return rho, u


def make_pair(res, tau, vs, *, density=None, velocity=None, force=None, temperature=None, ids=None,
              objects=None, periodic=(True, True, True), storage=0, multiphase=False, esoteric=True,
              boundary_mode=0, collision=0, trt_magic=0.25, G=-6.0, tau_t=2.0, beta=0.5,
              thermal_init_equilibrium=False, two_buffer_fixed=False, velocity_limit=0.25,
              velocity_limit_extreme=0.30, precision=32):
    s = bf.LBM()
    s.is_collide_esoteric = esoteric
    s.boundary_mode = boundary_mode
    s.collision = collision
    s.trt_magic = trt_magic
    s.intermolecular_interaction_strength = G
    s.thermal_expansion_coefficient = beta
    s.thermal_init_equilibrium = thermal_init_equilibrium
    s.two_buffer_fixed = two_buffer_fixed
    s.velocity_limit = velocity_limit
    s.velocity_limit_extreme = velocity_limit_extreme
    s.clear_boundry_properties()
    for k, o in (objects or {}).items():
        s.set_boundry_properties(k, velocity_translational=o.get("velocity", (0, 0, 0)),
                                 temperature=o.get("temperature", 1.0),
                                 effective_density=o.get("effective_density", 1.0),
                                 kind=o.get("kind", 0))
    s.initialize_fields_from_arrays(res, tau, density=density, velocity=velocity, force=force,
                                    temperature=temperature, boundry_id=ids, periodic=periodic,
                                    velocity_set=vs, fp_accuracy=storage, is_flow_multiphase=multiphase)
    # initialisation resets it to 2 (LBM.cpp:461); set afterwards, it takes
    # effect at the next step
    s.thermal_relaxation_time = tau_t
    o = Oracle(res, tau, density=density, velocity=velocity, force=force, temperature=temperature,
               boundry_id=ids, periodic=periodic, velocity_set=int(vs), storage=int(storage),
               multiphase=multiphase, esoteric=esoteric, boundary_mode=int(boundary_mode), collision=int(collision),
               trt_magic=trt_magic, velocity_limit=velocity_limit, velocity_limit_extreme=velocity_limit_extreme,
               G=G, tau_t=tau_t, beta=beta, thermal_init_equilibrium=thermal_init_equilibrium,
               two_buffer_fixed=two_buffer_fixed, objects=objects, precision=precision)
    return s, o


def fields_of(s):
    vd = s.get_velocity_density_texture().reshape(-1, 4).astype(np.float64)
    ft = s.get_force_temperature_texture().reshape(-1, 4).astype(np.float64)
    return vd, ft


def rel_errors(vd, vr, mask=None):
    if mask is not None:
        vd, vr = vd[mask], vr[mask]
    e_rho = float(np.max(np.abs(vd[:, 3] - vr[:, 3]) / np.abs(vr[:, 3])))
    u_scale = max(float(np.abs(vr[:, :3]).max()), U_FLOOR)
    e_u = float(np.abs(vd[:, :3] - vr[:, :3]).max() / u_scale)
    return e_rho, e_u


def step_and_compare(s, o, checkpoints, rtol=RTOL, mask=None, check_temperature=False, exact=True):
    """Steps both to each checkpoint (saving fields there) and compares.

    The bar is RTOL; with exact=True the fields must also agree bit for bit:
    the kernels and the oracle evaluate the same expression trees with
    individually rounded operations."""
    done = 0
    worst = (0.0, 0.0)
    for k in checkpoints:
        s.iterate_time(steps=k - done, save=True)
        o.iterate(k - done, True)
        done = k
        vd, ft = fields_of(s)
        vr, fr = o.fields()
        e_rho, e_u = rel_errors(vd, vr, mask)
        worst = (max(worst[0], e_rho), max(worst[1], e_u))
        assert e_rho <= rtol, f"step {k}: rho rel err {e_rho:.3e}"
        assert e_u <= rtol, f"step {k}: u rel err {e_u:.3e}"
        if exact:
            m = slice(None) if mask is None else mask
            assert np.array_equal(vd[m], vr[m]), f"step {k}: fields within {max(e_rho, e_u):.2e} but not bit-exact"
        if check_temperature:
            m = slice(None) if mask is None else mask
            t_scale = max(float(np.abs(fr[m, 3]).max()), 1e-3)
            e_t = float(np.abs(ft[m, 3] - fr[m, 3]).max() / t_scale)
            assert e_t <= rtol, f"step {k}: T rel err {e_t:.3e}"
            if exact:
                assert np.array_equal(ft[m], fr[m]), f"step {k}: force/temperature not bit-exact"
    s.synchronize()
    return worst
