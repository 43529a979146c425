"""Multiphysics workloads on the GPU (Shan-Chen spinodal decomposition,
Rayleigh-Benard convection): conservation, the physics they must show, and
agreement with the FP64 oracle on small cases."""
import numpy as np
import pytest

import boltzmannfluids_gb300 as bf
from boltzmannfluids_gb300.workloads import nusselt, rayleigh_benard, spinodal
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def spinodal_solver(res, storage, seed=4):
    rho = spinodal(res, 0.69, 0.01, seed)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.intermolecular_interaction_strength = -5.0
    s.initialize_fields_from_arrays(res, 1.0, density=rho, velocity_set=bf.VelocitySet.D3Q19, fp_accuracy=storage,
                                    is_flow_multiphase=True)
    return s, rho


# Mass drift over 4000 steps at 128^3 (FP64 sums of the densities).  FP64
# arithmetic conserves mass to 1e-13 (the FP64 oracle); the FP32 update (the
# reference's unshifted arithmetic) gains ~1.5e-8 of the mass per step here.
# 16-bit storage rounds every population each step; rounded independently,
# the errors of a phase-separated flow add up (+1.8e-2 over 2000 steps at
# 48^3 in the oracle), so multiphase flow stores the last population of each
# cell as the rounding of the cell's mass less the others' stored values
# (+4.5e-7 over the same run).
SC_DRIFT_BOUND = {bf.FloatingPointAccuracy.fp32: 2e-4, bf.FloatingPointAccuracy.fp16s: 1e-5,
                  bf.FloatingPointAccuracy.fp16c: 1e-5}


@pytest.mark.parametrize("storage", list(SC_DRIFT_BOUND))
def test_spinodal_decomposition_mass_drift_and_separation(storage, product_lib):
    res = (128, 128, 128)
    s, rho0 = spinodal_solver(res, storage)
    m0 = s.reduce()[0]
    s.iterate_time(steps=4000, save=True)
    m1 = s.reduce()[0]
    rho = s.get_velocity_density_texture().reshape(-1, 4)[:, 3]
    # two phases: liquid and vapour densities far apart (G = -5)
    assert rho.max() > 1.5 and rho.min() < 0.4, (rho.min(), rho.max())
    assert abs(m1 - m0) / m0 < SC_DRIFT_BOUND[storage], (m0, m1)


def test_spinodal_against_fp64_oracle(product_lib):
    res = (24, 24, 24)
    s, rho0 = spinodal_solver(res, bf.FloatingPointAccuracy.fp32, seed=11)
    o = Oracle(res, 1.0, density=rho0, velocity_set=4, esoteric=True, multiphase=True, G=-5.0, precision=64)
    s.iterate_time(steps=200, save=True)
    o.iterate(200, True)
    vd = s.get_velocity_density_texture().reshape(-1, 4).astype(np.float64)
    vr, _ = o.fields()
    # early spinodal growth is exponential in the seeded noise; FP32 against FP64 stays close for 200 steps
    assert np.abs(vd[:, 3] - vr[:, 3]).max() / np.abs(vr[:, 3]).max() < 1e-3
    # the FP32 mass drift (~1.5e-8 per step) against FP64 conservation
    assert abs(vd[:, 3].sum() - vr[:, 3].sum()) / vr[:, 3].sum() < 1e-5


def test_rayleigh_benard_convects_with_plausible_nusselt(product_lib):
    s, kappa, h = rayleigh_benard((64, 64, 34))
    m0 = s.reduce()[0]
    s.iterate_time(steps=20000, save=True)
    nu_num = nusselt(s, kappa, h)
    m1 = s.reduce()[0]
    # Ra = 1e5 is ~60x the onset: convection carries several times the conductive flux
    assert 2.0 < nu_num < 7.0, nu_num
    # FP32 mass drift (the FP64 oracle conserves this flow's mass to 1e-13 and
    # its FP32 restatement gains ~2.7e-8 per step, bit-exact with the GPU)
    assert abs(m1 - m0) / m0 < 2e-3, (m0, m1)


def test_flow_past_sphere_full_size(product_lib):
    """The 3D plain-method configuration: D3Q19 TRT (1/4, tau 0.55) flow past a
    sphere r 16 at (64, 64, 64) in 256x128x128, velocity inlet 0.05, density
    outlet 1, periodic y/z, 5000 steps: stable, a wake behind the sphere, a
    stagnation point in front, the outlet at rho 1."""
    from boltzmannfluids_gb300.workloads import sphere_channel
    res = (256, 128, 128)
    rho, u, ids, objs = sphere_channel(res)
    s = bf.LBM()
    s.is_collide_esoteric = True
    s.collision = bf.Collision.trt
    s.boundary_mode = bf.BoundaryMode.bounce_back
    for k, o in objs.items():
        s.set_boundry_properties(k, velocity_translational=(0, 0, 0), kind=o["kind"])
    s.initialize_fields_from_arrays(res, 0.55, density=rho, velocity=u, boundry_id=ids, periodic=(False, True, True),
                                    velocity_set=bf.VelocitySet.D3Q19)
    s.iterate_time(steps=5000, save=True)
    s.synchronize()
    vd = s.get_velocity_density_texture().reshape(128, 128, 256, 4)
    assert np.isfinite(vd).all()
    ux = vd[..., 0]
    assert ux[64, 64, 64 + 24] < 0.5 * 0.05          # wake just behind the sphere
    assert abs(ux[64, 64, 64 - 20]) < 0.8 * 0.05     # slowed ahead of the stagnation point
    # the mass flux through cross-sections up- and downstream agrees (steady flow)
    flux = (vd[..., 3] * ux).sum(axis=(0, 1))
    assert abs(flux[40] - flux[200]) / flux[40] < 0.02, (flux[40], flux[200])
    assert np.abs(vd[:, :, -2, 3] - 1.0).max() < 0.02  # next to the density outlet
