"""The GPU kernels against outputs of the reference's own shader code
(tests/golden/ref_fields.npz, written by tests/golden/make_ref_golden.py from
the reference-built checker) on the seeded cases of tests/ref_cases.py: the
u/rho and force/temperature fields at every stated step -- 1, 100 and 10,000
steps of the 256^2 cavity on the reference's AA path; 1, 100 and 1,000 of the
D3Q19 sphere, the periodic von Karman street and the droplet collision that
drives the velocity limiter, its extreme branch and the density floor --
are bit-identical (SHA-256), and within 1e-5 where the field is stored."""
import numpy as np
import pytest

from ref_cases import NAMES, case, steps_of
from test_oracle_vs_ref import GOLD, check_against_gold

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_reference_shader_outputs(name, product_lib):
    import boltzmannfluids_gb300 as bf
    gold = np.load(GOLD)
    d = case(name)
    s = bf.LBM()
    s.is_collide_esoteric = d["esoteric"]
    s.boundary_mode = bf.BoundaryMode.skip
    s.two_buffer_fixed = False
    s.intermolecular_interaction_strength = d["G"]
    s.velocity_limit = d["velocity_limit"]
    s.velocity_limit_extreme = d["velocity_limit_extreme"]
    s.clear_boundry_properties()
    for k, o in (d["objects"] or {}).items():
        s.set_boundry_properties(k, velocity_translational=o.get("velocity", (0, 0, 0)),
                                 temperature=o.get("temperature", 1.0),
                                 effective_density=o.get("effective_density", 1.0))
    s.initialize_fields_from_arrays(d["res"], d["tau"], density=d["density"], velocity=d["velocity"],
                                    force=d["force"], temperature=d["temperature"], boundry_id=d["ids"],
                                    periodic=d["periodic"], velocity_set=d["velocity_set"],
                                    fp_accuracy=d["storage"], is_flow_multiphase=d["multiphase"])
    n = d["res"][0] * d["res"][1] * d["res"][2]
    fluid = np.ones(n, bool) if d["ids"] is None else (np.asarray(d["ids"]) == 0)
    done = 0
    for k in steps_of(name):
        s.iterate_time(steps=k - done, save=True)
        done = k
        vo = s.get_velocity_density_texture().reshape(-1, 4)
        fo = s.get_force_temperature_texture().reshape(-1, 4)
        check_against_gold(gold, name, k, vo, fo, fluid)
