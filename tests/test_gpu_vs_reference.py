"""The GPU kernels against outputs of the reference's own shader code
(tests/golden/ref_fields.npz, written by tests/golden/make_ref_golden.py from
the reference-built checker), on the seeded cases of tests/ref_cases.py,
with the criteria of tests/test_oracle_vs_ref.py."""
import os

import numpy as np
import pytest

from ref_cases import NAMES, STEPS, case
from test_oracle_vs_ref import FP16_LATE_RTOL, RTOL, assert_close

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_fields.npz")


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
    for k in STEPS:
        s.iterate_time(steps=k - done, save=True)
        done = k
        vo = s.get_velocity_density_texture().reshape(-1, 4).astype(np.float64)[fluid]
        fo = s.get_force_temperature_texture().reshape(-1, 4).astype(np.float64)[fluid]
        vr = gold[f"{name}/vd/{k}"].astype(np.float64)[fluid]
        fr = gold[f"{name}/ft/{k}"].astype(np.float64)[fluid]
        tol = FP16_LATE_RTOL if (d["storage"] != 0 and k > 5) else RTOL
        assert_close(vo, fo, vr, fr, tol, k)
