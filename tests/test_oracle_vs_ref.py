"""The oracle against the reference's own shader code compiled on the host
(oracle/_ref, built by oracle/build_ref.py from the reference's sources),
on the seeded cases of tests/ref_cases.py, bit for bit:
  * live, where the checker is built (the reference sources are present):
    fields and raw lattices after 1, 2, 5 and 30 steps of every case;
  * everywhere, against the checker's committed outputs
    (tests/golden/ref_fields.npz): the fields at every stated step of every
    case -- up to 10,000 steps of the 256^2 cavity -- by SHA-256 digest.
The GPU kernels are held to the same digests (tests/test_gpu_vs_reference.py)."""
import hashlib
import os

import numpy as np
import pytest

from oracle import ref as R
from oracle.oracle import Oracle
from ref_cases import NAMES, STEPS, case, steps_of

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_fields.npz")
# the plain FP32 path's parity bar, asserted wherever fields differ at all:
# max relative difference in rho, and in u against max(|u|, U_SCALE)
RTOL = 1e-5
U_SCALE = 0.05


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).digest(), np.uint8)


def solver_kwargs(d):
    return dict(density=d["density"], velocity=d["velocity"], force=d["force"], temperature=d["temperature"],
                boundry_id=d["ids"], objects=d["objects"], G=d["G"], velocity_limit=d["velocity_limit"],
                velocity_limit_extreme=d["velocity_limit_extreme"])


def make_oracle(d):
    return Oracle(d["res"], d["tau"], periodic=d["periodic"], velocity_set=d["velocity_set"], storage=d["storage"],
                  multiphase=d["multiphase"], esoteric=d["esoteric"], **solver_kwargs(d))


def rel_errors(vo, vr):
    e_rho = float(np.max(np.abs(vo[:, 3] - vr[:, 3]) / np.abs(vr[:, 3])))
    e_u = float(np.abs(vo[:, :3] - vr[:, :3]).max() / max(float(np.abs(vr[:, :3]).max()), U_SCALE))
    return e_rho, e_u


def check_against_gold(gold, name, k, vd, ft, fluid):
    """Bit-exact by digest; where the golden field is stored, the rho/u bar too."""
    key = f"{name}/vd/{k}"
    if key in gold.files:
        vr = gold[key].astype(np.float64)[fluid]
        e_rho, e_u = rel_errors(vd.astype(np.float64)[fluid], vr)
        assert e_rho <= RTOL and e_u <= RTOL, (name, k, e_rho, e_u)
    assert np.array_equal(digest(vd), gold[f"{name}/vd_sha/{k}"]), (name, k, "u/rho field differs")
    assert np.array_equal(digest(ft), gold[f"{name}/ft_sha/{k}"]), (name, k, "force/temperature field differs")


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_shaders_live(name, oracle_mod):
    if not R.available(name):
        pytest.skip("reference-built checker not present (reference sources absent)")
    d = case(name)
    r = R.RefShaders(name, d["res"], d["tau"], **solver_kwargs(d))
    o = make_oracle(d)
    done = 0
    for k in STEPS:
        r.iterate(k - done, True)
        o.iterate(k - done, True)
        done = k
        vr, fr = r.fields()
        vo, fo = o.fields()
        assert np.array_equal(vr, vo), (name, k, rel_errors(vo, vr))
        assert np.array_equal(fr, fo), (name, k)
        assert np.array_equal(r.lattice(), o.lattice()), (name, k)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_outputs_at_stated_steps(name, oracle_mod):
    gold = np.load(GOLD)
    d = case(name)
    o = make_oracle(d)
    n = d["res"][0] * d["res"][1] * d["res"][2]
    fluid = np.ones(n, bool) if d["ids"] is None else (np.asarray(d["ids"]) == 0)
    done = 0
    for k in steps_of(name):
        o.iterate(k - done, True)
        done = k
        vo, fo = o.fields()
        check_against_gold(gold, name, k, vo.astype(np.float32), fo.astype(np.float32), fluid)
