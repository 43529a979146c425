"""Writes tests/golden/ref_fields.npz: outputs of the reference's own shader
code (compiled on the host by oracle/build_ref.py from the reference's
sources) for the seeded cases of tests/ref_cases.py, so that tests on a
machine without the reference sources can compare against them.

For each case and each of its stated steps (ref_cases.steps_of): SHA-256
digests of the u/rho field (float4 per cell) and of the force/temperature
field (float4 per cell) -- the kernels are compared bit for bit -- and the
u/rho field itself (float32) at the last stated step, with the force /
temperature field where it varies (thermal and multiphase cases), so that a
mismatch can be measured.  The short cases keep every step's fields.
Run from the repository root with REFERENCE naming a checkout of the
reference:
    REFERENCE=<checkout> python tests/golden/make_ref_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import build_ref  # noqa: E402
from oracle import ref as R  # noqa: E402
from ref_cases import LONG_STEPS, NAMES, case, steps_of  # noqa: E402


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).digest(), np.uint8)


def main():
    if not build_ref.build():
        sys.exit("reference sources not found: set REFERENCE")
    out = {}
    for name in NAMES:
        d = case(name)
        r = R.RefShaders(name, d["res"], d["tau"], density=d["density"], velocity=d["velocity"], force=d["force"],
                         temperature=d["temperature"], boundry_id=d["ids"], objects=d["objects"], G=d["G"],
                         velocity_limit=d["velocity_limit"], velocity_limit_extreme=d["velocity_limit_extreme"])
        steps = steps_of(name)
        varying_ft = d["multiphase"] or d["temperature"] is not None or (d["objects"] and any(
            "temperature" in o for o in d["objects"].values()))
        done = 0
        for k in steps:
            r.iterate(k - done, True)
            done = k
            vd, ft = r.fields()
            vd, ft = vd.astype(np.float32), ft.astype(np.float32)
            out[f"{name}/vd_sha/{k}"] = digest(vd)
            out[f"{name}/ft_sha/{k}"] = digest(ft)
            if name not in LONG_STEPS or k == steps[-1]:
                out[f"{name}/vd/{k}"] = vd
                if name not in LONG_STEPS or varying_ft:
                    out[f"{name}/ft/{k}"] = ft
            print(name, k, flush=True)
    path = os.path.join(ROOT, "tests", "golden", "ref_fields.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
