"""Writes tests/golden/ref_fields.npz: outputs of the reference's own shader
code (compiled on the host by oracle/build_ref.py from the reference's
sources) for the seeded cases of tests/ref_cases.py, so that tests on a
machine without the reference sources can compare against them.

For each case: the u/rho field (float4) and force/temperature field (float4)
saved at each step of ref_cases.STEPS.  Run from the repository root with
REFERENCE naming a checkout of the reference:
    REFERENCE=<checkout> python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import build_ref  # noqa: E402
from oracle import ref as R  # noqa: E402
from ref_cases import NAMES, STEPS, case  # noqa: E402


def main():
    if not build_ref.build():
        sys.exit("reference sources not found")
    out = {}
    for name in NAMES:
        d = case(name)
        r = R.RefShaders(name, d["res"], d["tau"], density=d["density"], velocity=d["velocity"], force=d["force"],
                         temperature=d["temperature"], boundry_id=d["ids"], objects=d["objects"], G=d["G"])
        done = 0
        for k in STEPS:
            r.iterate(k - done, True)
            done = k
            vd, ft = r.fields()
            out[f"{name}/vd/{k}"] = vd.astype(np.float32)
            out[f"{name}/ft/{k}"] = ft.astype(np.float32)
    path = os.path.join(ROOT, "tests", "golden", "ref_fields.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
